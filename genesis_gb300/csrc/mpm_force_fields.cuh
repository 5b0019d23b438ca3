// mpm_force_fields.cuh - the external acceleration fields of the grid op (engine/force_fields.py
// _get_acc of each built-in type), shared by the substep grid op and the differentiable one, and
// their Jacobians with respect to the node velocity (the differentiable grid op's adjoint).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "gbmpm.h"
#include "mpm_kernels.cuh"

namespace gbmpm {
namespace {

// splitmix64 (Steele, Lea and Flood 2014): one step of the generator as a 64-bit mixing function.
__device__ __forceinline__ unsigned long long splitmix64(unsigned long long z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

// Perlin's improved noise (force_fields.py:441-544) over a 256-entry permutation p, at frequency f.
__device__ __forceinline__ float perlin_fade(float t) { return t * t * t * (t * (t * 6.f - 15.f) + 10.f); }
__device__ __forceinline__ float perlin_lerp(float t, float a, float b) { return a + t * (b - a); }
__device__ __forceinline__ float perlin_grad(int h, float x, float y, float z) {
  h &= 15;
  const float u = h < 8 ? x : y;
  float v = y;
  if (h >= 4) v = (h == 12 || h == 14) ? x : z;
  return ((h & 1) == 0 ? u : -u) + ((h & 2) == 0 ? v : -v);
}
__device__ float perlin(const uint8_t* p, float f, float x, float y, float z) {
  x *= f;
  y *= f;
  z *= f;
  const float fx = floorf(x), fy = floorf(y), fz = floorf(z);
  const int X = (int)fx & 255, Y = (int)fy & 255, Z = (int)fz & 255;
  x -= fx;
  y -= fy;
  z -= fz;
  const float u = perlin_fade(x), v = perlin_fade(y), w = perlin_fade(z);
  // the reference's table is the permutation written twice (512 entries): index & 255
  const int A = p[X] + Y, AA = p[A & 255] + Z, AB = p[(A + 1) & 255] + Z;
  const int B = p[(X + 1) & 255] + Y, BA = p[B & 255] + Z, BB = p[(B + 1) & 255] + Z;
  return perlin_lerp(
      w,
      perlin_lerp(v, perlin_lerp(u, perlin_grad(p[AA & 255], x, y, z), perlin_grad(p[BA & 255], x - 1.f, y, z)),
                  perlin_lerp(u, perlin_grad(p[AB & 255], x, y - 1.f, z), perlin_grad(p[BB & 255], x - 1.f, y - 1.f, z))),
      perlin_lerp(v,
                  perlin_lerp(u, perlin_grad(p[(AA + 1) & 255], x, y, z - 1.f),
                              perlin_grad(p[(BA + 1) & 255], x - 1.f, y, z - 1.f)),
                  perlin_lerp(u, perlin_grad(p[(AB + 1) & 255], x, y - 1.f, z - 1.f),
                              perlin_grad(p[(BB + 1) & 255], x - 1.f, y - 1.f, z - 1.f))));
}

// engine/force_fields.py _get_acc of each field type (Constant :73, Wind :122, Point :178,
// Drag :220, Noise :243, Vortex :319, Turbulence :400) at node position x (world node index gw of
// scene `scene`) with the current node velocity v; `step` counts substeps for the noise draws.
__device__ __forceinline__ void ff_acc(const ForceFieldDev& f, const float* x, const float* v, float eps, float* a,
                                       int32_t scene, const int* gw, unsigned long long step) {
  a[0] = a[1] = a[2] = 0.f;
  if (f.type == MPM_FF_CONSTANT) {
    for (int k = 0; k < 3; ++k) a[k] = f.dir[k] * f.strength;
  } else if (f.type == MPM_FF_WIND) {
    const float r[3] = {x[0] - f.center[0], x[1] - f.center[1], x[2] - f.center[2]};
    const float c[3] = {r[1] * f.dir[2] - r[2] * f.dir[1], r[2] * f.dir[0] - r[0] * f.dir[2],
                        r[0] * f.dir[1] - r[1] * f.dir[0]};
    if (!(sqrtf(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]) > f.radius))
      for (int k = 0; k < 3; ++k) a[k] = f.dir[k] * f.strength;
  } else if (f.type == MPM_FF_POINT) {
    const float r[3] = {x[0] - f.center[0], x[1] - f.center[1], x[2] - f.center[2]};
    const float rad = sqrtf(r[0] * r[0] + r[1] * r[1] + r[2] * r[2] + eps);  // norm(gs.EPS)
    const float fall = 1.f / powf(rad + 1.f, f.falloff_pow);
    for (int k = 0; k < 3; ++k) {
      float ak = f.strength * (r[k] / rad);
      ak += (ak - v[k]) * f.flow;
      a[k] = ak * fall;
    }
  } else if (f.type == MPM_FF_DRAG) {
    const float vn = sqrtf(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    for (int k = 0; k < 3; ++k) a[k] = -f.linear * v[k] - f.quadratic * vn * v[k];
  } else if (f.type == MPM_FF_VORTEX) {
    const float rx = x[0] - f.center[0], ry = x[1] - f.center[1];
    const float rad = sqrtf(rx * rx + ry * ry);
    float fall = 0.f;
    if (rad < f.falloff_min) fall = 1.f;
    else if (rad < f.falloff_max) fall = 1.f / powf(rad - f.falloff_min + 1.f, f.falloff_pow);
    a[0] = fall * (f.s_perp * -ry + f.s_radial * -rx) - f.damping * v[0];
    a[1] = fall * (f.s_perp * rx + f.s_radial * -ry) - f.damping * v[1];
    a[2] = fall * 0.f - f.damping * v[2];
  } else if (f.type == MPM_FF_NOISE) {
    const unsigned long long node = ((unsigned long long)((uint32_t)gw[0] & 0x1fffffu)) |
                                    ((unsigned long long)((uint32_t)gw[1] & 0x1fffffu) << 21) |
                                    ((unsigned long long)((uint32_t)gw[2] & 0x1fffffu) << 42);
    const unsigned long long h =
        splitmix64(splitmix64(splitmix64(splitmix64(f.seed) ^ step) ^ (unsigned long long)(uint32_t)scene) ^ node);
    for (int k = 0; k < 3; ++k) {
      const float u = (float)(splitmix64(h + (unsigned long long)k) >> 40) * 0x1p-24f;
      a[k] = (u * 2.f - 1.f) * f.strength;
    }
  } else if (f.type == MPM_FF_TURBULENCE) {
    for (int k = 0; k < 3; ++k) a[k] = perlin(f.perm[k], f.frequency, x[0], x[1], x[2]) * f.strength;
    for (int k = 0; k < 3; ++k) a[k] += (a[k] - v[k]) * f.flow;
  }
}

// dL/dv before a field from dL/dv after it: v' = v + dt acc(x, v), so g += dt J^T g with
// J = d acc / d v at the velocity the field saw.  Constant, Wind and Noise do not depend on v
// (Noise's draws are constants of the substep); Point, Vortex and Turbulence are linear in v
// (J = -flow falloff I, -damping I, -flow I); Drag's -quadratic |v| v term has
// J = -quadratic (|v| I + v v^T / |v|), taken as 0 at v = 0 (its limit; the reference's autodiff of
// norm() divides by zero there).  J is symmetric in every case.
__device__ __forceinline__ void ff_acc_vjp(const ForceFieldDev& f, const float* x, const float* v, float eps,
                                           float dt, float* g) {
  float c = 0.f;  // J = -c I (+ the Drag outer product)
  if (f.type == MPM_FF_POINT) {
    const float r[3] = {x[0] - f.center[0], x[1] - f.center[1], x[2] - f.center[2]};
    const float rad = sqrtf(r[0] * r[0] + r[1] * r[1] + r[2] * r[2] + eps);
    c = f.flow / powf(rad + 1.f, f.falloff_pow);
  } else if (f.type == MPM_FF_VORTEX) {
    c = f.damping;
  } else if (f.type == MPM_FF_TURBULENCE) {
    c = f.flow;
  } else if (f.type == MPM_FF_DRAG) {
    const float vn = sqrtf(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    c = f.linear + f.quadratic * vn;
    if (vn > 0.f) {
      const float s = f.quadratic * (v[0] * g[0] + v[1] * g[1] + v[2] * g[2]) / vn;
      const float g0[3] = {g[0], g[1], g[2]};
      for (int k = 0; k < 3; ++k) g[k] = g0[k] - dt * (c * g0[k] + s * v[k]);
      return;
    }
  } else {
    return;
  }
  for (int k = 0; k < 3; ++k) g[k] -= dt * c * g[k];
}

}  // namespace
}  // namespace gbmpm
