// mpm_colliders.cuh - kinematic rigid colliders of the grid op (legacy_coupler.py:134-218,
// 284-347): signed distance and normal of each shape, the velocity update of a node inside a
// collider's influence, and that update's transposed Jacobian in the node velocity (the
// differentiable grid op's adjoint).  Shared by the substep grid op and the differentiable one.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "gbmpm.h"
#include "mpm_kernels.cuh"

namespace gbmpm {
namespace {

__device__ __forceinline__ void rot(const float* q, const float* v, float* o) {  // gu.qd_transform_by_quat
  const float w = q[0], x = q[1], y = q[2], z = q[3];
  o[0] = v[0] * (x * x + w * w - y * y - z * z) + v[1] * (2.f * x * y - 2.f * w * z) + v[2] * (2.f * x * z + 2.f * w * y);
  o[1] = v[0] * (2.f * w * z + 2.f * x * y) + v[1] * (w * w - x * x + y * y - z * z) + v[2] * (-2.f * w * x + 2.f * y * z);
  o[2] = v[0] * (-2.f * w * y + 2.f * x * z) + v[1] * (2.f * w * x + 2.f * y * z) + v[2] * (w * w - x * x - y * y + z * z);
}


// ---- voxel SDF grids (MPM_COLLIDER_SDF: utils/sdf.py; MPM_COLLIDER_TOOL: tool_entity/mesh.py)
// World point x -> mesh frame (inverse pose) -> voxel coordinates ps (T_mesh_to_sdf).
__device__ __forceinline__ void sdf_voxel_pos(const ColliderDev& c, const float* pos, const float* quat,
                                              const float* x, float* pm, float* ps) {
  const float d[3] = {x[0] - pos[0], x[1] - pos[1], x[2] - pos[2]};
  const float qi[4] = {quat[0], -quat[1], -quat[2], -quat[3]};
  rot(qi, d, pm);
  for (int r = 0; r < 3; ++r) ps[r] = c.T[r * 4 + 0] * pm[0] + c.T[r * 4 + 1] * pm[1] + c.T[r * 4 + 2] * pm[2] + c.T[r * 4 + 3];
}

// Trilinear interpolation over the 8 voxels from `base` (utils/sdf.py:167-184, 283-294;
// mesh.py:101-107), in the reference's corner order (z fastest); the gradient too when g != null.
__device__ __forceinline__ float sdf_trilinear(const ColliderDev& c, const float* ps, const int* base, float* g) {
  float sd = 0.f;
  if (g) g[0] = g[1] = g[2] = 0.f;
  for (int o = 0; o < 8; ++o) {
    const int cx = base[0] + (o >> 2), cy = base[1] + ((o >> 1) & 1), cz = base[2] + (o & 1);
    const float w = (1.f - fabsf(ps[0] - (float)cx)) * (1.f - fabsf(ps[1] - (float)cy)) * (1.f - fabsf(ps[2] - (float)cz));
    const int64_t cell = ((int64_t)cx * c.res[1] + cy) * c.res[2] + cz;
    sd = sd + w * c.val[cell];
    if (g)
      for (int k = 0; k < 3; ++k) g[k] = g[k] + w * c.grad[cell * 3 + k];
  }
  return sd;
}

// Rigid geom SDF grid (utils/sdf.py:137-184, 223-296): value and gradient in the voxel frame.
__device__ __forceinline__ float sdf_grid_value_grad(const ColliderDev& c, const float* ps, float eps, float* g) {
  bool outside = false;
  for (int k = 0; k < 3; ++k) outside = outside || ps[k] >= (float)(c.res[k] - 1) || ps[k] <= 0.f;
  if (outside) {  // proxy: distance to the grid centre (sdf_func_proxy_sdf / _proxy_grad)
    float d[3];
    for (int k = 0; k < 3; ++k) d[k] = ps[k] - (float)(c.res[k] - 1) / 2.f;
    const float len2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    const float ln = sqrtf(len2 + eps);
    for (int k = 0; k < 3; ++k) g[k] = d[k] / ln;
    return sqrtf(len2) / c.cell_size + c.sdf_max;
  }
  int base[3];
  for (int k = 0; k < 3; ++k) base[k] = min((int)floorf(ps[k]), c.res[k] - 2);
  return sdf_trilinear(c, ps, base, g);
}

// Signed distance and outward unit normal of a collider at world point x
// (utils/sdf.py:119-126 and 372-378 for sphere and plane; analytic box; SDF grid).
__device__ __forceinline__ float collider_sdf(const ColliderDev& c, const float* x, float eps, float* n) {
  float d[3] = {x[0] - c.pos[0], x[1] - c.pos[1], x[2] - c.pos[2]};
  if (c.type == MPM_COLLIDER_SDF) {
    float pm[3], ps[3], gv[3], g[3];
    sdf_voxel_pos(c, c.pos, c.quat, x, pm, ps);
    const float sd = sdf_grid_value_grad(c, ps, eps, gv);
    rot(c.quat, gv, g);  // no rotation between the mesh and SDF frames (utils/sdf.py:383)
    const float gn = sqrtf(g[0] * g[0] + g[1] * g[1] + g[2] * g[2] + eps);
    for (int k = 0; k < 3; ++k) n[k] = g[k] / gn;
    return sd;
  }
  if (c.type == MPM_COLLIDER_SPHERE) {
    const float len = sqrtf(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    const float ln = sqrtf(d[0] * d[0] + d[1] * d[1] + d[2] * d[2] + eps);  // norm(EPS)
    for (int k = 0; k < 3; ++k) n[k] = d[k] / ln;
    return len - c.size[0];
  }
  const float qi[4] = {c.quat[0], -c.quat[1], -c.quat[2], -c.quat[3]};
  float l[3];
  rot(qi, d, l);  // position in the collider frame
  float gl[3];
  float sd;
  if (c.type == MPM_COLLIDER_PLANE) {
    sd = l[0] * c.size[0] + l[1] * c.size[1] + l[2] * c.size[2];
    gl[0] = c.size[0], gl[1] = c.size[1], gl[2] = c.size[2];
  } else {  // box
    float q[3], outside = 0.f;
    int ax = 0;
    for (int k = 0; k < 3; ++k) {
      q[k] = fabsf(l[k]) - c.size[k];
      const float o = fmaxf(q[k], 0.f);
      outside += o * o;
      if (q[k] > q[ax]) ax = k;
    }
    const float inside = fminf(fmaxf(q[0], fmaxf(q[1], q[2])), 0.f);
    sd = sqrtf(outside) + inside;
    for (int k = 0; k < 3; ++k) {
      const float sg = l[k] < 0.f ? -1.f : 1.f;
      gl[k] = outside > 0.f ? sg * fmaxf(q[k], 0.f) : (k == ax ? sg : 0.f);
    }
  }
  float g[3];
  rot(c.quat, gl, g);
  const float gn = sqrtf(g[0] * g[0] + g[1] * g[1] + g[2] * g[2] + eps);
  for (int k = 0; k < 3; ++k) n[k] = g[k] / gn;
  return sd;
}

// The node velocity v at x after collider c (normal n, influence in (0.1, 1]), as
// _func_collide_in_rigid_geom computes it: the velocity relative to the collider loses its inward
// normal part (restitution) and tangential speed (friction), blended by the influence.  False (v
// unchanged) when the relative velocity does not point into the collider.
__device__ __forceinline__ bool collide_in_velocity(const ColliderDev& c, float eps, const float* x, float* v,
                                                    const float* n, float influence) {
  const float r[3] = {x[0] - c.com[0], x[1] - c.com[1], x[2] - c.com[2]};
  const float vr[3] = {c.ang[1] * r[2] - c.ang[2] * r[1] + c.lin[0], c.ang[2] * r[0] - c.ang[0] * r[2] + c.lin[1],
                       c.ang[0] * r[1] - c.ang[1] * r[0] + c.lin[2]};
  const float rv[3] = {v[0] - vr[0], v[1] - vr[1], v[2] - vr[2]};
  const float rvn = rv[0] * n[0] + rv[1] * n[1] + rv[2] * n[2];
  if (!(rvn < 0.f)) return false;
  float rt[3];
  for (int k = 0; k < 3; ++k) rt[k] = rv[k] - rvn * n[k];
  const float rtn = sqrtf(rt[0] * rt[0] + rt[1] * rt[1] + rt[2] * rt[2] + eps);  // norm(gs.EPS)
  const float scale = fmaxf(0.f, rtn + rvn * c.friction) / rtn;
  for (int k = 0; k < 3; ++k)
    v[k] = vr[k] + (rt[k] * scale - n[k] * rvn * c.restitution) * influence + rv[k] * (1.f - influence);
  return true;
}

// g <- J^T g for J = d(collide_in_velocity)/dv at the velocity v the collider saw.  With
// rv = v - v_collider, rvn = n.rv, P = I - n n^T, rt = P rv, |rt| = sqrt(|rt|^2 + eps) and
// s = max(0, |rt| + f rvn) / |rt|:  J = infl (s P + rt (grad s)^T - e n n^T) + (1 - infl) I,
// grad s = f (n / |rt| - rvn P rt / |rt|^3) where |rt| + f rvn > 0, else 0.
__device__ __forceinline__ void collide_in_vjp(const ColliderDev& c, float eps, const float* x, const float* v,
                                               const float* n, float influence, float* g) {
  const float r[3] = {x[0] - c.com[0], x[1] - c.com[1], x[2] - c.com[2]};
  const float vr[3] = {c.ang[1] * r[2] - c.ang[2] * r[1] + c.lin[0], c.ang[2] * r[0] - c.ang[0] * r[2] + c.lin[1],
                       c.ang[0] * r[1] - c.ang[1] * r[0] + c.lin[2]};
  const float rv[3] = {v[0] - vr[0], v[1] - vr[1], v[2] - vr[2]};
  const float rvn = rv[0] * n[0] + rv[1] * n[1] + rv[2] * n[2];
  if (!(rvn < 0.f)) return;
  float rt[3];
  for (int k = 0; k < 3; ++k) rt[k] = rv[k] - rvn * n[k];
  const float rtn = sqrtf(rt[0] * rt[0] + rt[1] * rt[1] + rt[2] * rt[2] + eps);
  const float f = c.friction, e = c.restitution;
  const bool sliding = rtn + rvn * f > 0.f;
  const float s = sliding ? (rtn + rvn * f) / rtn : 0.f;
  const float ng = n[0] * g[0] + n[1] * g[1] + n[2] * g[2];
  const float rtg = rt[0] * g[0] + rt[1] * g[1] + rt[2] * g[2];
  const float nrt = n[0] * rt[0] + n[1] * rt[1] + n[2] * rt[2];
  float out[3];
  for (int k = 0; k < 3; ++k) {
    const float Pg = g[k] - n[k] * ng;                 // P g
    const float Prt = rt[k] - n[k] * nrt;              // P rt
    const float gs = sliding ? f * (n[k] / rtn - rvn * Prt / (rtn * rtn * rtn)) : 0.f;
    out[k] = influence * (s * Pg + gs * rtg - e * n[k] * ng) + (1.f - influence) * g[k];
  }
  for (int k = 0; k < 3; ++k) g[k] = out[k];
}

}  // namespace
}  // namespace gbmpm
