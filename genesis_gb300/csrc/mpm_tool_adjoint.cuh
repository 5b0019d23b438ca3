// mpm_tool_adjoint.cuh - a tool entity's collision (tool_entity/mesh.py Mesh.collide,
// legacy_coupler.py:349-354) in the differentiable form: written once for float (the forward
// grid op) and for forward-mode dual numbers with 9 tangents (the node velocity, the tool's
// position and its linear velocity), whose tangents give the Jacobians the adjoint grid op needs.
//
// The tool's orientation and angular velocity enter as constants: their derivatives are not
// formed (the reference's tool quaternion chain is left out of the differentiable form).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace gbmpm {

constexpr int TOOL_ND = 9;  // d/d v (3), d/d tool position (3), d/d tool linear velocity (3)

struct TD {
  float v;
  float d[TOOL_ND];
};

__device__ __forceinline__ TD td_const(float v) {
  TD r;
  r.v = v;
#pragma unroll
  for (int k = 0; k < TOOL_ND; ++k) r.d[k] = 0.f;
  return r;
}
__device__ __forceinline__ TD td_var(float v, int k) {
  TD r = td_const(v);
  r.d[k] = 1.f;
  return r;
}
__device__ __forceinline__ TD operator+(const TD& a, const TD& b) {
  TD r;
  r.v = a.v + b.v;
#pragma unroll
  for (int k = 0; k < TOOL_ND; ++k) r.d[k] = a.d[k] + b.d[k];
  return r;
}
__device__ __forceinline__ TD operator-(const TD& a, const TD& b) {
  TD r;
  r.v = a.v - b.v;
#pragma unroll
  for (int k = 0; k < TOOL_ND; ++k) r.d[k] = a.d[k] - b.d[k];
  return r;
}
__device__ __forceinline__ TD operator*(const TD& a, const TD& b) {
  TD r;
  r.v = a.v * b.v;
#pragma unroll
  for (int k = 0; k < TOOL_ND; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
  return r;
}
__device__ __forceinline__ TD operator/(const TD& a, const TD& b) {
  TD r;
  r.v = a.v / b.v;
  const float ib = 1.f / b.v;
#pragma unroll
  for (int k = 0; k < TOOL_ND; ++k) r.d[k] = (a.d[k] - r.v * b.d[k]) * ib;
  return r;
}
__device__ __forceinline__ TD operator*(float s, const TD& a) {
  TD r;
  r.v = s * a.v;
#pragma unroll
  for (int k = 0; k < TOOL_ND; ++k) r.d[k] = s * a.d[k];
  return r;
}
__device__ __forceinline__ TD operator+(const TD& a, float s) {
  TD r = a;
  r.v += s;
  return r;
}
__device__ __forceinline__ TD td_sqrt(const TD& a) {
  TD r;
  r.v = sqrtf(a.v);
  const float h = 0.5f / r.v;
#pragma unroll
  for (int k = 0; k < TOOL_ND; ++k) r.d[k] = a.d[k] * h;
  return r;
}
__device__ __forceinline__ TD td_exp(const TD& a) {
  TD r;
  r.v = expf(a.v);
#pragma unroll
  for (int k = 0; k < TOOL_ND; ++k) r.d[k] = a.d[k] * r.v;
  return r;
}

// value / derivative access and the few functions the collision needs, for both scalar types
__device__ __forceinline__ float val(float a) { return a; }
__device__ __forceinline__ float val(const TD& a) { return a.v; }
template <typename S> __device__ __forceinline__ S cst(float v);
template <> __device__ __forceinline__ float cst<float>(float v) { return v; }
template <> __device__ __forceinline__ TD cst<TD>(float v) { return td_const(v); }
__device__ __forceinline__ float ssqrt(float a) { return sqrtf(a); }
__device__ __forceinline__ TD ssqrt(const TD& a) { return td_sqrt(a); }
__device__ __forceinline__ float sexp(float a) { return expf(a); }
__device__ __forceinline__ TD sexp(const TD& a) { return td_exp(a); }

// A tool of the differentiable form: its SDF grid (values, T_mesh_to_sdf rows, the inverse of its
// 3x3 block), coupling parameters and floor height.
struct DiffToolDev {
  const float* sdf;
  int32_t res[3];
  float T[12];
  float Rinv[9];
  float friction, softness, floor_h;
};

// Rotation matrix of a unit quaternion (w, x, y, z).
__device__ __forceinline__ void quat_R(const float* q, float* R) {
  const float w = q[0], x = q[1], y = q[2], z = q[3];
  R[0] = 1.f - 2.f * (y * y + z * z), R[1] = 2.f * (x * y - w * z), R[2] = 2.f * (x * z + w * y);
  R[3] = 2.f * (x * y + w * z), R[4] = 1.f - 2.f * (x * x + z * z), R[5] = 2.f * (y * z - w * x);
  R[6] = 2.f * (x * z - w * y), R[7] = 2.f * (y * z + w * x), R[8] = 1.f - 2.f * (x * x + y * y);
}

// Mesh.sdf_ (mesh.py:90-104): trilinear value at voxel position pv, 1 where the base voxel leaves
// the grid.  Inside a voxel the weights are linear in pv, so the tangents follow it exactly.
template <typename S>
__device__ S tool_sdf_t(const DiffToolDev& t, const S* pv) {
  int b[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    b[k] = (int)floorf(val(pv[k]));
    if (b[k] >= t.res[k] - 1 || b[k] < 0) return cst<S>(1.f);
  }
  S f[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) f[k] = pv[k] + (-(float)b[k]);
  S acc = cst<S>(0.f);
#pragma unroll
  for (int o = 0; o < 8; ++o) {
    const int ox = o >> 2, oy = (o >> 1) & 1, oz = o & 1;
    const S wx = ox ? f[0] : cst<S>(1.f) - f[0];
    const S wy = oy ? f[1] : cst<S>(1.f) - f[1];
    const S wz = oz ? f[2] : cst<S>(1.f) - f[2];
    const float value = t.sdf[((int64_t)(b[0] + ox) * t.res[1] + (b[1] + oy)) * t.res[2] + (b[2] + oz)];
    acc = acc + value * (wx * wy * wz);
  }
  return acc;
}

// Mesh.collide (mesh.py:148-177) at node position x for node velocity v, with the tool at
// position p and orientation q and its next pose one substep later (ToolEntity.advect: p + u dt
// above the floor, q turned by ang dt, qn given); v is updated in place.
template <typename S>
__device__ void tool_collide_t(const DiffToolDev& t, const float* x, S* v, const S* p, const float* q, const S* u,
                               const float* qn, float dt, float eps) {
  float R[9], Rn[9];
  quat_R(q, R);
  quat_R(qn, Rn);
  S d[3], pm[3], pv[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) d[k] = cst<S>(x[k]) - p[k];
#pragma unroll
  for (int r = 0; r < 3; ++r) pm[r] = R[0 * 3 + r] * d[0] + R[1 * 3 + r] * d[1] + R[2 * 3 + r] * d[2];  // R^T d
#pragma unroll
  for (int r = 0; r < 3; ++r) pv[r] = t.T[r * 4 + 0] * pm[0] + t.T[r * 4 + 1] * pm[1] + t.T[r * 4 + 2] * pm[2] + t.T[r * 4 + 3];
  const S sd = tool_sdf_t(t, pv);
  S infl = sexp((-1.f / fmaxf(eps, t.softness)) * sd);
  if (val(infl) >= 1.f) infl = cst<S>(1.f);  // min(exp(-sd / softness), 1)
  if (!(val(sd) <= 0.f || val(infl) > 0.1f)) return;
  // next pose and the collider velocity at x
  S pn[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) pn[k] = p[k] + dt * u[k];
  if (val(pn[2]) < t.floor_h) pn[2] = cst<S>(t.floor_h);  // FloorBoundary.impose_pos
  S vc[3], rv[3];
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    const S xn = Rn[r * 3 + 0] * pm[0] + Rn[r * 3 + 1] * pm[1] + Rn[r * 3 + 2] * pm[2] + pn[r];
    vc[r] = (1.f / dt) * (xn + (-x[r]));
    rv[r] = v[r] - vc[r];
  }
  // normal: central differences in voxel space (delta 1e-2), to the mesh frame, then the world
  S nv[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    S inc[3] = {pv[0], pv[1], pv[2]}, dec[3] = {pv[0], pv[1], pv[2]};
    inc[i] = inc[i] + 1e-2f;
    dec[i] = dec[i] + (-1e-2f);
    nv[i] = (1.f / (2.f * 1e-2f)) * (tool_sdf_t(t, inc) - tool_sdf_t(t, dec));
  }
  S l = ssqrt(nv[0] * nv[0] + nv[1] * nv[1] + nv[2] * nv[2] + eps);
  S nm[3], n[3];
#pragma unroll
  for (int r = 0; r < 3; ++r) nm[r] = (t.Rinv[r * 3 + 0] * nv[0] + t.Rinv[r * 3 + 1] * nv[1] + t.Rinv[r * 3 + 2] * nv[2]) / l;
#pragma unroll
  for (int r = 0; r < 3; ++r) n[r] = R[r * 3 + 0] * nm[0] + R[r * 3 + 1] * nm[1] + R[r * 3 + 2] * nm[2];
  l = ssqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2] + eps);
#pragma unroll
  for (int r = 0; r < 3; ++r) n[r] = n[r] / l;
  const S rvn = rv[0] * n[0] + rv[1] * n[1] + rv[2] * n[2];
  if (!(val(rvn) < 0.f)) return;
  S rt[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) rt[k] = rv[k] - rvn * n[k];
  const S rtn = ssqrt(rt[0] * rt[0] + rt[1] * rt[1] + rt[2] * rt[2] + eps);
  S mag = rtn + t.friction * rvn;
  if (val(mag) < 0.f) mag = cst<S>(0.f);
  const S keep = (mag / rtn) * infl;
  const S rest = cst<S>(1.f) - infl;
#pragma unroll
  for (int k = 0; k < 3; ++k) v[k] = vc[k] + rt[k] * keep + rv[k] * rest;
}

// ToolEntity.advect (tool_entity.py:193-206) of one tool state (pos 3, quat 4, vel 3, ang 3).
__device__ __forceinline__ void tool_advance_state(const float* s, float dt, float eps, float floor_h, float* o) {
#pragma unroll
  for (int k = 0; k < 3; ++k) o[k] = s[k] + s[7 + k] * dt;
  o[2] = fmaxf(o[2], floor_h);
  const float rv[3] = {s[10] * dt, s[11] * dt, s[12] * dt};
  const float th2 = rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2];
  float w[4] = {1.f, 0.f, 0.f, 0.f};
  if (th2 > eps * eps) {  // qd_rotvec_to_quat with its first-order normalisation
    const float th = sqrtf(th2);
    w[0] = cosf(0.5f * th);
    const float sn = sinf(0.5f * th) / th;
    for (int k = 0; k < 3; ++k) w[k + 1] = sn * rv[k];
    const float sc = 0.5f * (3.f - (w[0] * w[0] + w[1] * w[1] + w[2] * w[2] + w[3] * w[3]));
    for (int k = 0; k < 4; ++k) w[k] *= sc;
  }
  const float* q = s + 3;  // qd_transform_quat_by_quat(q, w) = normalize(w * q)
  float r[4] = {w[0] * q[0] - w[1] * q[1] - w[2] * q[2] - w[3] * q[3], w[0] * q[1] + w[1] * q[0] + w[2] * q[3] - w[3] * q[2],
                w[0] * q[2] - w[1] * q[3] + w[2] * q[0] + w[3] * q[1], w[0] * q[3] + w[1] * q[2] - w[2] * q[1] + w[3] * q[0]};
  const float len = sqrtf(r[0] * r[0] + r[1] * r[1] + r[2] * r[2] + r[3] * r[3]);
#pragma unroll
  for (int k = 0; k < 4; ++k) o[3 + k] = r[k] / len;
#pragma unroll
  for (int k = 0; k < 6; ++k) o[7 + k] = s[7 + k];
}

}  // namespace gbmpm
