// mpm_grad.cu - differentiable MPM substep: forward with per-particle Lame parameters and its
// hand-written adjoint (G2P, grid op, P2G, elastic stress through the polar decomposition).
//
// Reference counterpart: Genesis differentiates the substep with Quadrants autodiff
// (p2g.grad, mpm_grid_op.grad, g2p.grad, compute_F_tmp.grad: mpm_solver.py:517-554,
// legacy_coupler.py:998-1019) and a custom SVD backward (backward_svd, mpm_solver.py:1229-1252).
// Here the stress adjoint differentiates the rotation of the polar decomposition F = R S
// directly: with S = V diag(s) V^T, dR = R Omega where (V^T Omega V)_ij = (V^T (R^T dF -
// dF^T R) V)_ij / (s_i + s_j); it has no 1/(s_j^2 - s_i^2) factors, so it stays finite at
// F = I where the generic SVD backward relies on cancelling 1e6-sized terms.
//
// Materials: Elastic (corotated and neo-Hookean), Liquid, Sand and Snow; the grid op also applies
// the built-in force fields and tool entities.  Grid: dense [res^3] float4 buffers owned
// by the caller (torch tensors); particles: caller arrays in the reference layout.  The
// scatter uses global vector atomics (no sort): the differentiable path favours clarity.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>

#include "gbmpm.h"
#include "mpm_adjoint.cuh"
#include "mpm_colliders.cuh"
#include "mpm_force_fields.cuh"
#include "mpm_kernels.cuh"
#include "mpm_tool_adjoint.cuh"

namespace gbmpm {
int derive_scene(const mpm_scene_config& c, SceneDev& S, std::string& err);

namespace {

struct DiffParams {
  SceneDev S;
  float mass;
  int32_t neohookean;
  const float* pmass;     // per-particle mass (mixed scenes) or null: `mass` for all
  const int32_t* pkind;   // per-particle material (DIFF_*) or null: `neohookean` for all
  const float* aux;       // per particle [2]: Sand alpha | Snow clamp bounds (null without them)
  const float* Jp;        // plastic state Jp [n] (null: Elastic / Liquid only, Jp unused)
  float* Jp1;
  const float* gJp1;      // dL/dJp of the next state (null: zero)
  float* gJp;
  int64_t n;
  const float *x, *v, *C, *F, *mu, *lam;
  float *x1, *v1, *C1, *F1;
  float4* pm;  // (momentum, mass)
  float4* gvel;  // (velocity after boundary, mass)
  // adjoints
  const float *gx1, *gv1, *gC1, *gF1;
  float *gx, *gv, *gC, *gF, *gmu, *glam;
  float4* g_grid_v;   // adjoint of the node velocity (xyz)
  float4* g_grid_pm;  // adjoint of (momentum, mass)
  uint32_t* status;
  // tool entities of the scene (Mesh.collide in the grid op, legacy_coupler.py:386-387)
  int32_t n_tools;
  DiffToolDev tools[MPM_DIFF_MAX_TOOLS];
  const float* tool_f;  // tool states (pos 3, quat 4, vel 3, ang 3) at this substep [n_tools][13]
  float* tool_f1;       // ... one substep later (written by k_dtool_advance)
  float* g_tool;        // [n_tools][12]: dL/d(pos, vel) of the next state (in) / this one (out); accumulator
  // Muscle particles (kinds DIFF_MUSCLE_*): actuation [n] (constant over the substeps of a call),
  // fibre direction [n][3], dL/dactuation [n] (added)
  const float* actu;
  const float* mdir;
  float* g_actu;
  // particle constraints (apply_particle_constraints, mpm_solver.py:1099-1128, after G2P):
  // stiffness [n] (0: none) and target [n][3], fixed over the substeps of a call; null: none
  const float* con_k;
  const float* con_t;
  // particle activity (particles_ng.active; null: all active): an inactive particle takes no part in
  // P2G and G2P and keeps its state, as mpm_solver.py's p2g / g2p skip it and copy it to f + 1
  const uint8_t* active;
};

__device__ __forceinline__ bool d_active(const DiffParams& Q, int64_t i) { return !Q.active || Q.active[i]; }

// The critically damped spring of a constrained particle of real mass m: v' = a v + b x + c with
// a = 1 - dt 2 sqrt(k m) / m, b = -dt k / m (the reference's dv = dt (-k (x - t) - 2 sqrt(k m) v) / m).
__device__ __forceinline__ void constraint_apply(float k, float m, float dt, const float* t, const float* x,
                                                 float* v) {
  const float damp = 2.f * sqrtf(k * m);
  for (int d = 0; d < 3; ++d) {
    const float f = -k * (x[d] - t[d]) - damp * v[d];
    v[d] = v[d] + dt * f / m;
  }
}

// Force fields of the differentiable grid op (legacy_coupler.py:381-383), passed by value to the
// two grid kernels only: scene index and substep counter of the noise draws, then the fields in
// the order they act.
struct DiffFields {
  int32_t n, scene;
  unsigned long long step;
  ForceFieldDev f[MPM_DIFF_MAX_FORCE_FIELDS];
};

// Kinematic rigid colliders of the differentiable grid op (legacy_coupler.py:389-403), by value like
// the fields: poses fixed over the call, applied after the tools; scene -1 or the env index.
struct DiffColliders {
  int32_t n, pad0;
  ColliderDev c[MPM_DIFF_MAX_COLLIDERS];
};

// The influence of collider c at x (normal in n), or 0 when the node is outside its reach
// (_func_collide_with_rigid: exp(-sd / softness) capped at 1, acting above 0.1).
__device__ __forceinline__ float dcollider_influence(const ColliderDev& c, const float* x, float eps, float* n) {
  const float sd = collider_sdf(c, x, eps, n);
  const float influence = fminf(expf(-sd / fmaxf(1e-10f, c.softness)), 1.f);
  return influence > 0.1f ? influence : 0.f;
}

__device__ __forceinline__ int64_t didx(const SceneDev& S, int gx, int gy, int gz) {
  return ((int64_t)gx * S.res[1] + gy) * S.res[2] + gz;
}

struct Stencil {
  int b[3];
  float fx[3], w[3][3], dw[3][3];  // weights and d w / d fx per axis
};

__device__ __forceinline__ bool make_stencil(const SceneDev& S, const float* x, Stencil& st) {
  if (!stencil_origin(S, x, st.b)) return false;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const float t = __fmul_rn(x[d], S.inv_dx);
    const float f = t - (float)(st.b[d] + S.offset[d]);
    st.fx[d] = f;
    bspline_w(f, st.w[d]);
    st.dw[d][0] = -(1.5f - f);
    st.dw[d][1] = -2.f * (f - 1.f);
    st.dw[d][2] = f - 0.5f;
  }
  return true;
}

// Material of the differentiable form (the `neohookean` argument of the entry points, or the
// per-particle kind): aux holds Sand alpha | Snow and clamped ElastoPlastic clamp bounds | von Mises
// yield_stress / (2 mu) | Muscle stiffness.
constexpr int DIFF_COROTATED = 0, DIFF_NEOHOOKEAN = 1, DIFF_LIQUID = 2, DIFF_SAND = 3, DIFF_SNOW = 4,
              DIFF_MUSCLE_COROTATED = 5, DIFF_MUSCLE_NEOHOOKEAN = 6, DIFF_EP_CLAMP = 7, DIFF_EP_VON_MISES = 8;

__device__ __forceinline__ bool diff_plastic(int kind) {
  return kind == DIFF_SAND || kind == DIFF_SNOW || kind == DIFF_EP_CLAMP || kind == DIFF_EP_VON_MISES;
}
__device__ __forceinline__ bool diff_muscle(int kind) {
  return kind == DIFF_MUSCLE_COROTATED || kind == DIFF_MUSCLE_NEOHOOKEAN;
}
// the law of plastic_adjoint (mpm_adjoint.cuh) for a plastic kind
__device__ __forceinline__ int diff_plastic_law(int kind) {
  return kind == DIFF_SAND ? MT_SAND : (kind == DIFF_SNOW ? MT_SNOW : (kind == DIFF_EP_CLAMP ? MT_ELASTOPLASTIC : EP_VON_MISES));
}

// A plastic particle's material as the product path's material table holds it (mpm_math.cuh)
__device__ __forceinline__ MaterialDev plastic_material(int kind, float mu, float lam, const float* aux) {
  MaterialDev M;
  M.type = kind == DIFF_SAND ? MT_SAND : (kind == DIFF_SNOW ? MT_SNOW : MT_ELASTOPLASTIC);
  M.flags = kind == DIFF_EP_VON_MISES ? MF_VON_MISES : 0;
  M.mu = mu;
  M.lam = lam;
  M.alpha = kind == DIFF_SAND ? aux[0] : 0.f;
  M.sand_coef = (3.f * lam + 2.f * mu) / (2.f * mu);
  M.clamp_lo = aux[0];
  M.clamp_hi = aux[1];
  M.vm_ratio = aux[0];
  return M;
}

// Muscle actuation stress (muscle.py:46-53): stiffness * actu * (F m)(F m)^T, added as the product
// path's material_update adds it
__device__ __forceinline__ void muscle_stress(const float* Ft, const float* m, float stiffness, float actu, float* P) {
  float fm[3];
  for (int r = 0; r < 3; ++r) fm[r] = Ft[r * 3 + 0] * m[0] + Ft[r * 3 + 1] * m[1] + Ft[r * 3 + 2] * m[2];
  const float k = stiffness * actu;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) P[r * 3 + c] += k * fm[r] * fm[c];
}

__device__ __forceinline__ float p_mass(const DiffParams& Q, int64_t i) { return Q.pmass ? Q.pmass[i] : Q.mass; }
__device__ __forceinline__ int p_kind(const DiffParams& Q, int64_t i) { return Q.pkind ? Q.pkind[i] : Q.neohookean; }

// corotated / neo-Hookean stress of elastic.py:48-60 with per-particle mu, lam; F_new = F_tmp
// (liquid: the corotated form with its mu, 0 unless viscous; F_new = J^(1/3) I)
__device__ __forceinline__ void elastic_stress(const float* Ft, float mu, float lam, bool neo, const float* U,
                                               const float* sig, const float* V, float* P) {
  const float J = sig[0] * sig[1] * sig[2];
  if (neo) {
    stress_neohookean(mu, lam, Ft, J, P);
  } else {
    stress_corotated(mu, lam, Ft, U, V, J, P);
  }
}

__device__ __forceinline__ void f_tmp(const float* C, const float* F, float dt, float* Ft) {
  float A[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) A[k] = ((k % 4 == 0) ? 1.f : 0.f) + dt * C[k];
  mat_mul(A, F, Ft);
}

__device__ __forceinline__ void svd_f32(const float* Ft, float* U, float* sig, float* V) {
  const float res = svd3<float, SVD_SWEEPS>(Ft, U, sig, V);
  if (!svd_accurate(res, sig, SVD_FP64_TOL)) {
    double Ad[9], Ud[9], sd[3], Vd[9];
    for (int k = 0; k < 9; ++k) Ad[k] = Ft[k];
    svd3<double, 8>(Ad, Ud, sd, Vd);
    for (int k = 0; k < 9; ++k) {
      U[k] = (float)Ud[k];
      V[k] = (float)Vd[k];
    }
    for (int k = 0; k < 3; ++k) sig[k] = (float)sd[k];
  }
}

// ------------------------------------------------------------------ forward
__global__ void k_dclear(DiffParams Q, int64_t nodes, float4* buf) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nodes; i += (int64_t)gridDim.x * blockDim.x)
    buf[i] = make_float4(0.f, 0.f, 0.f, 0.f);
}

// One particle's part of P2G: the material update (F1, Jp1 written), its stencil, A = s P + m C and
// m v.  False when it scatters nothing (inactive: carried unchanged; outside the grid: flagged).
__device__ __forceinline__ bool dp2g_particle(const DiffParams& Q, int64_t i, Stencil& st, float* A, float* mv,
                                              float& mass) {
  const SceneDev& S = Q.S;
  float x[3], v[3], C[9], F[9];
  for (int d = 0; d < 3; ++d) {
    x[d] = Q.x[i * 3 + d];
    v[d] = Q.v[i * 3 + d];
  }
  for (int k = 0; k < 9; ++k) {
    C[k] = Q.C[i * 9 + k];
    F[k] = Q.F[i * 9 + k];
  }
  if (!d_active(Q, i)) {  // carried unchanged (g2p's else branch copies F and Jp)
    if (Q.F1)
      for (int k = 0; k < 9; ++k) Q.F1[i * 9 + k] = F[k];
    if (Q.Jp1) Q.Jp1[i] = Q.Jp[i];
    return false;
  }
  if (!make_stencil(S, x, st)) {
    atomicOr(Q.status, 2u);
    return false;
  }
  mass = p_mass(Q, i);
  const int kind = p_kind(Q, i);
  float Ft[9], U[9], sig[3], V[9], P[9];
  f_tmp(C, F, S.dt, Ft);
  svd_f32(Ft, U, sig, V);
  const bool plastic = diff_plastic(kind);
  if (plastic) {  // sand.py:47-84, snow.py:56-74, elasto_plastic.py:44-71 (the product path's code)
    const MaterialDev M = plastic_material(kind, Q.mu[i], Q.lam[i], Q.aux + i * 2);
    const float mdir[3] = {0.f, 0.f, 1.f};
    float Fn[9], Jpn;
    material_update<float>(M, Ft, U, sig, V, Q.Jp[i], 0.f, mdir, S.eps, Fn, Jpn, P);
    if (Q.F1)
      for (int k = 0; k < 9; ++k) Q.F1[i * 9 + k] = Fn[k];
    if (Q.Jp1) Q.Jp1[i] = Jpn;
  } else {
    elastic_stress(Ft, Q.mu[i], Q.lam[i], kind == DIFF_NEOHOOKEAN || kind == DIFF_MUSCLE_NEOHOOKEAN, U, sig, V, P);
    if (diff_muscle(kind) && Q.actu) muscle_stress(Ft, Q.mdir + i * 3, Q.aux[i * 2], Q.actu[i], P);
    if (Q.Jp1) Q.Jp1[i] = Q.Jp[i];
  }
  if (Q.F1 && !plastic) {
    if (kind == DIFF_LIQUID) {  // liquid.py:36-40: F_new = J^(1/3) I
      const float j3 = powf(sig[0] * sig[1] * sig[2], 1.f / 3.f);
      for (int k = 0; k < 9; ++k) Q.F1[i * 9 + k] = (k % 4 == 0) ? j3 : 0.f;
    } else {
      for (int k = 0; k < 9; ++k) Q.F1[i * 9 + k] = Ft[k];
    }
  }
  for (int k = 0; k < 9; ++k) A[k] = S.stress_scale * P[k] + mass * C[k];
  for (int d = 0; d < 3; ++d) mv[d] = mass * v[d];
  return true;
}

// Groups of the lanes of a warp with equal keys (particles with the same stencil origin scatter to
// the same 27 nodes; neighbours in memory often share a cell).  peer_sum adds a value over the group
// into its lowest lane (`lead`), which alone then issues the float4 global atomic.  The sum is a tree
// over the group's ranks: in round r every lane adds the value of its next remaining peer above
// (nxt[r] = that lane + 1, 0 for none), then the lanes whose rank has bit r set drop out; five rounds
// cover a group of 32.  Every lane of the warp must call both (full-warp shuffles).
struct PeerTree {
  int nxt[5];
  int rounds;  // the same for the whole warp
  bool lead;
};

__device__ __forceinline__ PeerTree peer_tree(unsigned long long key) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const unsigned peers = __match_any_sync(full, key);
  PeerTree t;
  t.lead = (peers & ((1u << lane) - 1u)) == 0u;
  unsigned above = peers & (0xfffffffeu << lane);
  unsigned rank = __popc(peers & ((1u << lane) - 1u));
  t.rounds = 0;
#pragma unroll
  for (int r = 0; r < 5; ++r) {
    t.nxt[r] = 0;
    if (__any_sync(full, above != 0u)) {
      t.nxt[r] = __ffs(above);
      above &= ~__ballot_sync(full, (rank & 1u) != 0u);
      rank >>= 1;
      t.rounds = r + 1;
    }
  }
  return t;
}

__device__ __forceinline__ float4 peer_sum(const PeerTree& t, float4 g) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int r = 0; r < 5; ++r) {
    if (r < t.rounds) {
      const int src = t.nxt[r] ? t.nxt[r] - 1 : lane;
      const float tx = __shfl_sync(full, g.x, src), ty = __shfl_sync(full, g.y, src);
      const float tz = __shfl_sync(full, g.z, src), tw = __shfl_sync(full, g.w, src);
      if (t.nxt[r]) g.x += tx, g.y += ty, g.z += tz, g.w += tw;
    }
  }
  return g;
}

// A key no stencil origin has, distinct per lane (a lane without a particle to scatter).
__device__ __forceinline__ unsigned long long no_peer_key() { return ~0ull - (unsigned long long)(threadIdx.x & 31); }

// P2G, its float4 global atomics summed over peer groups first.
__global__ void __launch_bounds__(256) k_dp2g(DiffParams Q) {
  const SceneDev& S = Q.S;
  // the trip count is the same for the whole warp (blockDim and the stride are multiples of 32),
  // so every lane reaches the warp-wide operations below
  for (int64_t w0 = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31); w0 < Q.n;
       w0 += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = w0 + (threadIdx.x & 31);
    Stencil st;
    float A[9], mv[3], mass = 0.f;
    const bool has = i < Q.n && dp2g_particle(Q, i, st, A, mv, mass);
    const PeerTree pt = peer_tree(has ? (unsigned long long)didx(S, st.b[0], st.b[1], st.b[2]) : no_peer_key());
#pragma unroll
    for (int ox = 0; ox < 3; ++ox)
#pragma unroll
      for (int oy = 0; oy < 3; ++oy)
#pragma unroll
        for (int oz = 0; oz < 3; ++oz) {
          float4 g = make_float4(0.f, 0.f, 0.f, 0.f);
          if (has) {
            const float wt = st.w[0][ox] * st.w[1][oy] * st.w[2][oz];
            const float dp[3] = {((float)ox - st.fx[0]) * S.dx, ((float)oy - st.fx[1]) * S.dx,
                                 ((float)oz - st.fx[2]) * S.dx};
            g.x = wt * (mv[0] + A[0] * dp[0] + A[1] * dp[1] + A[2] * dp[2]);
            g.y = wt * (mv[1] + A[3] * dp[0] + A[4] * dp[1] + A[5] * dp[2]);
            g.z = wt * (mv[2] + A[6] * dp[0] + A[7] * dp[1] + A[8] * dp[2]);
            g.w = wt * mass;
          }
          g = peer_sum(pt, g);
          if (has && pt.lead) atomicAdd(&Q.pm[didx(S, st.b[0] + ox, st.b[1] + oy, st.b[2] + oz)], g);
        }
  }
}

// Tools advance one substep (ToolEntity.advect) before the grid op that needs both poses.
__global__ void k_dtool_advance(DiffParams Q) {
  const int t = threadIdx.x;
  if (t < Q.n_tools)
    tool_advance_state(Q.tool_f + t * 13, Q.S.dt, Q.S.eps, Q.tools[t].floor_h, Q.tool_f1 + t * 13);
}

__device__ __forceinline__ void node_world_pos(const SceneDev& S, const int* g, float* x) {
#pragma unroll
  for (int d = 0; d < 3; ++d) x[d] = (float)(g[d] + S.offset[d]) * S.dx;
}

// The velocity one force field leaves at node g (world position x), as the product grid op adds it.
__device__ __forceinline__ void dfield_apply(const DiffFields& FF, int f, const SceneDev& S, const int* g,
                                             const float* x, float* v) {
  const int gw[3] = {g[0] + S.offset[0], g[1] + S.offset[1], g[2] + S.offset[2]};
  float a[3];
  ff_acc(FF.f[f], x, v, S.eps, a, FF.scene, gw, FF.step);
  for (int k = 0; k < 3; ++k) v[k] += a[k] * S.dt;
}

// The grid op, whole (stage 0) or in the stages a Custom force field splits it into (the product
// path's mpm_substep_grid_stage): stage 1 gravity and the fields given, from the P2G grid into the
// velocity buffer; stage 2 more fields on the velocity buffer; stage 3 the tools, colliders and
// boundary on it.  Nodes without mass hold zero velocity.
__global__ void k_dgrid(DiffParams Q, int64_t nodes, const DiffFields FF, const DiffColliders CC, int stage) {
  const SceneDev& S = Q.S;
  const bool fields = stage <= 2, tail = stage == 0 || stage == 3;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nodes; i += (int64_t)gridDim.x * blockDim.x) {
    const float4 q = Q.pm[i];
    float v[3] = {0.f, 0.f, 0.f};
    if (q.w > S.eps) {
      const int g[3] = {(int)(i / ((int64_t)S.res[1] * S.res[2])), (int)((i / S.res[2]) % S.res[1]), (int)(i % S.res[2])};
      if (stage <= 1) {
        const float inv = 1.f / q.w;
        v[0] = inv * q.x + S.dt * S.grav[0];
        v[1] = inv * q.y + S.dt * S.grav[1];
        v[2] = inv * q.z + S.dt * S.grav[2];
      } else {  // the velocity the earlier stages (and the Custom fields between them) left
        const float4 u = Q.gvel[i];
        v[0] = u.x, v[1] = u.y, v[2] = u.z;
      }
      if ((fields && FF.n > 0) || (tail && (Q.n_tools > 0 || CC.n > 0))) {
        float x[3];
        node_world_pos(S, g, x);
        if (fields)
          for (int f = 0; f < FF.n; ++f)  // force fields after gravity, before the tools
            if (FF.f[f].active) dfield_apply(FF, f, S, g, x, v);
        if (tail) {
          for (int t = 0; t < Q.n_tools; ++t) {
            const float* st = Q.tool_f + t * 13;
            tool_collide_t<float>(Q.tools[t], x, v, st, st + 3, st + 7, Q.tool_f1 + t * 13 + 3, S.dt, S.eps);
          }
          for (int ci = 0; ci < CC.n; ++ci) {  // rigid colliders after the tools (legacy_coupler.py:386-403)
            const ColliderDev& c = CC.c[ci];
            if (c.scene >= 0 && c.scene != FF.scene) continue;
            float n[3];
            const float infl = dcollider_influence(c, x, S.eps, n);
            if (infl > 0.f) collide_in_velocity(c, S.eps, x, v, n, infl);
          }
        }
      }
      if (tail)
        for (int d = 0; d < 3; ++d) {
          const float p = (float)(g[d] + S.offset[d]) * S.dx;
          if ((p >= S.hi[d] && v[d] >= 0.f) || (p <= S.lo[d] && v[d] <= 0.f)) v[d] = 0.f;
        }
    }
    Q.gvel[i] = make_float4(v[0], v[1], v[2], q.w);
  }
}

__global__ void __launch_bounds__(256) k_dg2p(DiffParams Q) {
  const SceneDev& S = Q.S;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < Q.n; i += (int64_t)gridDim.x * blockDim.x) {
    float x[3];
    for (int d = 0; d < 3; ++d) x[d] = Q.x[i * 3 + d];
    if (!d_active(Q, i)) {
      for (int d = 0; d < 3; ++d) {
        Q.x1[i * 3 + d] = x[d];
        Q.v1[i * 3 + d] = Q.v[i * 3 + d];
      }
      for (int k = 0; k < 9; ++k) Q.C1[i * 9 + k] = Q.C[i * 9 + k];
      continue;
    }
    Stencil st;
    if (!make_stencil(S, x, st)) continue;
    float v[3] = {0.f, 0.f, 0.f}, Cn[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int ox = 0; ox < 3; ++ox)
      for (int oy = 0; oy < 3; ++oy)
        for (int oz = 0; oz < 3; ++oz) {
          const float4 g = Q.gvel[didx(S, st.b[0] + ox, st.b[1] + oy, st.b[2] + oz)];
          const float wt = st.w[0][ox] * st.w[1][oy] * st.w[2][oz];
          const float dp[3] = {(float)ox - st.fx[0], (float)oy - st.fx[1], (float)oz - st.fx[2]};
          const float gv[3] = {g.x, g.y, g.z};
          for (int r = 0; r < 3; ++r) {
            v[r] += wt * gv[r];
            for (int c = 0; c < 3; ++c) Cn[r * 3 + c] += 4.f * S.inv_dx * wt * gv[r] * dp[c];
          }
        }
    float x1[3], v1[3];
    for (int d = 0; d < 3; ++d) {
      const float xn = x[d] + S.dt * v[d];
      float vd = v[d];
      if ((xn >= S.hi[d] && vd >= 0.f) || (xn <= S.lo[d] && vd <= 0.f)) vd = 0.f;
      x1[d] = fmaxf(fminf(xn, S.hi[d]), S.lo[d]);
      v1[d] = vd;
      if (!isfinite(xn)) atomicOr(Q.status, 1u);
    }
    if (Q.con_k && Q.con_k[i] > 0.f) constraint_apply(Q.con_k[i], p_mass(Q, i) / 1e3f, S.dt, Q.con_t + i * 3, x1, v1);
    for (int d = 0; d < 3; ++d) {
      Q.x1[i * 3 + d] = x1[d];
      Q.v1[i * 3 + d] = v1[d];
    }
    for (int k = 0; k < 9; ++k) Q.C1[i * 9 + k] = Cn[k];
  }
}

// ------------------------------------------------------------------ adjoint
// G2P adjoint: from dL/d(x1, v1, C1) to dL/d(node velocity) (atomics) and the part of dL/dx
// through x1 = clamp(x + dt v1), the G2P weights and the (x_i - x_p) factor of C1.
__global__ void __launch_bounds__(256) k_dg2p_adj(DiffParams Q) {
  const SceneDev& S = Q.S;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < Q.n; i += (int64_t)gridDim.x * blockDim.x) {
    float x[3];
    for (int d = 0; d < 3; ++d) x[d] = Q.x[i * 3 + d];
    if (!d_active(Q, i)) {  // x1 = x
      for (int d = 0; d < 3; ++d) Q.gx[i * 3 + d] = Q.gx1[i * 3 + d];
      continue;
    }
    Stencil st;
    if (!make_stencil(S, x, st)) {
      for (int d = 0; d < 3; ++d) Q.gx[i * 3 + d] = 0.f;
      continue;
    }
    // recompute the gathered velocity (needed for the boundary masks)
    float v[3] = {0.f, 0.f, 0.f};
    for (int ox = 0; ox < 3; ++ox)
      for (int oy = 0; oy < 3; ++oy)
        for (int oz = 0; oz < 3; ++oz) {
          const float4 g = Q.gvel[didx(S, st.b[0] + ox, st.b[1] + oy, st.b[2] + oz)];
          const float wt = st.w[0][ox] * st.w[1][oy] * st.w[2][oz];
          v[0] += wt * g.x;
          v[1] += wt * g.y;
          v[2] += wt * g.z;
        }
    float gx1[3], gv1[3];
    for (int d = 0; d < 3; ++d) {
      gx1[d] = Q.gx1[i * 3 + d];
      gv1[d] = Q.gv1[i * 3 + d];
    }
    if (Q.con_k && Q.con_k[i] > 0.f) {  // back through the constraint spring: v' = a v + b x + c
      const float k = Q.con_k[i], m = p_mass(Q, i) / 1e3f;
      const float a = 1.f - S.dt * 2.f * sqrtf(k * m) / m, b = -S.dt * k / m;
      for (int d = 0; d < 3; ++d) {
        gx1[d] += b * gv1[d];
        gv1[d] *= a;
      }
    }
    float gxn[3], gvv[3], gx[3];
    for (int d = 0; d < 3; ++d) {
      const float xn = x[d] + S.dt * v[d];
      const bool zero_v = (xn >= S.hi[d] && v[d] >= 0.f) || (xn <= S.lo[d] && v[d] <= 0.f);
      const bool inside = xn > S.lo[d] && xn < S.hi[d];
      gxn[d] = inside ? gx1[d] : 0.f;
      gvv[d] = (zero_v ? 0.f : gv1[d]) + S.dt * gxn[d];
      gx[d] = gxn[d];
    }
    float gC[9];
    for (int k = 0; k < 9; ++k) gC[k] = Q.gC1[i * 9 + k];
    const float kc = 4.f * S.inv_dx;
    for (int ox = 0; ox < 3; ++ox)
      for (int oy = 0; oy < 3; ++oy)
        for (int oz = 0; oz < 3; ++oz) {
          const int o[3] = {ox, oy, oz};
          const float4 g = Q.gvel[didx(S, st.b[0] + ox, st.b[1] + oy, st.b[2] + oz)];
          const float gvn[3] = {g.x, g.y, g.z};
          const float wt = st.w[0][ox] * st.w[1][oy] * st.w[2][oz];
          const float dp[3] = {(float)ox - st.fx[0], (float)oy - st.fx[1], (float)oz - st.fx[2]};
          // gC dp (3-vector) and gC^T v_i
          float gCdp[3], gCtv[3];
          for (int r = 0; r < 3; ++r) gCdp[r] = gC[r * 3 + 0] * dp[0] + gC[r * 3 + 1] * dp[1] + gC[r * 3 + 2] * dp[2];
          for (int c = 0; c < 3; ++c) gCtv[c] = gC[0 * 3 + c] * gvn[0] + gC[1 * 3 + c] * gvn[1] + gC[2 * 3 + c] * gvn[2];
          float4 add;
          add.x = wt * (gvv[0] + kc * gCdp[0]);
          add.y = wt * (gvv[1] + kc * gCdp[1]);
          add.z = wt * (gvv[2] + kc * gCdp[2]);
          add.w = 0.f;
          atomicAdd(&Q.g_grid_v[didx(S, st.b[0] + ox, st.b[1] + oy, st.b[2] + oz)], add);
          // d(dp)/dx = -inv_dx I
          for (int c = 0; c < 3; ++c) gx[c] += -kc * S.inv_dx * wt * gCtv[c];
          // weight adjoint
          const float wbar = gvv[0] * gvn[0] + gvv[1] * gvn[1] + gvv[2] * gvn[2] + kc * (gvn[0] * gCdp[0] + gvn[1] * gCdp[1] + gvn[2] * gCdp[2]);
          const float dw[3] = {st.dw[0][o[0]] * st.w[1][o[1]] * st.w[2][o[2]], st.w[0][o[0]] * st.dw[1][o[1]] * st.w[2][o[2]],
                               st.w[0][o[0]] * st.w[1][o[1]] * st.dw[2][o[2]]};
          for (int c = 0; c < 3; ++c) gx[c] += wbar * dw[c] * S.inv_dx;
        }
    for (int d = 0; d < 3; ++d) Q.gx[i * 3 + d] = gx[d];
  }
}

// grid-op adjoint: v = B(T(F(p/m + dt g))) (force fields F, tools T, boundary B) -> dL/dp, dL/dm
// Adjoint of one stage of k_dgrid (0: whole).  Stages 2 and 3 take the velocity that stage began
// from in vin and turn dL/d(its output) in g_grid_v into dL/d(its input) in place; stages 0 and 1
// end at the P2G grid, dL/d(momentum, mass) into g_grid_pm.
__global__ void k_dgrid_adj(DiffParams Q, int64_t nodes, const DiffFields FF, const DiffColliders CC, int stage,
                            const float4* vstage) {
  const bool fields = stage <= 2, tail = stage == 0 || stage == 3, from_pm = stage <= 1;
  const SceneDev& S = Q.S;
  const int lane = threadIdx.x & 31;
  for (int64_t i0 = (int64_t)blockIdx.x * blockDim.x; i0 < nodes; i0 += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = i0 + threadIdx.x;  // warp-uniform loop: the tool sums are reduced across the warp
    const float4 q = i < nodes ? Q.pm[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    float4 out = make_float4(0.f, 0.f, 0.f, 0.f);
    float tacc[MPM_DIFF_MAX_TOOLS][6];
    for (int t = 0; t < Q.n_tools; ++t)
      for (int k = 0; k < 6; ++k) tacc[t][k] = 0.f;
    if (i < nodes && q.w > S.eps) {
      const float4 gv = Q.g_grid_v[i];
      const int g[3] = {(int)(i / ((int64_t)S.res[1] * S.res[2])), (int)((i / S.res[2]) % S.res[1]), (int)(i % S.res[2])};
      const float inv = 1.f / q.w;
      float u[3] = {inv * q.x + S.dt * S.grav[0], inv * q.y + S.dt * S.grav[1], inv * q.z + S.dt * S.grav[2]};
      if (!from_pm) {
        const float4 w = vstage[i];
        u[0] = w.x, u[1] = w.y, u[2] = w.z;
      }
      float gu[3] = {gv.x, gv.y, gv.z};
      float vin[MPM_DIFF_MAX_TOOLS][3], fin[MPM_DIFF_MAX_FORCE_FIELDS][3], cin[MPM_DIFF_MAX_COLLIDERS][3];
      float x[3];
      node_world_pos(S, g, x);
      const int n_ff = fields ? FF.n : 0, n_tools = tail ? Q.n_tools : 0, n_col = tail ? CC.n : 0;
      for (int f = 0; f < n_ff; ++f) {  // forward through the force fields, keeping each one's input
        for (int k = 0; k < 3; ++k) fin[f][k] = u[k];
        if (FF.f[f].active) dfield_apply(FF, f, S, g, x, u);
      }
      for (int t = 0; t < n_tools; ++t) {  // forward through the tools, keeping each one's input
        for (int k = 0; k < 3; ++k) vin[t][k] = u[k];
        const float* st = Q.tool_f + t * 13;
        tool_collide_t<float>(Q.tools[t], x, u, st, st + 3, st + 7, Q.tool_f1 + t * 13 + 3, S.dt, S.eps);
      }
      for (int ci = 0; ci < n_col; ++ci) {  // forward through the rigid colliders, keeping each one's input
        for (int k = 0; k < 3; ++k) cin[ci][k] = u[k];
        const ColliderDev& c = CC.c[ci];
        if (c.scene >= 0 && c.scene != FF.scene) continue;
        float n[3];
        const float infl = dcollider_influence(c, x, S.eps, n);
        if (infl > 0.f) collide_in_velocity(c, S.eps, x, u, n, infl);
      }
      if (tail)
        for (int d = 0; d < 3; ++d) {  // the boundary acts on the velocity the tools and colliders left
          const float p = (float)(g[d] + S.offset[d]) * S.dx;
          if ((p >= S.hi[d] && u[d] >= 0.f) || (p <= S.lo[d] && u[d] <= 0.f)) gu[d] = 0.f;
        }
      for (int ci = n_col - 1; ci >= 0; --ci) {  // back through the rigid colliders
        const ColliderDev& c = CC.c[ci];
        if (c.scene >= 0 && c.scene != FF.scene) continue;
        float n[3];
        const float infl = dcollider_influence(c, x, S.eps, n);
        if (infl > 0.f) collide_in_vjp(c, S.eps, x, cin[ci], n, infl, gu);
      }
      for (int t = n_tools - 1; t >= 0; --t) {  // back through the tools: Jacobians from dual numbers
        const float* st = Q.tool_f + t * 13;
        TD vt[3], pt[3], ut[3];
        for (int k = 0; k < 3; ++k) {
          vt[k] = td_var(vin[t][k], k);
          pt[k] = td_var(st[k], 3 + k);
          ut[k] = td_var(st[7 + k], 6 + k);
        }
        tool_collide_t<TD>(Q.tools[t], x, vt, pt, st + 3, ut, Q.tool_f1 + t * 13 + 3, S.dt, S.eps);
        float gin[3];
        for (int j = 0; j < 3; ++j) {
          gin[j] = gu[0] * vt[0].d[j] + gu[1] * vt[1].d[j] + gu[2] * vt[2].d[j];
          tacc[t][j] = gu[0] * vt[0].d[3 + j] + gu[1] * vt[1].d[3 + j] + gu[2] * vt[2].d[3 + j];
          tacc[t][3 + j] = gu[0] * vt[0].d[6 + j] + gu[1] * vt[1].d[6 + j] + gu[2] * vt[2].d[6 + j];
        }
        for (int j = 0; j < 3; ++j) gu[j] = gin[j];
      }
      for (int f = n_ff - 1; f >= 0; --f)  // back through the force fields: g += dt J^T g
        if (FF.f[f].active) ff_acc_vjp(FF.f[f], x, fin[f], S.eps, S.dt, gu);
      if (from_pm) {
        out.x = gu[0] * inv;
        out.y = gu[1] * inv;
        out.z = gu[2] * inv;
        out.w = -(gu[0] * q.x + gu[1] * q.y + gu[2] * q.z) * inv * inv;
      } else {  // dL/d(the stage's input velocity)
        out = make_float4(gu[0], gu[1], gu[2], 0.f);
      }
    }
    if (i < nodes) {
      if (from_pm) Q.g_grid_pm[i] = out;
      else Q.g_grid_v[i] = out;
    }
    for (int t = 0; t < Q.n_tools; ++t)  // the tool's share of dL/d(pos, vel), one atomic per warp
      for (int k = 0; k < 6; ++k) {
        float a = tacc[t][k];
        for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
        if (lane == 0 && a != 0.f) atomicAdd(Q.g_tool + t * 12 + 6 + k, a);
      }
  }
}

// The tool state chain backwards over one substep (ToolEntity.advect: pos' = max(pos + vel dt,
// floor) in z, vel' = vel), plus this substep's collision terms; the accumulator is cleared.
__global__ void k_dtool_adj(DiffParams Q) {
  const int t = threadIdx.x;
  if (t >= Q.n_tools) return;
  float* g = Q.g_tool + t * 12;
  const float* s = Q.tool_f + t * 13;
  const bool clamped = s[2] + s[9] * Q.S.dt < Q.tools[t].floor_h;
  float gp[3] = {g[0], g[1], clamped ? 0.f : g[2]};
  for (int k = 0; k < 3; ++k) {
    const float gpk = gp[k];
    g[k] = gpk + g[6 + k];
    g[3 + k] = g[3 + k] + Q.S.dt * gpk + g[9 + k];
    g[6 + k] = 0.f;
    g[9 + k] = 0.f;
  }
}

__global__ void k_dtool_zero_acc(DiffParams Q) {
  const int t = threadIdx.x;
  if (t < Q.n_tools)
    for (int k = 6; k < 12; ++k) Q.g_tool[t * 12 + k] = 0.f;
}

// Adjoint of the rotation of the polar decomposition: given Rbar = dL/dR, returns dL/dF
// contribution 2 R Y with Y = V Z V^T, Z_ij = (V^T skew(R^T Rbar) V)_ij / (s_i + s_j).
__device__ __forceinline__ void polar_rotation_adj(const float* U, const float* sig, const float* V, const float* Rb,
                                                   float* Fb) {
  float R[9];
  mat_mul_bt(U, V, R);
  float RtRb[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) RtRb[i * 3 + j] = R[0 * 3 + i] * Rb[0 * 3 + j] + R[1 * 3 + i] * Rb[1 * 3 + j] + R[2 * 3 + i] * Rb[2 * 3 + j];
  float K[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) K[i * 3 + j] = 0.5f * (RtRb[i * 3 + j] - RtRb[j * 3 + i]);
  // W = V^T K V
  float KV[9], W[9];
  mat_mul(K, V, KV);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) W[i * 3 + j] = V[0 * 3 + i] * KV[0 * 3 + j] + V[1 * 3 + i] * KV[1 * 3 + j] + V[2 * 3 + i] * KV[2 * 3 + j];
  float Z[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      float den = sig[i] + sig[j];
      den = fabsf(den) < 1e-6f ? (den < 0.f ? -1e-6f : 1e-6f) : den;
      Z[i * 3 + j] = (i == j) ? 0.f : W[i * 3 + j] / den;
    }
  // Y = V Z V^T ; Fb += 2 R Y
  float VZ[9], Y[9], RY[9];
  mat_mul(V, Z, VZ);
  mat_mul_bt(VZ, V, Y);
  mat_mul(R, Y, RY);
  for (int k = 0; k < 9; ++k) Fb[k] += 2.f * RY[k];
}

// P2G adjoint + stress adjoint + F_tmp adjoint: from dL/d(node momentum, mass) and dL/dF1 to
// dL/d(x, v, C, F, mu, lam); adds the P2G part of dL/dx to the G2P part already in gx.
__global__ void __launch_bounds__(128) k_dp2g_adj(DiffParams Q) {
  const SceneDev& S = Q.S;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < Q.n; i += (int64_t)gridDim.x * blockDim.x) {
    float x[3], v[3], C[9], F[9];
    for (int d = 0; d < 3; ++d) {
      x[d] = Q.x[i * 3 + d];
      v[d] = Q.v[i * 3 + d];
    }
    for (int k = 0; k < 9; ++k) {
      C[k] = Q.C[i * 9 + k];
      F[k] = Q.F[i * 9 + k];
    }
    if (!d_active(Q, i)) {  // (v1, C1, F1, Jp1) = (v, C, F, Jp); dL/dx already holds dL/dx1
      for (int d = 0; d < 3; ++d) Q.gv[i * 3 + d] = Q.gv1[i * 3 + d];
      for (int k = 0; k < 9; ++k) {
        Q.gC[i * 9 + k] = Q.gC1[i * 9 + k];
        Q.gF[i * 9 + k] = Q.gF1 ? Q.gF1[i * 9 + k] : 0.f;
      }
      if (Q.gJp) Q.gJp[i] = Q.gJp1 ? Q.gJp1[i] : 0.f;
      continue;
    }
    Stencil st;
    if (!make_stencil(S, x, st)) {
      for (int d = 0; d < 3; ++d) Q.gv[i * 3 + d] = 0.f;
      for (int k = 0; k < 9; ++k) {
        Q.gC[i * 9 + k] = 0.f;
        Q.gF[i * 9 + k] = Q.gF1 ? Q.gF1[i * 9 + k] : 0.f;
      }
      if (Q.gJp) Q.gJp[i] = Q.gJp1 ? Q.gJp1[i] : 0.f;
      continue;
    }
    const float mu = Q.mu[i], lam = Q.lam[i];
    const float mass = p_mass(Q, i);
    const int kind = p_kind(Q, i);
    const bool plastic = diff_plastic(kind), neo = kind == DIFF_NEOHOOKEAN || kind == DIFF_MUSCLE_NEOHOOKEAN;
    float Ft[9], U[9], sig[3], V[9], P[9];
    f_tmp(C, F, S.dt, Ft);
    svd_f32(Ft, U, sig, V);
    if (plastic) {
      const MaterialDev M = plastic_material(kind, mu, lam, Q.aux + i * 2);
      const float mdir[3] = {0.f, 0.f, 1.f};
      float Fn[9], Jpn;
      material_update<float>(M, Ft, U, sig, V, Q.Jp[i], 0.f, mdir, S.eps, Fn, Jpn, P);
    } else {
      elastic_stress(Ft, mu, lam, neo, U, sig, V, P);
      if (diff_muscle(kind) && Q.actu) muscle_stress(Ft, Q.mdir + i * 3, Q.aux[i * 2], Q.actu[i], P);
    }
    float A[9];
    for (int k = 0; k < 9; ++k) A[k] = S.stress_scale * P[k] + mass * C[k];
    float gv[3] = {0.f, 0.f, 0.f}, gA[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, gx[3];
    for (int d = 0; d < 3; ++d) gx[d] = Q.gx[i * 3 + d];
    for (int ox = 0; ox < 3; ++ox)
      for (int oy = 0; oy < 3; ++oy)
        for (int oz = 0; oz < 3; ++oz) {
          const int o[3] = {ox, oy, oz};
          const float4 g = Q.g_grid_pm[didx(S, st.b[0] + ox, st.b[1] + oy, st.b[2] + oz)];
          const float gp[3] = {g.x, g.y, g.z};
          const float wt = st.w[0][ox] * st.w[1][oy] * st.w[2][oz];
          const float dp[3] = {((float)ox - st.fx[0]) * S.dx, ((float)oy - st.fx[1]) * S.dx,
                               ((float)oz - st.fx[2]) * S.dx};
          float mom[3];
          for (int r = 0; r < 3; ++r) mom[r] = mass * v[r] + A[r * 3 + 0] * dp[0] + A[r * 3 + 1] * dp[1] + A[r * 3 + 2] * dp[2];
          for (int r = 0; r < 3; ++r) {
            gv[r] += mass * wt * gp[r];
            for (int c = 0; c < 3; ++c) gA[r * 3 + c] += wt * gp[r] * dp[c];
          }
          // d(dp)/dx = -I : -A^T gp
          for (int c = 0; c < 3; ++c) gx[c] += -wt * (A[0 * 3 + c] * gp[0] + A[1 * 3 + c] * gp[1] + A[2 * 3 + c] * gp[2]);
          const float wbar = gp[0] * mom[0] + gp[1] * mom[1] + gp[2] * mom[2] + g.w * mass;
          const float dw[3] = {st.dw[0][o[0]] * st.w[1][o[1]] * st.w[2][o[2]], st.w[0][o[0]] * st.dw[1][o[1]] * st.w[2][o[2]],
                               st.w[0][o[0]] * st.w[1][o[1]] * st.dw[2][o[2]]};
          for (int c = 0; c < 3; ++c) gx[c] += wbar * dw[c] * S.inv_dx;
        }
    // A = s P + m C
    float gP[9], gC[9], gFt[9];
    const float J = sig[0] * sig[1] * sig[2];
    for (int k = 0; k < 9; ++k) {
      gP[k] = S.stress_scale * gA[k];
      gC[k] = mass * gA[k];
      gFt[k] = (Q.gF1 && kind != DIFF_LIQUID) ? Q.gF1[i * 9 + k] : 0.f;  // F1 = F_tmp
    }
    if (Q.gF1 && kind == DIFF_LIQUID) {
      // F1 = J^(1/3) I: dL/dJ = tr(gF1) J^(-2/3) / 3, dJ/dF_tmp = cof(F_tmp)
      const float gJ = (Q.gF1[i * 9 + 0] + Q.gF1[i * 9 + 4] + Q.gF1[i * 9 + 8]) * powf(J, -2.f / 3.f) / 3.f;
      gFt[0] += gJ * (Ft[4] * Ft[8] - Ft[5] * Ft[7]);
      gFt[1] += gJ * (Ft[5] * Ft[6] - Ft[3] * Ft[8]);
      gFt[2] += gJ * (Ft[3] * Ft[7] - Ft[4] * Ft[6]);
      gFt[3] += gJ * (Ft[2] * Ft[7] - Ft[1] * Ft[8]);
      gFt[4] += gJ * (Ft[0] * Ft[8] - Ft[2] * Ft[6]);
      gFt[5] += gJ * (Ft[1] * Ft[6] - Ft[0] * Ft[7]);
      gFt[6] += gJ * (Ft[1] * Ft[5] - Ft[2] * Ft[4]);
      gFt[7] += gJ * (Ft[2] * Ft[3] - Ft[0] * Ft[5]);
      gFt[8] += gJ * (Ft[0] * Ft[4] - Ft[1] * Ft[3]);
    }
    const float trP = gP[0] + gP[4] + gP[8];
    float gmu = 0.f, glam = 0.f;
    if (plastic) {
      // F_new = U diag(sn) V^T and P = U diag(tau) U^T of (F_tmp, Jp): mpm_adjoint.cuh
      const float* aux = Q.aux + i * 2;
      float gFn[9];
      for (int k = 0; k < 9; ++k) gFn[k] = Q.gF1 ? Q.gF1[i * 9 + k] : 0.f;
      float gJ = 0.f;
      plastic_adjoint<float>(diff_plastic_law(kind), U, sig, V, Q.Jp[i], mu, lam, aux[0],
                             (kind == DIFF_SAND || kind == DIFF_EP_VON_MISES) ? 0.f : aux[1], S.eps, gFn, gP,
                             Q.gJp1 ? Q.gJp1[i] : 0.f, gFt, gJ, gmu, glam);
      if (Q.gJp) Q.gJp[i] = gJ;
    } else if (neo) {
      // P = mu F F^T + (lam log J - mu) I
      float FFt[9];
      mat_mul_bt(Ft, Ft, FFt);
      gmu = 0.f;
      for (int k = 0; k < 9; ++k) gmu += gP[k] * FFt[k];
      gmu -= trP;
      glam = trP * logf(J);
      // d/dF <gP, mu F F^T> = mu (gP + gP^T) F
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
          float s = 0.f;
          for (int k = 0; k < 3; ++k) s += (gP[r * 3 + k] + gP[k * 3 + r]) * Ft[k * 3 + c];
          gFt[r * 3 + c] += mu * s;
        }
      // d log J / dF = F^{-T} = cof(F) / J
      float cof[9];
      cof[0] = Ft[4] * Ft[8] - Ft[5] * Ft[7];
      cof[1] = Ft[5] * Ft[6] - Ft[3] * Ft[8];
      cof[2] = Ft[3] * Ft[7] - Ft[4] * Ft[6];
      cof[3] = Ft[2] * Ft[7] - Ft[1] * Ft[8];
      cof[4] = Ft[0] * Ft[8] - Ft[2] * Ft[6];
      cof[5] = Ft[1] * Ft[6] - Ft[0] * Ft[7];
      cof[6] = Ft[1] * Ft[5] - Ft[2] * Ft[4];
      cof[7] = Ft[2] * Ft[3] - Ft[0] * Ft[5];
      cof[8] = Ft[0] * Ft[4] - Ft[1] * Ft[3];
      for (int k = 0; k < 9; ++k) gFt[k] += lam * trP * cof[k] / J;
    } else {
      // P = 2 mu (F - R) F^T + lam J (J - 1) I (corotated elastic; liquid.py:42-49 with F = F_tmp)
      float R[9], D[9], DFt[9];
      mat_mul_bt(U, V, R);
      for (int k = 0; k < 9; ++k) D[k] = Ft[k] - R[k];
      mat_mul_bt(D, Ft, DFt);
      gmu = 0.f;
      for (int k = 0; k < 9; ++k) gmu += 2.f * gP[k] * DFt[k];
      glam = trP * J * (J - 1.f);
      // direct terms: 2 mu gP F + 2 mu gP^T (F - R)
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
          float s1 = 0.f, s2 = 0.f;
          for (int k = 0; k < 3; ++k) {
            s1 += gP[r * 3 + k] * Ft[k * 3 + c];
            s2 += gP[k * 3 + r] * D[k * 3 + c];
          }
          gFt[r * 3 + c] += 2.f * mu * (s1 + s2);
        }
      // rotation term: Rbar = -2 mu gP F
      float Rb[9];
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
          float s = 0.f;
          for (int k = 0; k < 3; ++k) s += gP[r * 3 + k] * Ft[k * 3 + c];
          Rb[r * 3 + c] = -2.f * mu * s;
        }
      polar_rotation_adj(U, sig, V, Rb, gFt);
      // J term: lam (2J - 1) tr(gP) dJ,  dJ/dF = cof(F)
      float cof[9];
      cof[0] = Ft[4] * Ft[8] - Ft[5] * Ft[7];
      cof[1] = Ft[5] * Ft[6] - Ft[3] * Ft[8];
      cof[2] = Ft[3] * Ft[7] - Ft[4] * Ft[6];
      cof[3] = Ft[2] * Ft[7] - Ft[1] * Ft[8];
      cof[4] = Ft[0] * Ft[8] - Ft[2] * Ft[6];
      cof[5] = Ft[1] * Ft[6] - Ft[0] * Ft[7];
      cof[6] = Ft[1] * Ft[5] - Ft[2] * Ft[4];
      cof[7] = Ft[2] * Ft[3] - Ft[0] * Ft[5];
      cof[8] = Ft[0] * Ft[4] - Ft[1] * Ft[3];
      for (int k = 0; k < 9; ++k) gFt[k] += lam * (2.f * J - 1.f) * trP * cof[k];
    }
    if (diff_muscle(kind) && Q.actu) {
      // P += k a w w^T, w = F_tmp m: dL/dF_tmp += k a (gP + gP^T) w m^T, dL/da += k w^T gP w
      const float* m = Q.mdir + i * 3;
      const float k = Q.aux[i * 2], a = Q.actu[i];
      float w[3], y[3];
      for (int r = 0; r < 3; ++r) w[r] = Ft[r * 3 + 0] * m[0] + Ft[r * 3 + 1] * m[1] + Ft[r * 3 + 2] * m[2];
      float ga = 0.f;
      for (int r = 0; r < 3; ++r) {
        y[r] = 0.f;
        for (int c = 0; c < 3; ++c) {
          y[r] += (gP[r * 3 + c] + gP[c * 3 + r]) * w[c];
          ga += w[r] * gP[r * 3 + c] * w[c];
        }
      }
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) gFt[r * 3 + c] += k * a * y[r] * m[c];
      if (Q.g_actu) Q.g_actu[i] += k * ga;
    }
    if (!plastic && Q.gJp) Q.gJp[i] = Q.gJp1 ? Q.gJp1[i] : 0.f;  // Jp passes through unchanged
    // F_tmp = (I + dt C) F
    float Am[9];
    for (int k = 0; k < 9; ++k) Am[k] = ((k % 4 == 0) ? 1.f : 0.f) + S.dt * C[k];
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) {
        float sF = 0.f, sC = 0.f;
        for (int k = 0; k < 3; ++k) {
          sF += Am[k * 3 + r] * gFt[k * 3 + c];  // (I + dt C)^T gFt
          sC += gFt[r * 3 + k] * F[c * 3 + k];   // gFt F^T
        }
        Q.gF[i * 9 + r * 3 + c] = sF;
        gC[r * 3 + c] += S.dt * sC;
      }
    for (int d = 0; d < 3; ++d) {
      Q.gv[i * 3 + d] = gv[d];
      Q.gx[i * 3 + d] = gx[d];
    }
    for (int k = 0; k < 9; ++k) Q.gC[i * 9 + k] = gC[k];
    Q.gmu[i] += gmu;
    Q.glam[i] += glam;
  }
}

}  // namespace
}  // namespace gbmpm

using namespace gbmpm;

namespace {

const DiffFields kNoFields{};
const DiffColliders kNoColliders{};

// Per-particle inputs of a call: Muscle actuation (null: no actuation stress) and particle
// constraints (null: none)
struct DiffMuscle {
  const float* actu;
  const float* mdir;
  float* g_actu;
  const float* con_k;
  const float* con_t;
  const uint8_t* active;
};

// The fields of substep k of a sequence that starts at the fields' substep counter ff->step.
const DiffFields* fields_at(const DiffFields* ff, int32_t k, DiffFields& tmp) {
  if (!ff) return nullptr;
  tmp = *ff;
  tmp.step = ff->step + (unsigned long long)k;
  return &tmp;
}

// One forward substep; mass_pp / kind_pp (per particle) override rho / neohookean when given.
int diff_forward(const mpm_scene_config* scene, double rho, int32_t neohookean, const float* mass_pp,
                 const int32_t* kind_pp, const float* aux, int64_t n, const float* x, const float* v, const float* C,
                 const float* F, const float* Jp, const float* mu, const float* lam, float* x1, float* v1, float* C1,
                 float* F1, float* Jp1, void* grid_pm, void* grid_v, uint32_t* status, void* stream, int n_tools = 0,
                 const DiffToolDev* tools = nullptr, const float* tool_f = nullptr, float* tool_f1 = nullptr,
                 const DiffFields* ff = nullptr, const DiffMuscle* mus = nullptr,
                 const DiffColliders* cc = nullptr, int phase = -1, int stage = 0) {
  if (!scene || n < 0 || !grid_pm || !grid_v || !status) return MPM_ERR_BAD_ARG;
  DiffParams Q;
  std::memset(&Q, 0, sizeof(Q));
  std::string err;
  if (derive_scene(*scene, Q.S, err)) return MPM_ERR_BAD_ARG;
  const double pvol = scene->particle_size * scene->particle_size * scene->particle_size * 1e3;
  Q.mass = (float)pvol * (float)rho;
  Q.neohookean = neohookean;
  Q.pmass = mass_pp;
  Q.pkind = kind_pp;
  Q.aux = aux;
  Q.n = n;
  Q.x = x, Q.v = v, Q.C = C, Q.F = F, Q.mu = mu, Q.lam = lam;
  Q.x1 = x1, Q.v1 = v1, Q.C1 = C1, Q.F1 = F1;
  Q.Jp = Jp, Q.Jp1 = Jp1;
  Q.pm = (float4*)grid_pm;
  Q.gvel = (float4*)grid_v;
  Q.status = status;
  Q.n_tools = n_tools;
  for (int t = 0; t < n_tools; ++t) Q.tools[t] = tools[t];
  Q.tool_f = tool_f;
  Q.tool_f1 = tool_f1;
  if (mus && mus->actu && mus->mdir) Q.actu = mus->actu, Q.mdir = mus->mdir;
  if (mus && mus->con_k && mus->con_t) Q.con_k = mus->con_k, Q.con_t = mus->con_t;
  if (mus) Q.active = mus->active;
  const int64_t nodes = (int64_t)Q.S.res[0] * Q.S.res[1] * Q.S.res[2];
  cudaStream_t s = (cudaStream_t)stream;
  const int gb = (int)((nodes + 255) / 256 < 8192 ? (nodes + 255) / 256 : 8192);
  const int pb = (int)((n + 255) / 256 < 8192 ? (n + 255) / 256 : 8192);
  // phase -1: the whole substep; else one part of a staged one (0: P2G, 1: grid stage, 2: G2P)
  if (phase < 0 || phase == 0) {
    k_dclear<<<gb, 256, 0, s>>>(Q, nodes, Q.pm);
    if (n > 0) k_dp2g<<<pb, 256, 0, s>>>(Q);
    if (n_tools > 0) k_dtool_advance<<<1, 32, 0, s>>>(Q);
  }
  if (phase < 0 || phase == 1)
    k_dgrid<<<gb, 256, 0, s>>>(Q, nodes, ff ? *ff : kNoFields, cc ? *cc : kNoColliders, phase < 0 ? 0 : stage);
  if ((phase < 0 || phase == 2) && n > 0) k_dg2p<<<pb, 256, 0, s>>>(Q);
  return cudaGetLastError() == cudaSuccess ? MPM_OK : MPM_ERR_CUDA;
}

int diff_backward(const mpm_scene_config* scene, double rho, int32_t neohookean, const float* mass_pp,
                  const int32_t* kind_pp, const float* aux, int64_t n, const float* x, const float* v, const float* C,
                  const float* F, const float* Jp, const float* mu, const float* lam, const float* gx1,
                  const float* gv1, const float* gC1, const float* gF1, const float* gJp1, float* gx, float* gv,
                  float* gC, float* gF, float* gJp, float* gmu, float* glam, void* grid_pm, void* grid_v,
                  void* g_grid_v, void* g_grid_pm, uint32_t* status, void* stream, int n_tools = 0,
                  const DiffToolDev* tools = nullptr, const float* tool_f = nullptr, const float* tool_f1 = nullptr,
                  float* g_tool = nullptr, const DiffFields* ff = nullptr, const DiffMuscle* mus = nullptr,
                  const DiffColliders* cc = nullptr, int phase = -1, int stage = 0, const void* vstage = nullptr) {
  if (!scene || n < 0 || !grid_pm || !grid_v || !g_grid_v || !g_grid_pm) return MPM_ERR_BAD_ARG;
  DiffParams Q;
  std::memset(&Q, 0, sizeof(Q));
  std::string err;
  if (derive_scene(*scene, Q.S, err)) return MPM_ERR_BAD_ARG;
  const double pvol = scene->particle_size * scene->particle_size * scene->particle_size * 1e3;
  Q.mass = (float)pvol * (float)rho;
  Q.neohookean = neohookean;
  Q.pmass = mass_pp;
  Q.pkind = kind_pp;
  Q.aux = aux;
  Q.n = n;
  Q.x = x, Q.v = v, Q.C = C, Q.F = F, Q.mu = mu, Q.lam = lam;
  Q.Jp = Jp;
  Q.gx1 = gx1, Q.gv1 = gv1, Q.gC1 = gC1, Q.gF1 = gF1, Q.gJp1 = gJp1;
  Q.gx = gx, Q.gv = gv, Q.gC = gC, Q.gF = gF, Q.gJp = gJp, Q.gmu = gmu, Q.glam = glam;
  Q.pm = (float4*)grid_pm;
  Q.gvel = (float4*)grid_v;
  Q.g_grid_v = (float4*)g_grid_v;
  Q.g_grid_pm = (float4*)g_grid_pm;
  Q.status = status;
  Q.n_tools = n_tools;
  for (int t = 0; t < n_tools; ++t) Q.tools[t] = tools[t];
  Q.tool_f = tool_f;
  Q.tool_f1 = const_cast<float*>(tool_f1);
  Q.g_tool = g_tool;
  if (mus && mus->actu && mus->mdir) Q.actu = mus->actu, Q.mdir = mus->mdir, Q.g_actu = mus->g_actu;
  if (mus && mus->con_k && mus->con_t) Q.con_k = mus->con_k, Q.con_t = mus->con_t;
  if (mus) Q.active = mus->active;
  const int64_t nodes = (int64_t)Q.S.res[0] * Q.S.res[1] * Q.S.res[2];
  cudaStream_t s = (cudaStream_t)stream;
  const int gb = (int)((nodes + 255) / 256 < 8192 ? (nodes + 255) / 256 : 8192);
  const int pb = (int)((n + 255) / 256 < 8192 ? (n + 255) / 256 : 8192);
  // phase -1: the whole adjoint substep; else one part of a staged one, in reverse order (2: G2P
  // adjoint, 1: a grid stage's adjoint, 0: the tools' chain and the P2G adjoint)
  if (phase < 0 || phase == 2) {
    k_dclear<<<gb, 256, 0, s>>>(Q, nodes, Q.g_grid_v);
    if (n > 0) k_dg2p_adj<<<pb, 256, 0, s>>>(Q);
  }
  if (phase < 0 || phase == 1)
    k_dgrid_adj<<<gb, 256, 0, s>>>(Q, nodes, ff ? *ff : kNoFields, cc ? *cc : kNoColliders, phase < 0 ? 0 : stage,
                                   (const float4*)vstage);
  if (phase < 0 || phase == 0) {
    if (n_tools > 0) k_dtool_adj<<<1, 32, 0, s>>>(Q);
    // 128-thread CTAs: at its ~160 registers three of them fit an SM (12 warps) where one of 256
    // threads does (8 warps)
    if (n > 0) k_dp2g_adj<<<(int)((n + 127) / 128 < 16384 ? (n + 127) / 128 : 16384), 128, 0, s>>>(Q);
  }
  return cudaGetLastError() == cudaSuccess ? MPM_OK : MPM_ERR_CUDA;
}

int diff_forward_seq(const mpm_scene_config* scene, double rho, int32_t neohookean, const float* mass_pp,
                     const int32_t* kind_pp, const float* aux, int64_t n, int32_t n_sub, float* x_seq, float* v_seq,
                     float* C_seq, float* F_seq, float* Jp_seq, int32_t ring, const float* mu, const float* lam,
                     void* grid_pm, void* grid_v, int32_t grids_per_substep, uint32_t* status, void* stream,
                     int n_tools = 0, const DiffToolDev* tools = nullptr, float* tool_seq = nullptr,
                     const DiffFields* ff = nullptr, const DiffMuscle* mus = nullptr,
                     const DiffColliders* cc = nullptr) {
  if (!scene || n < 0 || n_sub < 0 || ring < 2 || !x_seq || !v_seq || !C_seq || !F_seq) return MPM_ERR_BAD_ARG;
  DiffFields tmp;
  SceneDev S;
  std::string err;
  if (derive_scene(*scene, S, err)) return MPM_ERR_BAD_ARG;
  const int64_t nodes = (int64_t)S.res[0] * S.res[1] * S.res[2];
  for (int32_t k = 0; k < n_sub; ++k) {
    const int64_t a = k % ring, b = (k + 1) % ring;
    const int64_t go = grids_per_substep ? (int64_t)k * nodes : 0;
    const int r = diff_forward(scene, rho, neohookean, mass_pp, kind_pp, aux, n, x_seq + a * n * 3,
                               v_seq + a * n * 3, C_seq + a * n * 9, F_seq + a * n * 9, Jp_seq ? Jp_seq + a * n : nullptr,
                               mu, lam, x_seq + b * n * 3, v_seq + b * n * 3, C_seq + b * n * 9, F_seq + b * n * 9,
                               Jp_seq ? Jp_seq + b * n : nullptr, (float4*)grid_pm + go, (float4*)grid_v + go, status,
                               stream, n_tools, tools, tool_seq ? tool_seq + (int64_t)k * n_tools * 13 : nullptr,
                               tool_seq ? tool_seq + (int64_t)(k + 1) * n_tools * 13 : nullptr,
                               fields_at(ff, k, tmp), mus, cc);
    if (r) return r;
  }
  return MPM_OK;
}

// g_seq packs (dx, dv, dC, dF) per buffer (24 n floats), followed by dJp (n) when Jp_seq is given.
int diff_backward_seq(const mpm_scene_config* scene, double rho, int32_t neohookean, const float* mass_pp,
                      const int32_t* kind_pp, const float* aux, int64_t n, int32_t n_sub, const float* x_seq,
                      const float* v_seq, const float* C_seq, const float* F_seq, const float* Jp_seq, const float* mu,
                      const float* lam, float* g_seq, float* gmu, float* glam, void* grid_pm, void* grid_v,
                      void* g_grid_v, void* g_grid_pm, uint32_t* status, void* stream, int n_tools = 0,
                      const DiffToolDev* tools = nullptr, const float* tool_seq = nullptr, float* g_tool = nullptr,
                      const DiffFields* ff = nullptr, const DiffMuscle* mus = nullptr,
                      const DiffColliders* cc = nullptr) {
  if (!scene || n < 0 || n_sub < 0 || !g_seq) return MPM_ERR_BAD_ARG;
  DiffFields tmp;
  if (n_tools > 0) {
    DiffParams Qz;
    std::memset(&Qz, 0, sizeof(Qz));
    Qz.n_tools = n_tools;
    Qz.g_tool = g_tool;
    k_dtool_zero_acc<<<1, 32, 0, (cudaStream_t)stream>>>(Qz);
  }
  SceneDev S;
  std::string err;
  if (derive_scene(*scene, S, err)) return MPM_ERR_BAD_ARG;
  const int64_t nodes = (int64_t)S.res[0] * S.res[1] * S.res[2];
  const int64_t gs = (Jp_seq ? 25 : 24) * n;
  int cur = 0;
  for (int32_t k = n_sub - 1; k >= 0; --k) {
    float* gi = g_seq + cur * gs;
    float* go = g_seq + (1 - cur) * gs;
    const int r = diff_backward(scene, rho, neohookean, mass_pp, kind_pp, aux, n, x_seq + (int64_t)k * n * 3,
                                v_seq + (int64_t)k * n * 3, C_seq + (int64_t)k * n * 9, F_seq + (int64_t)k * n * 9,
                                Jp_seq ? Jp_seq + (int64_t)k * n : nullptr, mu, lam, gi, gi + 3 * n, gi + 6 * n,
                                gi + 15 * n, Jp_seq ? gi + 24 * n : nullptr, go, go + 3 * n, go + 6 * n, go + 15 * n,
                                Jp_seq ? go + 24 * n : nullptr, gmu, glam, (float4*)grid_pm + (int64_t)k * nodes,
                                (float4*)grid_v + (int64_t)k * nodes, g_grid_v, g_grid_pm, status, stream, n_tools,
                                tools, tool_seq ? tool_seq + (int64_t)k * n_tools * 13 : nullptr,
                                tool_seq ? tool_seq + (int64_t)(k + 1) * n_tools * 13 : nullptr, g_tool,
                                fields_at(ff, k, tmp), mus, cc);
    if (r) return r;
    cur = 1 - cur;
  }
  if (cur == 1 && cudaMemcpyAsync(g_seq, g_seq + gs, sizeof(float) * gs, cudaMemcpyDeviceToDevice,
                                  (cudaStream_t)stream) != cudaSuccess)
    return MPM_ERR_CUDA;
  return MPM_OK;
}

// The caller's tool records as the kernels read them (T_mesh_to_sdf rows and the inverse of
// its 3x3 block in float, computed in double).
int diff_tools_dev(const mpm_diff_tool* tools, int32_t n_tools, const void* tool_seq, DiffToolDev* out) {
  if (n_tools < 0 || n_tools > MPM_DIFF_MAX_TOOLS || (n_tools > 0 && (!tools || !tool_seq))) return MPM_ERR_BAD_ARG;
  for (int t = 0; t < n_tools; ++t) {
    const mpm_diff_tool& a = tools[t];
    DiffToolDev& d = out[t];
    if (!a.sdf || a.res[0] < 2 || a.res[1] < 2 || a.res[2] < 2) return MPM_ERR_BAD_ARG;
    d.sdf = a.sdf;
    for (int k = 0; k < 3; ++k) d.res[k] = a.res[k];
    for (int k = 0; k < 12; ++k) d.T[k] = (float)a.T_mesh_to_sdf[k];
    const double* T = a.T_mesh_to_sdf;
    const double det = T[0] * (T[5] * T[10] - T[6] * T[9]) - T[1] * (T[4] * T[10] - T[6] * T[8]) +
                       T[2] * (T[4] * T[9] - T[5] * T[8]);
    if (!(std::fabs(det) > 0)) return MPM_ERR_BAD_ARG;
    const double inv[9] = {(T[5] * T[10] - T[6] * T[9]) / det, (T[2] * T[9] - T[1] * T[10]) / det,
                           (T[1] * T[6] - T[2] * T[5]) / det,  (T[6] * T[8] - T[4] * T[10]) / det,
                           (T[0] * T[10] - T[2] * T[8]) / det, (T[2] * T[4] - T[0] * T[6]) / det,
                           (T[4] * T[9] - T[5] * T[8]) / det,  (T[1] * T[8] - T[0] * T[9]) / det,
                           (T[0] * T[5] - T[1] * T[4]) / det};
    for (int k = 0; k < 9; ++k) d.Rinv[k] = (float)inv[k];
    d.friction = (float)a.friction;
    d.softness = (float)a.softness;
    d.floor_h = (float)a.floor_height;
  }
  return MPM_OK;
}

// The caller's force fields as the differentiable grid kernels take them.
int diff_fields(const mpm_force_field* fields, int32_t n, int32_t scene_index, uint64_t step0, DiffFields& out) {
  if (n < 0 || n > MPM_DIFF_MAX_FORCE_FIELDS || (n > 0 && !fields) || scene_index < 0) return MPM_ERR_BAD_ARG;
  std::memset(&out, 0, sizeof(out));
  out.n = n;
  out.scene = scene_index;
  out.step = (unsigned long long)step0;
  for (int32_t i = 0; i < n; ++i)
    if (!force_field_dev(fields[i], out.f[i])) return MPM_ERR_BAD_ARG;
  return MPM_OK;
}

// The extras of a sequence (tools, force fields, Muscle inputs) as the internal calls take them.
int diff_extras(const mpm_diff_extras* ex, DiffToolDev* td, DiffFields& ff, DiffMuscle& mus, DiffColliders& cc) {
  std::memset(&mus, 0, sizeof(mus));
  std::memset(&cc, 0, sizeof(cc));
  if (!ex) return diff_fields(nullptr, 0, 0, 0, ff);
  int r = diff_tools_dev(ex->tools, ex->n_tools, ex->tool_seq, td);
  if (r) return r;
  if ((r = diff_fields(ex->force_fields, ex->n_force_fields, ex->scene_index, ex->ff_step, ff))) return r;
  if ((ex->actu == nullptr) != (ex->muscle_dir == nullptr)) return MPM_ERR_BAD_ARG;
  mus.actu = ex->actu;
  mus.mdir = ex->muscle_dir;
  mus.g_actu = ex->g_actu;
  if ((ex->constraint_stiffness == nullptr) != (ex->constraint_target == nullptr)) return MPM_ERR_BAD_ARG;
  mus.con_k = ex->constraint_stiffness;
  mus.con_t = ex->constraint_target;
  mus.active = ex->active;
  if (ex->n_colliders < 0 || ex->n_colliders > MPM_DIFF_MAX_COLLIDERS || (ex->n_colliders > 0 && !ex->colliders))
    return MPM_ERR_BAD_ARG;
  cc.n = ex->n_colliders;
  for (int32_t i = 0; i < cc.n; ++i) {
    const mpm_collider& c = ex->colliders[i];
    if (c.type == MPM_COLLIDER_TOOL || c.scene < -1) return MPM_ERR_BAD_ARG;  // tools: the tool records
    if (collider_dev(ex->sdf_ctx, c, cc.c[i])) return MPM_ERR_BAD_ARG;
  }
  return MPM_OK;
}

}  // namespace

extern "C" {

// One differentiable substep of one scene: (x, v, C, F) -> (x1, v1, C1, F1) with per-particle
// Lame parameters (Elastic material, corotated or neo-Hookean), all device arrays in the
// reference layout.  grid_pm and grid_v are caller buffers of res^3 float4 (res from the
// scene), left holding this substep's grid (needed by mpm_diff_backward).
int mpm_diff_forward(const mpm_scene_config* scene, double rho, int32_t neohookean, int64_t n, const float* x,
                     const float* v, const float* C, const float* F, const float* mu, const float* lam, float* x1,
                     float* v1, float* C1, float* F1, void* grid_pm, void* grid_v, uint32_t* status, void* stream) {
  return diff_forward(scene, rho, neohookean, nullptr, nullptr, nullptr, n, x, v, C, F, nullptr, mu, lam, x1, v1, C1,
                      F1, nullptr, grid_pm, grid_v, status, stream);
}

// Adjoint of mpm_diff_forward at state (x, v, C, F): given dL/d(x1, v1, C1, F1) (gF1 may be
// NULL), writes dL/d(x, v, C, F) and adds dL/d(mu, lam).  grid_pm/grid_v must hold the
// forward grid of this substep (call mpm_diff_forward on the same state first); g_grid_v and
// g_grid_pm are res^3 float4 scratch buffers.
int mpm_diff_backward(const mpm_scene_config* scene, double rho, int32_t neohookean, int64_t n, const float* x,
                      const float* v, const float* C, const float* F, const float* mu, const float* lam,
                      const float* gx1, const float* gv1, const float* gC1, const float* gF1, float* gx, float* gv,
                      float* gC, float* gF, float* gmu, float* glam, void* grid_pm, void* grid_v, void* g_grid_v,
                      void* g_grid_pm, uint32_t* status, void* stream) {
  return diff_backward(scene, rho, neohookean, nullptr, nullptr, nullptr, n, x, v, C, F, nullptr, mu, lam, gx1, gv1,
                       gC1, gF1, nullptr, gx, gv, gC, gF, nullptr, gmu, glam, grid_pm, grid_v, g_grid_v, g_grid_pm,
                       status, stream);
}

// n_sub forward substeps in one call (no host round trip per substep).  State k (k = 0..n_sub)
// lives in slot k % ring of x_seq [ring, n, 3], v_seq [ring, n, 3], C_seq [ring, n, 9] and
// F_seq [ring, n, 9]; slot 0 holds the input.  ring = 2 ping-pongs; ring > n_sub keeps every
// state.  With grids_per_substep, substep k leaves its grid in grid_pm + k * nodes and
// grid_v + k * nodes (n_sub grids each); otherwise every substep uses the one grid given.
int mpm_diff_forward_seq(const mpm_scene_config* scene, double rho, int32_t neohookean, int64_t n, int32_t n_sub,
                         float* x_seq, float* v_seq, float* C_seq, float* F_seq, int32_t ring, const float* mu,
                         const float* lam, void* grid_pm, void* grid_v, int32_t grids_per_substep, uint32_t* status,
                         void* stream) {
  return diff_forward_seq(scene, rho, neohookean, nullptr, nullptr, nullptr, n, n_sub, x_seq, v_seq, C_seq, F_seq,
                          nullptr, ring, mu, lam, grid_pm, grid_v, grids_per_substep, status, stream);
}

// Adjoint of n_sub substeps whose states 0..n_sub-1 and grids were kept by mpm_diff_forward_seq
// (ring > n_sub - 1, grids_per_substep).  g_seq [2, 24 n] holds two packed gradient buffers
// (dx [n,3], dv [n,3], dC [n,9], dF [n,9]); buffer 0 holds dL/d(state n_sub) on entry and
// dL/d(state 0) on return.  dL/d(mu, lam) accumulate into gmu, glam.
int mpm_diff_backward_seq(const mpm_scene_config* scene, double rho, int32_t neohookean, int64_t n, int32_t n_sub,
                          const float* x_seq, const float* v_seq, const float* C_seq, const float* F_seq,
                          const float* mu, const float* lam, float* g_seq, float* gmu, float* glam, void* grid_pm,
                          void* grid_v, void* g_grid_v, void* g_grid_pm, uint32_t* status, void* stream) {
  return diff_backward_seq(scene, rho, neohookean, nullptr, nullptr, nullptr, n, n_sub, x_seq, v_seq, C_seq, F_seq,
                           nullptr, mu, lam, g_seq, gmu, glam, grid_pm, grid_v, g_grid_v, g_grid_pm, status, stream);
}

// mpm_diff_forward_seq / mpm_diff_backward_seq for a scene of several entities: the particle
// mass [n], material kind [n] (0 corotated Elastic, 1 neo-Hookean Elastic, 2 Liquid, 3 Sand, 4 Snow)
// and aux [n, 2] (Sand: friction alpha; Snow: clamp bounds 1 - yield_lower, 1 + yield_higher) are given
// per particle, as the reference's differentiable MPM path reads them per particle through
// particles_info and the material dispatch (mpm_solver.py:341-375); the state includes Jp
// (Jp_seq [ring, n]) and g_seq packs dJp after (dx, dv, dC, dF): [2, 25 n].
int mpm_diff_forward_seq_pp(const mpm_scene_config* scene, const float* mass, const int32_t* kind, const float* aux,
                            int64_t n, int32_t n_sub, float* x_seq, float* v_seq, float* C_seq, float* F_seq,
                            float* Jp_seq, int32_t ring, const float* mu, const float* lam, void* grid_pm, void* grid_v,
                            int32_t grids_per_substep, uint32_t* status, void* stream) {
  if (n > 0 && (!mass || !kind || !aux || !Jp_seq)) return MPM_ERR_BAD_ARG;
  return diff_forward_seq(scene, 0.0, 0, mass, kind, aux, n, n_sub, x_seq, v_seq, C_seq, F_seq, Jp_seq, ring, mu, lam,
                          grid_pm, grid_v, grids_per_substep, status, stream);
}

int mpm_diff_backward_seq_pp(const mpm_scene_config* scene, const float* mass, const int32_t* kind, const float* aux,
                             int64_t n, int32_t n_sub, const float* x_seq, const float* v_seq, const float* C_seq,
                             const float* F_seq, const float* Jp_seq, const float* mu, const float* lam, float* g_seq,
                             float* gmu, float* glam, void* grid_pm, void* grid_v, void* g_grid_v, void* g_grid_pm,
                             uint32_t* status, void* stream) {
  if (n > 0 && (!mass || !kind || !aux || !Jp_seq)) return MPM_ERR_BAD_ARG;
  return diff_backward_seq(scene, 0.0, 0, mass, kind, aux, n, n_sub, x_seq, v_seq, C_seq, F_seq, Jp_seq, mu, lam,
                           g_seq, gmu, glam, grid_pm, grid_v, g_grid_v, g_grid_pm, status, stream);
}

int mpm_diff_forward_seq_ex(const mpm_scene_config* scene, const float* mass, const int32_t* kind, const float* aux,
                            int64_t n, int32_t n_sub, float* x_seq, float* v_seq, float* C_seq, float* F_seq,
                            float* Jp_seq, int32_t ring, const float* mu, const float* lam, const mpm_diff_extras* ex,
                            void* grid_pm, void* grid_v, int32_t grids_per_substep, uint32_t* status, void* stream) {
  if (n > 0 && (!mass || !kind || !aux || !Jp_seq)) return MPM_ERR_BAD_ARG;
  DiffToolDev td[MPM_DIFF_MAX_TOOLS];
  DiffFields ff;
  DiffMuscle mus;
  DiffColliders cc;
  const int r = diff_extras(ex, td, ff, mus, cc);
  if (r) return r;
  const int nt = ex ? ex->n_tools : 0;
  return diff_forward_seq(scene, 0.0, 0, mass, kind, aux, n, n_sub, x_seq, v_seq, C_seq, F_seq, Jp_seq, ring, mu, lam,
                          grid_pm, grid_v, grids_per_substep, status, stream, nt, td, ex ? ex->tool_seq : nullptr, &ff,
                          &mus, &cc);
}

int mpm_diff_backward_seq_ex(const mpm_scene_config* scene, const float* mass, const int32_t* kind, const float* aux,
                             int64_t n, int32_t n_sub, const float* x_seq, const float* v_seq, const float* C_seq,
                             const float* F_seq, const float* Jp_seq, const float* mu, const float* lam,
                             const mpm_diff_extras* ex, float* g_seq, float* gmu, float* glam, void* grid_pm,
                             void* grid_v, void* g_grid_v, void* g_grid_pm, uint32_t* status, void* stream) {
  if (n > 0 && (!mass || !kind || !aux || !Jp_seq)) return MPM_ERR_BAD_ARG;
  DiffToolDev td[MPM_DIFF_MAX_TOOLS];
  DiffFields ff;
  DiffMuscle mus;
  DiffColliders cc;
  const int r = diff_extras(ex, td, ff, mus, cc);
  if (r) return r;
  const int nt = ex ? ex->n_tools : 0;
  if (nt > 0 && !ex->g_tool) return MPM_ERR_BAD_ARG;
  return diff_backward_seq(scene, 0.0, 0, mass, kind, aux, n, n_sub, x_seq, v_seq, C_seq, F_seq, Jp_seq, mu, lam,
                           g_seq, gmu, glam, grid_pm, grid_v, g_grid_v, g_grid_pm, status, stream, nt, td,
                           ex ? ex->tool_seq : nullptr, ex ? ex->g_tool : nullptr, &ff, &mus, &cc);
}

// One part of a differentiable substep in stages (a Custom force field acts in the caller between
// grid stages); see gbmpm.h.
int mpm_diff_substep_stage(const mpm_scene_config* scene, const float* mass, const int32_t* kind, const float* aux,
                           int64_t n, const float* x, const float* v, const float* C, const float* F, const float* Jp,
                           const float* mu, const float* lam, const mpm_diff_extras* ex, int32_t phase, int32_t stage,
                           int32_t ff_begin, int32_t ff_end, float* x1, float* v1, float* C1, float* F1, float* Jp1,
                           void* grid_pm, void* grid_v, uint32_t* status, void* stream) {
  if (n > 0 && (!mass || !kind || !aux || !Jp)) return MPM_ERR_BAD_ARG;
  if (phase < 0 || phase > 2 || (phase == 1 && (stage < 1 || stage > 3))) return MPM_ERR_BAD_ARG;
  if (phase == 1 && stage <= 2 && (!ex || ff_begin < 0 || ff_end < ff_begin || ff_end > ex->n_force_fields))
    return MPM_ERR_BAD_ARG;
  DiffToolDev td[MPM_DIFF_MAX_TOOLS];
  DiffFields ff;
  DiffMuscle mus;
  DiffColliders cc;
  int r = diff_extras(ex, td, ff, mus, cc);
  if (r) return r;
  if (phase == 1 && stage <= 2 &&
      (r = diff_fields(ex->force_fields + ff_begin, ff_end - ff_begin, ex->scene_index, ex->ff_step, ff)))
    return r;
  const int nt = ex ? ex->n_tools : 0;
  float* ts = ex ? ex->tool_seq : nullptr;
  return diff_forward(scene, 0.0, 0, mass, kind, aux, n, x, v, C, F, Jp, mu, lam, x1, v1, C1, F1, Jp1, grid_pm,
                      grid_v, status, stream, nt, td, ts, ts ? ts + (int64_t)nt * 13 : nullptr, &ff, &mus, &cc, phase,
                      stage);
}

int mpm_diff_substep_stage_adj(const mpm_scene_config* scene, const float* mass, const int32_t* kind,
                               const float* aux, int64_t n, const float* x, const float* v, const float* C,
                               const float* F, const float* Jp, const float* mu, const float* lam,
                               const mpm_diff_extras* ex, int32_t phase, int32_t stage, int32_t ff_begin,
                               int32_t ff_end, const void* vstage, const float* gx1, const float* gv1,
                               const float* gC1, const float* gF1, const float* gJp1, float* gx, float* gv, float* gC,
                               float* gF, float* gJp, float* gmu, float* glam, void* grid_pm, void* grid_v,
                               void* g_grid_v, void* g_grid_pm, uint32_t* status, void* stream) {
  if (n > 0 && (!mass || !kind || !aux || !Jp)) return MPM_ERR_BAD_ARG;
  if (phase < 0 || phase > 2 || (phase == 1 && (stage < 1 || stage > 3)) || (phase == 1 && stage >= 2 && !vstage))
    return MPM_ERR_BAD_ARG;
  if (phase == 1 && stage <= 2 && (!ex || ff_begin < 0 || ff_end < ff_begin || ff_end > ex->n_force_fields))
    return MPM_ERR_BAD_ARG;
  DiffToolDev td[MPM_DIFF_MAX_TOOLS];
  DiffFields ff;
  DiffMuscle mus;
  DiffColliders cc;
  int r = diff_extras(ex, td, ff, mus, cc);
  if (r) return r;
  if (phase == 1 && stage <= 2 &&
      (r = diff_fields(ex->force_fields + ff_begin, ff_end - ff_begin, ex->scene_index, ex->ff_step, ff)))
    return r;
  const int nt = ex ? ex->n_tools : 0;
  if (nt > 0 && !ex->g_tool) return MPM_ERR_BAD_ARG;
  const float* ts = ex ? ex->tool_seq : nullptr;
  return diff_backward(scene, 0.0, 0, mass, kind, aux, n, x, v, C, F, Jp, mu, lam, gx1, gv1, gC1, gF1, gJp1, gx, gv,
                       gC, gF, gJp, gmu, glam, grid_pm, grid_v, g_grid_v, g_grid_pm, status, stream, nt, td, ts,
                       ts ? ts + (int64_t)nt * 13 : nullptr, ex ? ex->g_tool : nullptr, &ff, &mus, &cc, phase, stage,
                       vstage);
}

int mpm_diff_forward_seq_tools(const mpm_scene_config* scene, const float* mass, const int32_t* kind, const float* aux,
                               int64_t n, int32_t n_sub, float* x_seq, float* v_seq, float* C_seq, float* F_seq,
                               float* Jp_seq, int32_t ring, const float* mu, const float* lam,
                               const mpm_diff_tool* tools, int32_t n_tools, float* tool_seq, void* grid_pm,
                               void* grid_v, int32_t grids_per_substep, uint32_t* status, void* stream) {
  mpm_diff_extras ex;
  std::memset(&ex, 0, sizeof(ex));
  ex.tools = tools;
  ex.n_tools = n_tools;
  ex.tool_seq = tool_seq;
  return mpm_diff_forward_seq_ex(scene, mass, kind, aux, n, n_sub, x_seq, v_seq, C_seq, F_seq, Jp_seq, ring, mu, lam,
                                 &ex, grid_pm, grid_v, grids_per_substep, status, stream);
}

int mpm_diff_backward_seq_tools(const mpm_scene_config* scene, const float* mass, const int32_t* kind, const float* aux,
                                int64_t n, int32_t n_sub, const float* x_seq, const float* v_seq, const float* C_seq,
                                const float* F_seq, const float* Jp_seq, const float* mu, const float* lam,
                                const mpm_diff_tool* tools, int32_t n_tools, const float* tool_seq, float* g_tool,
                                float* g_seq, float* gmu, float* glam, void* grid_pm, void* grid_v, void* g_grid_v,
                                void* g_grid_pm, uint32_t* status, void* stream) {
  mpm_diff_extras ex;
  std::memset(&ex, 0, sizeof(ex));
  ex.tools = tools;
  ex.n_tools = n_tools;
  ex.tool_seq = const_cast<float*>(tool_seq);
  ex.g_tool = g_tool;
  return mpm_diff_backward_seq_ex(scene, mass, kind, aux, n, n_sub, x_seq, v_seq, C_seq, F_seq, Jp_seq, mu, lam, &ex,
                                  g_seq, gmu, glam, grid_pm, grid_v, g_grid_v, g_grid_pm, status, stream);
}

}  // extern "C"
