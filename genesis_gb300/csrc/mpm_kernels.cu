// mpm_kernels.cu - sm_103a kernels of the MLS-MPM substep (P2G, grid op, G2P) and of the
// per-substep particle re-sort, plus the state I/O kernels.
//
// One substep = k_p2g -> k_grid_op -> k_g2p<true> -> k_scan_reduce -> k_scan_partials ->
// k_scan_apply -> k_perm.  Reference semantics: genesis/engine/solvers/mpm_solver.py
// (p2g :322-421, g2p :423-481) and genesis/engine/couplers/legacy_coupler.py
// (mpm_grid_op :356-501); see each kernel.
#include "mpm_kernels.cuh"

namespace gbmpm {

namespace {

__device__ __forceinline__ uint32_t ld_info(const float* base, int64_t cap, int64_t i) {
  return __float_as_uint(base[(int64_t)PF_INFO * cap + i]);
}

__device__ __forceinline__ int64_t grid_stride_begin() { return (int64_t)blockIdx.x * blockDim.x + threadIdx.x; }
__device__ __forceinline__ int64_t grid_stride_step() { return (int64_t)gridDim.x * blockDim.x; }

// Scene of a particle, through its material.
__device__ __forceinline__ int32_t scene_of(const KParams& P, uint32_t info) {
  return P.mats[info & INFO_MAT_MASK].scene;
}

// Output row of a particle in the reference [B, N] layout of scenes [s0, s1).
__device__ __forceinline__ int64_t out_row(const KParams& P, int32_t s, int64_t s0, uint32_t pid) {
  return P.scenes[s].p_begin - P.scenes[s0].p_begin + (int64_t)pid;
}

__device__ __forceinline__ void write_defaults(float* D, int64_t cap, int64_t i, int nf, float default_jp) {
#pragma unroll
  for (int k = 0; k < 6; ++k) D[(int64_t)k * cap + i] = 0.f;
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    D[(int64_t)(PF_C + k) * cap + i] = 0.f;
    D[(int64_t)(PF_F + k) * cap + i] = (k % 4 == 0) ? 1.f : 0.f;
  }
  D[(int64_t)PF_JP * cap + i] = default_jp;
  if (nf > NF_BASE) {
    D[(int64_t)PF_ACTU * cap + i] = 0.f;
    D[(int64_t)(PF_MDIR + 0) * cap + i] = 0.f;
    D[(int64_t)(PF_MDIR + 1) * cap + i] = 0.f;
    D[(int64_t)(PF_MDIR + 2) * cap + i] = 1.f;
  }
}

// FP64 re-solve for the rare particle whose FP32 factor fails its residual check; kept out
// of line so its registers do not weigh on the P2G kernel.
__device__ __noinline__ void svd3_fp64(const float* Ft, float* U, float* sig, float* V) {
  double Ad[9], Ud[9], sd[3], Vd[9];
  for (int k = 0; k < 9; ++k) Ad[k] = Ft[k];
  svd3<double, 8>(Ad, Ud, sd, Vd);
  for (int k = 0; k < 9; ++k) {
    U[k] = (float)Ud[k];
    V[k] = (float)Vd[k];
  }
  for (int k = 0; k < 3; ++k) sig[k] = (float)sd[k];
}

}  // namespace

// ------------------------------------------------------------------ state set-up and I/O
__global__ void k_init_particles(KParams P, const int64_t* scene_pbegin, const int32_t* scene_first_mat,
                                 int64_t n_scenes) {
  for (int64_t i = grid_stride_begin(); i < P.n; i += grid_stride_step()) {
    int64_t lo = 0, hi = n_scenes - 1;  // last scene with p_begin <= i
    while (lo < hi) {
      int64_t mid = (lo + hi + 1) >> 1;
      if (scene_pbegin[mid] <= i) lo = mid; else hi = mid - 1;
    }
    const int32_t mat = scene_first_mat[lo];
    write_defaults(P.dst, P.cap, i, P.nf, P.mats[mat].default_Jp);
    P.dst[(int64_t)PF_INFO * P.cap + i] = __uint_as_float((uint32_t)mat | INFO_FREE);
    P.dst[(int64_t)PF_PID * P.cap + i] = __uint_as_float((uint32_t)(i - scene_pbegin[lo]));
  }
}

// mpm_solver.py:806-838 (_kernel_add_particles)
__global__ void k_add_particles(KParams P, int64_t s0, int64_t s1, int64_t start, int64_t n_add, int32_t mat_local,
                                int32_t active, const float* pos) {
  float* D = P.dst;
  for (int64_t i = grid_stride_begin(); i < P.n; i += grid_stride_step()) {
    const uint32_t info = ld_info(D, P.cap, i);
    if (info & INFO_DEAD) continue;
    const int32_t s = scene_of(P, info);
    if (s < s0 || s >= s1) continue;
    const int64_t pid = (int64_t)__float_as_uint(D[(int64_t)PF_PID * P.cap + i]);
    if (pid < start || pid >= start + n_add) continue;
    const int64_t j = pid - start;
    const uint32_t gmat = (uint32_t)(P.scenes[s].mat_begin + mat_local);
    write_defaults(D, P.cap, i, P.nf, P.mats[gmat].default_Jp);
#pragma unroll
    for (int d = 0; d < 3; ++d) D[(int64_t)(PF_POS + d) * P.cap + i] = pos[j * 3 + d];
    D[(int64_t)PF_INFO * P.cap + i] = __uint_as_float(gmat | INFO_FREE | (active ? INFO_ACTIVE : 0u));
  }
}

// mpm_solver.py:759-778 (_kernel_get_state)
__global__ void k_get_state(KParams P, int64_t s0, int64_t s1, float* pos, float* vel, float* C, float* F,
                            float* Jp, uint8_t* active) {
  const float* D = P.dst;
  for (int64_t i = grid_stride_begin(); i < P.n; i += grid_stride_step()) {
    const uint32_t info = ld_info(D, P.cap, i);
    if (info & INFO_DEAD) continue;
    const int32_t s = scene_of(P, info);
    if (s < s0 || s >= s1) continue;
    const int64_t r = out_row(P, s, s0, __float_as_uint(D[(int64_t)PF_PID * P.cap + i]));
    if (pos)
      for (int d = 0; d < 3; ++d) pos[r * 3 + d] = D[(int64_t)(PF_POS + d) * P.cap + i];
    if (vel)
      for (int d = 0; d < 3; ++d) vel[r * 3 + d] = D[(int64_t)(PF_VEL + d) * P.cap + i];
    if (C)
      for (int d = 0; d < 9; ++d) C[r * 9 + d] = D[(int64_t)(PF_C + d) * P.cap + i];
    if (F)
      for (int d = 0; d < 9; ++d) F[r * 9 + d] = D[(int64_t)(PF_F + d) * P.cap + i];
    if (Jp) Jp[r] = D[(int64_t)PF_JP * P.cap + i];
    if (active) active[r] = (info & INFO_ACTIVE) ? 1 : 0;
  }
}

// mpm_solver.py:729-749 (_kernel_set_state)
__global__ void k_set_state(KParams P, int64_t s0, int64_t s1, const float* pos, const float* vel, const float* C,
                            const float* F, const float* Jp, const uint8_t* active) {
  float* D = P.dst;
  for (int64_t i = grid_stride_begin(); i < P.n; i += grid_stride_step()) {
    const uint32_t info = ld_info(D, P.cap, i);
    if (info & INFO_DEAD) continue;
    const int32_t s = scene_of(P, info);
    if (s < s0 || s >= s1) continue;
    const int64_t r = out_row(P, s, s0, __float_as_uint(D[(int64_t)PF_PID * P.cap + i]));
    if (pos)
      for (int d = 0; d < 3; ++d) D[(int64_t)(PF_POS + d) * P.cap + i] = pos[r * 3 + d];
    if (vel)
      for (int d = 0; d < 3; ++d) D[(int64_t)(PF_VEL + d) * P.cap + i] = vel[r * 3 + d];
    if (C)
      for (int d = 0; d < 9; ++d) D[(int64_t)(PF_C + d) * P.cap + i] = C[r * 9 + d];
    if (F)
      for (int d = 0; d < 9; ++d) D[(int64_t)(PF_F + d) * P.cap + i] = F[r * 9 + d];
    if (Jp) D[(int64_t)PF_JP * P.cap + i] = Jp[r];
    if (active) {
      const uint32_t ni = active[r] ? (info | INFO_ACTIVE) : (info & ~INFO_ACTIVE);
      D[(int64_t)PF_INFO * P.cap + i] = __uint_as_float(ni);
    }
  }
}

// Per-field access to a contiguous per-scene particle range (mpm_solver.py:840-1026).
__global__ void k_particles_field(KParams P, int field, int write, int64_t s0, int64_t s1, int64_t start,
                                  int64_t n_sel, float* data) {
  float* D = P.dst;
  for (int64_t i = grid_stride_begin(); i < P.n; i += grid_stride_step()) {
    const uint32_t info = ld_info(D, P.cap, i);
    if (info & INFO_DEAD) continue;
    const int32_t s = scene_of(P, info);
    if (s < s0 || s >= s1) continue;
    const int64_t pid = (int64_t)__float_as_uint(D[(int64_t)PF_PID * P.cap + i]);
    if (pid < start || pid >= start + n_sel) continue;
    const int64_t r = (int64_t)(s - s0) * n_sel + (pid - start);
    int base = -1, width = 0;
    switch (field) {
      case 0: base = PF_POS; width = 3; break;
      case 1: base = PF_VEL; width = 3; break;
      case 2: base = PF_C; width = 9; break;
      case 3: base = PF_F; width = 9; break;
      case 4: base = PF_JP; width = 1; break;
      case 6: base = (P.nf > NF_BASE) ? PF_ACTU : -1; width = 1; break;
      case 8: base = (P.nf > NF_BASE) ? PF_MDIR : -1; width = 3; break;
      default: break;
    }
    if (field == 5 || field == 7) {  // active / free flags
      const uint32_t bit = field == 5 ? INFO_ACTIVE : INFO_FREE;
      if (write) {
        const uint32_t ni = data[r] != 0.f ? (info | bit) : (info & ~bit);
        D[(int64_t)PF_INFO * P.cap + i] = __uint_as_float(ni);
      } else {
        data[r] = (info & bit) ? 1.f : 0.f;
      }
    } else if (field == 9) {  // set position and reset v, F, C, Jp (mpm_solver.py:840-859)
      if (write) {
        write_defaults(D, P.cap, i, NF_BASE, P.mats[info & INFO_MAT_MASK].default_Jp);
        for (int d = 0; d < 3; ++d) D[(int64_t)(PF_POS + d) * P.cap + i] = data[r * 3 + d];
      }
    } else if (base >= 0) {
      for (int d = 0; d < width; ++d) {
        if (write) D[(int64_t)(base + d) * P.cap + i] = data[r * width + d];
        else data[r * width + d] = D[(int64_t)(base + d) * P.cap + i];
      }
    }
  }
}

// ------------------------------------------------------------------ G2P (+ re-keying)
// mpm_solver.py:423-481 (g2p) with the particle boundary of boundaries.py:22-32, followed by
// the bucket key of the new position and a warp-aggregated rank within the bucket.
// UPDATE=false only computes keys (after a state change).
template <bool UPDATE>
__device__ __forceinline__ void g2p_body(const KParams& P) {
  if (UPDATE && blockIdx.x == 0 && threadIdx.x == 0) *P.nlist_other = 0;
  float* D = P.dst;
  const int64_t cap = P.cap;
  const int lane = threadIdx.x & 31;
  const int64_t warp0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int32_t kInactive = (int32_t)P.K, kDead = (int32_t)P.K + 1;
  for (int64_t base = warp0 * 32; base < P.n; base += nwarps * 32) {
    const int64_t i = base + lane;
    const bool valid = i < P.n;
    int32_t key = kInactive;
    if (valid) {
      const uint32_t info = ld_info(D, cap, i);
      if (info & INFO_DEAD) {
        key = kDead;
      } else if (info & INFO_ACTIVE) {
        const SceneDev& S = P.scenes[scene_of(P, info)];
        float x[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) x[d] = D[(int64_t)(PF_POS + d) * cap + i];
        int b[3];
        const bool ok = stencil_origin(S, x, b);
        if (!ok) {
          atomicOr(P.status, (isfinite(x[0]) && isfinite(x[1]) && isfinite(x[2])) ? 2u : 1u);
        } else if (!UPDATE) {
          key = (int32_t)block_of(S, b[0], b[1], b[2]);
        } else {
          float fx[3], w[3][3];
#pragma unroll
          for (int d = 0; d < 3; ++d) {
            const float t = __fmul_rn(x[d], S.inv_dx);
            fx[d] = t - (float)(b[d] + S.offset[d]);
            bspline_w(fx[d], w[d]);
          }
          // per-axis address terms of the 3 stencil nodes
          int64_t ax[3];
          int ay[3], az[3];
#pragma unroll
          for (int o = 0; o < 3; ++o) {
            const int gx = b[0] + o, gy = b[1] + o, gz = b[2] + o;
            ax[o] = (S.block_base + (int64_t)(gx >> 2) * S.bres[1] * S.bres[2]) * BLK_NODES + (gx & 3) * 16;
            ay[o] = (gy >> 2) * S.bres[2] * BLK_NODES + (gy & 3) * 4;
            az[o] = (gz >> 2) * BLK_NODES + (gz & 3);
          }
          float v[3] = {0.f, 0.f, 0.f};
          float Cn[9];
#pragma unroll
          for (int k = 0; k < 9; ++k) Cn[k] = 0.f;
#pragma unroll
          for (int ox = 0; ox < 3; ++ox)
#pragma unroll
            for (int oy = 0; oy < 3; ++oy)
#pragma unroll
              for (int oz = 0; oz < 3; ++oz) {
                const float4 g = __ldg(&P.grid[ax[ox] + ay[oy] + az[oz]]);
                const float wt = w[0][ox] * w[1][oy] * w[2][oz];
                const float dp[3] = {(float)ox - fx[0], (float)oy - fx[1], (float)oz - fx[2]};
                const float gv[3] = {g.x, g.y, g.z};
#pragma unroll
                for (int r = 0; r < 3; ++r) {
                  v[r] += wt * gv[r];
                  const float s = 4.f * S.inv_dx * wt * gv[r];
#pragma unroll
                  for (int c = 0; c < 3; ++c) Cn[r * 3 + c] += s * dp[c];
                }
              }
          float xn[3];
          bool finite = true;
#pragma unroll
          for (int d = 0; d < 3; ++d) {
            xn[d] = x[d] + S.dt * v[d];
            finite = finite && isfinite(xn[d]) && isfinite(v[d]);
          }
          // CubeBoundary.impose_pos_vel (boundaries.py:22-32)
#pragma unroll
          for (int d = 0; d < 3; ++d) {
            if (xn[d] >= S.hi[d] && v[d] >= 0.f) v[d] *= -S.restitution;
            else if (xn[d] <= S.lo[d] && v[d] <= 0.f) v[d] *= -S.restitution;
            xn[d] = fmaxf(fminf(xn[d], S.hi[d]), S.lo[d]);
          }
#pragma unroll
          for (int d = 0; d < 3; ++d) {
            D[(int64_t)(PF_POS + d) * cap + i] = xn[d];
            D[(int64_t)(PF_VEL + d) * cap + i] = v[d];
          }
#pragma unroll
          for (int k = 0; k < 9; ++k) D[(int64_t)(PF_C + k) * cap + i] = Cn[k];
          if (!finite) {
            atomicOr(P.status, 1u);
          } else if (stencil_origin(S, xn, b)) {
            key = (int32_t)block_of(S, b[0], b[1], b[2]);
          } else {
            atomicOr(P.status, 2u);
          }
        }
      }
    }
    // warp-aggregated rank within the bucket
    const unsigned am = __ballot_sync(0xffffffffu, valid);
    if (valid) {
      const unsigned peers = __match_any_sync(am, key);
      const int leader = __ffs(peers) - 1;
      int r = 0;
      if (lane == leader) r = atomicAdd(&P.count[key], __popc(peers));
      r = __shfl_sync(peers, r, leader);
      r += __popc(peers & ((1u << lane) - 1u));
      P.key[i] = key;
      P.rank[i] = r;
    }
  }
}
__global__ void __launch_bounds__(256) k_g2p(KParams P) { g2p_body<true>(P); }
__global__ void __launch_bounds__(256) k_keys(KParams P) { g2p_body<false>(P); }

// ------------------------------------------------------------------ counting-sort scan
namespace {
__device__ __forceinline__ int items_of(int c, int chunk) { return (c + chunk - 1) / chunk; }

// Exclusive scan of (a, b) pairs over the CTA (blockDim.x == SCAN_THREADS); returns totals.
__device__ __forceinline__ int2 block_exclusive_scan2(int a, int b, int2& total) {
  __shared__ int2 warp_sums[SCAN_THREADS / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int ia = a, ib = b;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int ta = __shfl_up_sync(0xffffffffu, ia, o), tb = __shfl_up_sync(0xffffffffu, ib, o);
    if (lane >= o) {
      ia += ta;
      ib += tb;
    }
  }
  if (lane == 31) warp_sums[wid] = make_int2(ia, ib);
  __syncthreads();
  if (wid == 0) {
    int2 ws = lane < SCAN_THREADS / 32 ? warp_sums[lane] : make_int2(0, 0);
    int sa = ws.x, sb = ws.y;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int ta = __shfl_up_sync(0xffffffffu, sa, o), tb = __shfl_up_sync(0xffffffffu, sb, o);
      if (lane >= o) {
        sa += ta;
        sb += tb;
      }
    }
    if (lane < SCAN_THREADS / 32) warp_sums[lane] = make_int2(sa - ws.x, sb - ws.y);
  }
  __syncthreads();
  const int2 wo = warp_sums[wid];
  // totals: last thread's inclusive value + its warp offset
  __shared__ int2 s_total;
  if (threadIdx.x == SCAN_THREADS - 1) s_total = make_int2(wo.x + ia, wo.y + ib);
  __syncthreads();
  total = s_total;
  return make_int2(wo.x + ia - a, wo.y + ib - b);
}
}  // namespace

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_reduce(KParams P) {
  const int64_t nb = P.K + 2;
  const int64_t t0 = (int64_t)blockIdx.x * SCAN_TILE;
  int cs = 0, is = 0;
  for (int64_t k = t0 + threadIdx.x; k < t0 + SCAN_TILE && k < nb; k += blockDim.x) {
    const int c = P.count[k];
    cs += c;
    if (k <= P.K) is += items_of(c, P.chunk);
  }
  int2 total;
  block_exclusive_scan2(cs, is, total);
  if (threadIdx.x == 0) P.partials[blockIdx.x] = total;
}

// One CTA: exclusive scan of the tile partials in place; writes the P2G item count.
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_partials(KParams P, int n_tiles) {
  int2 carry = make_int2(0, 0);
  for (int t0 = 0; t0 < n_tiles; t0 += SCAN_THREADS) {
    const int t = t0 + threadIdx.x;
    const int2 v = t < n_tiles ? P.partials[t] : make_int2(0, 0);
    int2 total;
    const int2 ex = block_exclusive_scan2(v.x, v.y, total);
    if (t < n_tiles) P.partials[t] = make_int2(carry.x + ex.x, carry.y + ex.y);
    carry.x += total.x;
    carry.y += total.y;
    __syncthreads();
  }
  if (threadIdx.x == 0) *P.n_items = carry.y;
}

// Bucket offsets, P2G work items, and count reset for the next histogram.
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_apply(KParams P) {
  constexpr int PER = SCAN_TILE / SCAN_THREADS;
  const int64_t nb = P.K + 2;
  const int64_t k0 = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)threadIdx.x * PER;
  int c[PER];
  int cs = 0, is = 0;
#pragma unroll
  for (int j = 0; j < PER; ++j) {
    const int64_t k = k0 + j;
    c[j] = k < nb ? P.count[k] : 0;
    cs += c[j];
    if (k <= P.K) is += items_of(c[j], P.chunk);
  }
  int2 total;
  const int2 ex = block_exclusive_scan2(cs, is, total);
  const int2 base = P.partials[blockIdx.x];
  int off = base.x + ex.x, it = base.y + ex.y;
#pragma unroll
  for (int j = 0; j < PER; ++j) {
    const int64_t k = k0 + j;
    if (k >= nb) break;
    P.offset[k] = off;
    if (k <= P.K) {
      for (int s = 0; s < c[j]; s += P.chunk) {
        const int e = min(s + P.chunk, c[j]);
        P.items[it++] = make_int4((int)k, off + s, off + e, 0);
      }
    }
    off += c[j];
    P.count[k] = 0;
  }
}

__global__ void k_perm(KParams P) {
  for (int64_t i = grid_stride_begin(); i < P.n; i += grid_stride_step())
    P.perm[P.offset[P.key[i]] + P.rank[i]] = (int32_t)i;
}

// ------------------------------------------------------------------ P2G
// Per work item (one grid block's bucket, up to `chunk` particles): gather each particle
// from the old order through perm, run compute_F_tmp + svd + material update + stress
// (mpm_solver.py:293-307, 339-377), write the full particle to its sorted slot, and
// scatter mass and APIC momentum (mpm_solver.py:379-418) into a 6^3-node shared-memory
// tile.  The tile is flushed with one 16-byte vector reduction per touched node.
__global__ void __launch_bounds__(256) k_p2g(KParams P) {
  __shared__ float s_m[TILE_NODES], s_px[TILE_NODES], s_py[TILE_NODES], s_pz[TILE_NODES];
  __shared__ int s_touch[8];
  const int n_items = *P.n_items;
  const int64_t cap = P.cap;
  const float* Sx = P.src;
  float* Dx = P.dst;
  for (int it = blockIdx.x; it < n_items; it += gridDim.x) {
    const int4 item = P.items[it];
    const bool real = item.x < P.K;
    int32_t sid = 0;
    int org[3] = {0, 0, 0};
    if (real) {
      sid = P.block_scene[item.x];
      const SceneDev& S = P.scenes[sid];
      const int64_t lb = (int64_t)item.x - S.block_base;
      org[2] = (int)(lb % S.bres[2]) * BLK;
      org[1] = (int)((lb / S.bres[2]) % S.bres[1]) * BLK;
      org[0] = (int)(lb / ((int64_t)S.bres[2] * S.bres[1])) * BLK;
      for (int t = threadIdx.x; t < TILE_NODES; t += blockDim.x) {
        s_m[t] = 0.f;
        s_px[t] = 0.f;
        s_py[t] = 0.f;
        s_pz[t] = 0.f;
      }
      if (threadIdx.x < 8) s_touch[threadIdx.x] = 0;
    }
    __syncthreads();
    for (int slot = item.y + threadIdx.x; slot < item.z; slot += blockDim.x) {
      const int64_t si = P.perm[slot];
      const uint32_t info = __float_as_uint(Sx[(int64_t)PF_INFO * cap + si]);
      if (!real || !(info & INFO_ACTIVE)) {
        for (int k = 0; k < P.nf; ++k) Dx[(int64_t)k * cap + slot] = Sx[(int64_t)k * cap + si];
        continue;
      }
      const SceneDev& S = P.scenes[sid];
      const MaterialDev& M = P.mats[info & INFO_MAT_MASK];
      float x[3], v[3], C[9], F[9];
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        x[d] = Sx[(int64_t)(PF_POS + d) * cap + si];
        v[d] = Sx[(int64_t)(PF_VEL + d) * cap + si];
      }
#pragma unroll
      for (int k = 0; k < 9; ++k) {
        C[k] = Sx[(int64_t)(PF_C + k) * cap + si];
        F[k] = Sx[(int64_t)(PF_F + k) * cap + si];
      }
      const float Jp = Sx[(int64_t)PF_JP * cap + si];
      const float pid = Sx[(int64_t)PF_PID * cap + si];
      float actu = 0.f, mdir[3] = {0.f, 0.f, 1.f};
      if (P.nf > NF_BASE) {
        actu = Sx[(int64_t)PF_ACTU * cap + si];
#pragma unroll
        for (int d = 0; d < 3; ++d) mdir[d] = Sx[(int64_t)(PF_MDIR + d) * cap + si];
      }
      // F_tmp = (I + dt C) F   (compute_F_tmp, mpm_solver.py:293-299)
      float A[9], Ft[9];
#pragma unroll
      for (int k = 0; k < 9; ++k) A[k] = ((k % 4 == 0) ? 1.f : 0.f) + S.dt * C[k];
      mat_mul(A, F, Ft);
      // svd (mpm_solver.py:301-307)
      float U[9], sig[3], V[9];
      const float res = svd3<float, SVD_SWEEPS>(Ft, U, sig, V);
      if (!(res <= SVD_FP64_TOL)) {
        svd3_fp64(Ft, U, sig, V);
        atomicAdd(P.fp64_count, 1ull);
      }
      // material update + stress (mpm_solver.py:339-375)
      float Fn[9], Pk[9], Jpn;
      material_update<float>(M, Ft, U, sig, V, Jp, actu, mdir, P.eps_norm, Fn, Jpn, Pk);
      // write the particle to its sorted slot (frame f+1: F, Jp; pos/vel/C carried)
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        Dx[(int64_t)(PF_POS + d) * cap + slot] = x[d];
        Dx[(int64_t)(PF_VEL + d) * cap + slot] = v[d];
      }
#pragma unroll
      for (int k = 0; k < 9; ++k) {
        Dx[(int64_t)(PF_C + k) * cap + slot] = C[k];
        Dx[(int64_t)(PF_F + k) * cap + slot] = Fn[k];
      }
      Dx[(int64_t)PF_JP * cap + slot] = Jpn;
      Dx[(int64_t)PF_INFO * cap + slot] = __uint_as_float(info);
      Dx[(int64_t)PF_PID * cap + slot] = pid;
      if (P.nf > NF_BASE) {
        Dx[(int64_t)PF_ACTU * cap + slot] = actu;
#pragma unroll
        for (int d = 0; d < 3; ++d) Dx[(int64_t)(PF_MDIR + d) * cap + slot] = mdir[d];
      }
      // APIC scatter (mpm_solver.py:376-418)
      const float mass = M.mass;
      float aff[9];
#pragma unroll
      for (int k = 0; k < 9; ++k) aff[k] = S.stress_scale * Pk[k] + mass * C[k];
      int tb[3];
      float fx[3], w[3][3];
      bool inside = true;
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const float t = __fmul_rn(x[d], S.inv_dx);
        const int b = (int)floorf(__fsub_rn(t, 0.5f));
        fx[d] = t - (float)b;
        tb[d] = b - S.offset[d] - org[d];
        inside = inside && tb[d] >= 0 && tb[d] < BLK;
        bspline_w(fx[d], w[d]);
      }
      if (!inside) {  // cannot happen for a correctly keyed particle; never touch memory
        atomicOr(P.status, 2u);
        continue;
      }
      const float mv[3] = {mass * v[0], mass * v[1], mass * v[2]};
      const bool is_free = (info & INFO_FREE) != 0;
#pragma unroll
      for (int ox = 0; ox < 3; ++ox)
#pragma unroll
        for (int oy = 0; oy < 3; ++oy)
#pragma unroll
          for (int oz = 0; oz < 3; ++oz) {
            const float wt = w[0][ox] * w[1][oy] * w[2][oz];
            const float dp[3] = {((float)ox - fx[0]) * S.dx, ((float)oy - fx[1]) * S.dx, ((float)oz - fx[2]) * S.dx};
            const int idx = ((tb[0] + ox) * TILE + (tb[1] + oy)) * TILE + (tb[2] + oz);
            atomicAdd(&s_m[idx], wt * mass);
            atomicAdd(&s_px[idx], wt * (mv[0] + aff[0] * dp[0] + aff[1] * dp[1] + aff[2] * dp[2]));
            atomicAdd(&s_py[idx], wt * (mv[1] + aff[3] * dp[0] + aff[4] * dp[1] + aff[5] * dp[2]));
            atomicAdd(&s_pz[idx], wt * (mv[2] + aff[6] * dp[0] + aff[7] * dp[1] + aff[8] * dp[2]));
          }
      if (!is_free && P.pin) {  // non-free particle: its 27 nodes lose all momentum (mpm_solver.py:420-421)
        for (int o = 0; o < 27; ++o) {
          const int gx = tb[0] + org[0] + o / 9, gy = tb[1] + org[1] + (o / 3) % 3, gz = tb[2] + org[2] + o % 3;
          const int64_t a = node_addr(S, gx, gy, gz);
          atomicOr(&P.pin[a >> 5], 1u << (a & 31));
        }
      }
    }
    if (!real) continue;  // uniform across the CTA
    __syncthreads();
    const SceneDev& S = P.scenes[sid];
    for (int t = threadIdx.x; t < TILE_NODES; t += blockDim.x) {
      const float m = s_m[t];
      if (m == 0.f) continue;
      const int tx = t / (TILE * TILE), ty = (t / TILE) % TILE, tz = t % TILE;
      const int gx = org[0] + tx, gy = org[1] + ty, gz = org[2] + tz;
      if (gx >= S.res[0] || gy >= S.res[1] || gz >= S.res[2]) continue;
      atomicAdd(reinterpret_cast<float4*>(&P.grid[node_addr(S, gx, gy, gz)]), make_float4(s_px[t], s_py[t], s_pz[t], m));
      s_touch[(tx >> 2) * 4 + (ty >> 2) * 2 + (tz >> 2)] = 1;
    }
    __syncthreads();
    if (threadIdx.x < 8 && s_touch[threadIdx.x]) {
      const int bx = org[0] / BLK + (threadIdx.x >> 2), by = org[1] / BLK + ((threadIdx.x >> 1) & 1),
                bz = org[2] / BLK + (threadIdx.x & 1);
      if (bx < S.bres[0] && by < S.bres[1] && bz < S.bres[2]) {
        const int64_t blk = S.block_base + ((int64_t)bx * S.bres[1] + by) * S.bres[2] + bz;
        if (atomicExch(&P.flags[blk], 1) == 0) P.list[atomicAdd(P.nlist, 1)] = (int32_t)blk;
      }
    }
  }
}

// ------------------------------------------------------------------ grid op
// legacy_coupler.py:356-501 without coupling partners: for nodes with mass > eps,
// v = (1/m) p + dt g, then CubeBoundary.impose_pos_vel at the node position; 0 otherwise.
// Also clears the other grid buffer's blocks touched in the previous substep.
__global__ void __launch_bounds__(256) k_grid_op(KParams P) {
  const int sub = threadIdx.x >> 6, ln = threadIdx.x & 63;
  const int per_iter = (int)gridDim.x * (blockDim.x >> 6);
  const int n_other = *P.nlist_other;
  for (int i = blockIdx.x * (blockDim.x >> 6) + sub; i < n_other; i += per_iter) {
    const int32_t blk = P.list_other[i];
    P.grid_other[(int64_t)blk * BLK_NODES + ln] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (ln == 0) P.flags_other[blk] = 0;
  }
  const int n_cur = *P.nlist;
  for (int i = blockIdx.x * (blockDim.x >> 6) + sub; i < n_cur; i += per_iter) {
    const int32_t blk = P.list[i];
    const SceneDev& S = P.scenes[P.block_scene[blk]];
    const int64_t lb = (int64_t)blk - S.block_base;
    const int bz = (int)(lb % S.bres[2]), by = (int)((lb / S.bres[2]) % S.bres[1]),
              bx = (int)(lb / ((int64_t)S.bres[2] * S.bres[1]));
    const int g[3] = {bx * BLK + (ln >> 4), by * BLK + ((ln >> 2) & 3), bz * BLK + (ln & 3)};
    float4* node = &P.grid[(int64_t)blk * BLK_NODES + ln];
    float4 q = *node;
    if (P.pin) {  // nodes touched by a non-free particle keep no momentum (mpm_solver.py:420-421)
      const int64_t a = (int64_t)blk * BLK_NODES + ln;
      const uint32_t bit = 1u << (a & 31);
      if (P.pin[a >> 5] & bit) {
        q.x = q.y = q.z = 0.f;
        atomicAnd(&P.pin[a >> 5], ~bit);
      }
    }
    float v[3] = {0.f, 0.f, 0.f};
    if (q.w > S.eps) {
      const float inv = 1.f / q.w;
      v[0] = inv * q.x + S.dt * S.grav[0];
      v[1] = inv * q.y + S.dt * S.grav[1];
      v[2] = inv * q.z + S.dt * S.grav[2];
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const float pos = (float)(g[d] + S.offset[d]) * S.dx;
        if (pos >= S.hi[d] && v[d] >= 0.f) v[d] *= -S.restitution;
        else if (pos <= S.lo[d] && v[d] <= 0.f) v[d] *= -S.restitution;
      }
    }
    *node = make_float4(v[0], v[1], v[2], q.w);
  }
}

// Dense copy of one scene's grid in x-major [gx, gy, gz, 4] order.
__global__ void k_get_grid(KParams P, int64_t scene, float* out) {
  const SceneDev& S = P.scenes[scene];
  const int64_t total = (int64_t)S.res[0] * S.res[1] * S.res[2];
  for (int64_t i = grid_stride_begin(); i < total; i += grid_stride_step()) {
    const int gz = (int)(i % S.res[2]);
    const int gy = (int)((i / S.res[2]) % S.res[1]);
    const int gx = (int)(i / ((int64_t)S.res[2] * S.res[1]));
    const float4 q = P.grid[node_addr(S, gx, gy, gz)];
    out[i * 4 + 0] = q.x;
    out[i * 4 + 1] = q.y;
    out[i * 4 + 2] = q.z;
    out[i * 4 + 3] = q.w;
  }
}

__global__ void k_count_touched(KParams P, unsigned long long* out) {
  const int n_cur = *P.nlist;
  unsigned long long c = 0;
  for (int64_t i = grid_stride_begin(); i < (int64_t)n_cur * BLK_NODES; i += grid_stride_step()) {
    const int32_t blk = P.list[i / BLK_NODES];
    const SceneDev& S = P.scenes[P.block_scene[blk]];
    if (P.grid[(int64_t)blk * BLK_NODES + (i % BLK_NODES)].w > S.eps) ++c;
  }
  for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, c);
}

}  // namespace gbmpm
