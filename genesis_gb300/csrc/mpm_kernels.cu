// mpm_kernels.cu - sm_103a kernels of the MLS-MPM substep (P2G, grid op, G2P) and of the
// per-substep particle re-sort, plus the state I/O kernels.
//
// One substep = k_p2g -> k_grid_op -> k_g2p -> k_scan_onepass (or k_scan_single) -> k_perm;
// without particles pinned to their nodes the grid op runs inside k_g2p (per staged node) and
// k_grid_op is not launched.  Reference semantics:
// genesis/engine/solvers/mpm_solver.py (p2g :322-421, g2p :423-481) and
// genesis/engine/couplers/legacy_coupler.py
// (mpm_grid_op :356-501); see each kernel.
#include "mpm_kernels.cuh"
#include "mpm_colliders.cuh"
#include "mpm_force_fields.cuh"

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
  for (int k = NF_MUSCLE; k < nf; ++k) D[(int64_t)k * cap + i] = 0.f;  // CPIC normals
}

// FP64 re-solve for the rare particle whose FP32 factor fails its residual check; kept out
// of line so its registers do not weigh on the P2G kernel.
__device__ __forceinline__ void svd3_fp64(const float* Ft, float* U, float* sig, float* V) {
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

// Pool mode: append n_add particles of scene `s` at slots [n0, n0 + n_add) of the current
// buffer (pid 0..n_add-1, material = scene base + mat_local[i] or + 0).
__global__ void k_admit(KParams P, int32_t s, int64_t n0, int64_t n_add, const float* pos, const int32_t* mat_local) {
  float* D = P.dst;
  const SceneDev& S = P.scenes[s];
  for (int64_t j = grid_stride_begin(); j < n_add; j += grid_stride_step()) {
    const int64_t i = n0 + j;
    const uint32_t gmat = (uint32_t)(S.mat_begin + (mat_local ? mat_local[j] : 0));
    write_defaults(D, P.cap, i, P.nf, P.mats[gmat].default_Jp);
#pragma unroll
    for (int d = 0; d < 3; ++d) D[(int64_t)(PF_POS + d) * P.cap + i] = pos[j * 3 + d];
    D[(int64_t)PF_INFO * P.cap + i] = __uint_as_float(gmat | INFO_FREE | INFO_ACTIVE);
    D[(int64_t)PF_PID * P.cap + i] = __uint_as_float((uint32_t)j);
  }
}

// Pool mode: mark every particle of scene `s` dead (dropped by the next sort).
__global__ void k_retire(KParams P, int32_t s) {
  float* D = P.dst;
  for (int64_t i = grid_stride_begin(); i < P.n; i += grid_stride_step()) {
    const uint32_t info = ld_info(D, P.cap, i);
    if (!(info & INFO_DEAD) && scene_of(P, info) == s)
      D[(int64_t)PF_INFO * P.cap + i] = __uint_as_float(info | INFO_DEAD);
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

// Row-ordered state I/O (outside pool mode, where every row of scenes [s0, s1) holds exactly
// one particle).  k_row_slots inverts the sorted layout once: for each particle slot it stores
// the slot and the particle's info word at the particle's output row (4-byte writes into two
// cap-sized arrays that stay in L2).  The gather and the row-order rewrite then read and write
// the [B, N] rows coalesced.  The two arrays are the sort's key and rank arrays, which only
// k_perm reads, right after they are written within a substep or a re-keying; between substeps
// they are free.
__global__ void k_row_slots(KParams P, int64_t s0, int64_t s1, int32_t* row_slot, uint32_t* row_info) {
  const float* D = P.dst;
  for (int64_t i = grid_stride_begin(); i < P.n; i += grid_stride_step()) {
    const uint32_t info = ld_info(D, P.cap, i);
    const int32_t s = scene_of(P, info);
    if (s < s0 || s >= s1) continue;
    const int64_t r = out_row(P, s, s0, __float_as_uint(D[(int64_t)PF_PID * P.cap + i]));
    row_slot[r] = (int32_t)i;
    row_info[r] = info;
  }
}

// mpm_solver.py:759-778 (_kernel_get_state) in row order: gathers each row's particle through
// row_slot.
__global__ void k_get_state_rows(KParams P, int64_t rows, const int32_t* row_slot, const uint32_t* row_info,
                                 float* pos, float* vel, float* C, float* F, float* Jp, uint8_t* active) {
  const float* D = P.dst;
  for (int64_t r = grid_stride_begin(); r < rows; r += grid_stride_step()) {
    const int64_t i = row_slot[r];
    if (pos)
      for (int d = 0; d < 3; ++d) pos[r * 3 + d] = D[(int64_t)(PF_POS + d) * P.cap + i];
    if (vel)
      for (int d = 0; d < 3; ++d) vel[r * 3 + d] = D[(int64_t)(PF_VEL + d) * P.cap + i];
    if (C)
      for (int d = 0; d < 9; ++d) C[r * 9 + d] = D[(int64_t)(PF_C + d) * P.cap + i];
    if (F)
      for (int d = 0; d < 9; ++d) F[r * 9 + d] = D[(int64_t)(PF_F + d) * P.cap + i];
    if (Jp) Jp[r] = D[(int64_t)PF_JP * P.cap + i];
    if (active) active[r] = (row_info[r] & INFO_ACTIVE) ? 1 : 0;
  }
}

// mpm_solver.py:729-749 (_kernel_set_state) for a full state of every scene: particle r is
// rewritten into slot r (the layout the context starts with), so the new state is read and
// written coalesced; only its info word comes from its old slot (row_info).  The particle
// order no longer matches the last sort, which the caller marks stale (re-keying follows).
// Requires the base planes only (no muscle or CPIC planes to carry along).
__global__ void k_set_state_rows(KParams P, int64_t rows, const uint32_t* row_info, const float* pos,
                                 const float* vel, const float* C, const float* F, const float* Jp,
                                 const uint8_t* active) {
  float* D = P.dst;
  for (int64_t r = grid_stride_begin(); r < rows; r += grid_stride_step()) {
    uint32_t info = row_info[r];
    if (active) info = active[r] ? (info | INFO_ACTIVE) : (info & ~INFO_ACTIVE);
    const int32_t s = scene_of(P, info);
    for (int d = 0; d < 3; ++d) {
      D[(int64_t)(PF_POS + d) * P.cap + r] = pos[r * 3 + d];
      D[(int64_t)(PF_VEL + d) * P.cap + r] = vel[r * 3 + d];
    }
    for (int d = 0; d < 9; ++d) {
      D[(int64_t)(PF_C + d) * P.cap + r] = C[r * 9 + d];
      D[(int64_t)(PF_F + d) * P.cap + r] = F[r * 9 + d];
    }
    D[(int64_t)PF_JP * P.cap + r] = Jp[r];
    D[(int64_t)PF_INFO * P.cap + r] = __uint_as_float(info);
    D[(int64_t)PF_PID * P.cap + r] = __uint_as_float((uint32_t)(r - P.scenes[s].p_begin));
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

// ------------------------------------------------------------------ re-keying
// Bucket key and warp-aggregated rank of every particle from its current position (after
// a state change: load, set_state, set_particles).  The per-substep keys come from k_g2p.
__global__ void __launch_bounds__(256) k_keys(KParams P) {
  const float* D = P.dst;
  const int64_t cap = P.cap;
  const int lane = threadIdx.x & 31;
  const int64_t warp0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t base = warp0 * 32; base < P.n; base += nwarps * 32) {
    const int64_t i = base + lane;
    const bool valid = i < P.n;
    int32_t key = (int32_t)P.K;
    int cell = BLK_NODES;
    if (valid) {
      const uint32_t info = ld_info(D, cap, i);
      if (info & INFO_DEAD) {
        key = (int32_t)P.K + 1;
      } else if (info & INFO_ACTIVE) {
        const SceneDev& S = P.scenes[scene_of(P, info)];
        float x[3];
        int b[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) x[d] = D[(int64_t)(PF_POS + d) * cap + i];
        if (stencil_origin(S, x, b)) {
          key = (int32_t)block_of(S, b[0], b[1], b[2]);
          cell = ((b[0] & 3) * 4 + (b[1] & 3)) * 4 + (b[2] & 3);
        } else {
          atomicOr(P.status, (isfinite(x[0]) && isfinite(x[1]) && isfinite(x[2])) ? 2u : 1u);
        }
      }
    }
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
      P.cell8[i] = (uint8_t)cell;
    }
  }
}

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

// One-pass scan of the bucket counts with decoupled look-back (Merrill & Garland, "Single-pass
// Parallel Prefix Scan with Decoupled Look-back", 2016): a CTA takes the next tile by ticket,
// publishes its tile aggregate, sums its predecessors' words back to the nearest inclusive
// prefix (a warp reads 32 words per round), publishes its own inclusive prefix, then writes
// its tile's bucket offsets, P2G work items and count reset.  A predecessor holds an earlier
// ticket, so it is already running and publishes without waiting; the wait is still bounded
// (MPM_STATUS_WAIT on exhaustion).  The CTA that finishes last resets the tile words and the
// ticket for the next scan.
namespace {
constexpr unsigned long long SCAN_AGG = 1ull << 62, SCAN_PRE = 2ull << 62;
constexpr unsigned SCAN_SPIN_LIMIT = 1u << 20;
__device__ __forceinline__ unsigned long long scan_word(unsigned long long flag, int c, int i) {
  return flag | ((unsigned long long)(uint32_t)c << 31) | (unsigned long long)(uint32_t)i;
}
}  // namespace

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_onepass(KParams P) {
  constexpr int PER = SCAN_TILE / SCAN_THREADS;
  __shared__ int s_tile, s_last;
  __shared__ int2 s_prefix;
  // Only the live tiles take part (a pool's empty slots and the unused blocks of small grids hold
  // no particle, so their buckets are skipped; the captured launch keeps its full CTA count and the
  // extra CTAs return here, before any ticket).
  pdl_wait();
  const int n_live = *P.n_scan_tiles;
  if ((int)blockIdx.x >= n_live) return;
  if (threadIdx.x == 0) s_tile = atomicAdd(&P.scan_sync[0], 1);
  __syncthreads();
  const int tile = s_tile;
  const int2 range = P.scan_tiles[tile];
  const int64_t nb = range.y;
  const int64_t k0 = (int64_t)range.x + (int64_t)threadIdx.x * PER;
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
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    // (scan_hold_tile0: a failure-detection test keeps tile 0 from publishing, so its successor's
    // wait runs out)
    const bool hold = P.scan_hold_tile0 && tile == 0;
    if (lane == 0 && !hold)
      atomicExch(&P.scan_state[tile], scan_word(tile == 0 ? SCAN_PRE : SCAN_AGG, total.x, total.y));
    int pc = 0, pi = 0;
    int j = tile - 1;
    unsigned spins = 0;
    while (j >= 0) {
      const int idx = j - lane;
      const unsigned long long w = idx >= 0 ? atomicAdd(&P.scan_state[idx], 0ull) : SCAN_PRE;
      const unsigned long long flag = w & (3ull << 62);
      if (__any_sync(0xffffffffu, flag == 0ull)) {  // a predecessor has not published yet
        if (++spins > (P.scan_spin_limit ? P.scan_spin_limit : SCAN_SPIN_LIMIT)) {
          if (lane == 0) atomicOr(P.status, MPM_STATUS_WAIT);
          break;
        }
        continue;
      }
      const unsigned pre = __ballot_sync(0xffffffffu, flag == SCAN_PRE);
      const int stop = pre ? __ffs(pre) - 1 : 31;  // lanes 0..stop are summed
      int vc = lane <= stop ? (int)((w >> 31) & 0x7fffffffull) : 0;
      int vi = lane <= stop ? (int)(w & 0x7fffffffull) : 0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        vc += __shfl_xor_sync(0xffffffffu, vc, o);
        vi += __shfl_xor_sync(0xffffffffu, vi, o);
      }
      pc += vc;
      pi += vi;
      if (pre) break;
      j -= 32;
    }
    if (lane == 0) {
      if (tile > 0) atomicExch(&P.scan_state[tile], scan_word(SCAN_PRE, pc + total.x, pi + total.y));
      s_prefix = make_int2(pc, pi);
    }
  }
  __syncthreads();
  const int2 base = s_prefix;
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
  if (tile == n_live - 1 && threadIdx.x == 0) *P.n_items = base.y + total.y;
  if (threadIdx.x == 0) {
    __threadfence();
    s_last = atomicAdd(&P.scan_sync[1], 1) == n_live - 1;
  }
  __syncthreads();
  if (s_last) {  // every CTA is past its look-back: reset for the next scan
    for (int t = threadIdx.x; t < n_live; t += blockDim.x) P.scan_state[t] = 0ull;
    if (threadIdx.x == 0) {
      P.scan_sync[0] = 0;
      P.scan_sync[1] = 0;
    }
  }
  pdl_trigger();
}

// The whole scan in one CTA (1024 threads) when the bucket count is small: counts -> offsets,
// work items and count reset, in three passes over the buckets with block-wide scans.
__global__ void __launch_bounds__(1024) k_scan_single(KParams P) {
  __shared__ int2 s_warp[32];
  __shared__ int2 s_carry;
  const int64_t nb = P.K + 2;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  pdl_wait();
  if (threadIdx.x == 0) s_carry = make_int2(0, 0);
  __syncthreads();
  for (int64_t k0 = 0; k0 < nb; k0 += blockDim.x) {
    const int64_t k = k0 + threadIdx.x;
    const int c = k < nb ? P.count[k] : 0;
    const int ic = (k <= P.K) ? items_of(c, P.chunk) : 0;
    int a = c, b = ic;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int ta = __shfl_up_sync(0xffffffffu, a, o), tb = __shfl_up_sync(0xffffffffu, b, o);
      if (lane >= o) {
        a += ta;
        b += tb;
      }
    }
    if (lane == 31) s_warp[wid] = make_int2(a, b);
    __syncthreads();
    if (wid == 0) {
      int2 v = lane < nwarp ? s_warp[lane] : make_int2(0, 0);
      int x = v.x, y = v.y;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int tx = __shfl_up_sync(0xffffffffu, x, o), ty = __shfl_up_sync(0xffffffffu, y, o);
        if (lane >= o) {
          x += tx;
          y += ty;
        }
      }
      if (lane < nwarp) s_warp[lane] = make_int2(x - v.x, y - v.y);
    }
    __syncthreads();
    const int2 base = s_carry;
    const int2 wo = s_warp[wid];
    const int off = base.x + wo.x + a - c, it0 = base.y + wo.y + b - ic;
    if (k < nb) {
      P.offset[k] = off;
      for (int s = 0, j = 0; s < c && k <= P.K; s += P.chunk, ++j)
        P.items[it0 + j] = make_int4((int)k, off + s, off + min(s + P.chunk, c), 0);
      P.count[k] = 0;
    }
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) s_carry = make_int2(off + c, it0 + ic);
    __syncthreads();
  }
  if (threadIdx.x == 0) *P.n_items = s_carry.y;
  pdl_trigger();
}


// ------------------------------------------------------------------ kinematic colliders
namespace {
// Tool mesh SDF in voxel coordinates (mesh.py:92-107): 1 outside the grid.
__device__ __forceinline__ float tool_sdf_vox(const ColliderDev& c, const float* ps) {
  int base[3];
  bool outside = false;
  for (int k = 0; k < 3; ++k) {
    base[k] = (int)floorf(ps[k]);
    outside = outside || base[k] >= c.res[k] - 1 || base[k] < 0;
  }
  return outside ? 1.f : sdf_trilinear(c, ps, base, nullptr);
}

// The tool's pose one substep later (tool_entity.py:193-206): pos + v dt clamped to the floor,
// quat turned by the rotation vector w dt (qd_rotvec_to_quat with its first-order normalisation,
// then qd_transform_quat_by_quat: normalize(q_rot * quat)).
__device__ __forceinline__ void tool_next_pose(const ColliderDev& c, float dt, float eps, float* pn, float* qn) {
  for (int k = 0; k < 3; ++k) pn[k] = c.pos[k] + c.lin[k] * dt;
  pn[2] = fmaxf(pn[2], c.floor_h);
  const float rv[3] = {c.ang[0] * dt, c.ang[1] * dt, c.ang[2] * dt};
  const float th2 = rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2];
  float u[4] = {1.f, 0.f, 0.f, 0.f};
  if (th2 > eps * eps) {
    const float th = sqrtf(th2);
    const float cs = cosf(0.5f * th), sn = sinf(0.5f * th);
    u[0] = cs;
    for (int k = 0; k < 3; ++k) u[k + 1] = sn / th * rv[k];
    const float s = 0.5f * (3.f - (u[0] * u[0] + u[1] * u[1] + u[2] * u[2] + u[3] * u[3]));
    for (int k = 0; k < 4; ++k) u[k] *= s;
  }
  const float* v = c.quat;
  const float q[4] = {u[0] * v[0] - u[1] * v[1] - u[2] * v[2] - u[3] * v[3],
                      u[0] * v[1] + u[1] * v[0] + u[2] * v[3] - u[3] * v[2],
                      u[0] * v[2] - u[1] * v[3] + u[2] * v[0] + u[3] * v[1],
                      u[0] * v[3] + u[1] * v[2] - u[2] * v[1] + u[3] * v[0]};
  const float qn_len = sqrtf(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  for (int k = 0; k < 4; ++k) qn[k] = q[k] / qn_len;
}

// Mesh.collide (mesh.py:148-177) of a tool at node position x, node velocity v.
__device__ void collide_tool(const ColliderDev& c, const SceneDev& S, const float* x, float* v) {
  float pm[3], ps[3];
  sdf_voxel_pos(c, c.pos, c.quat, x, pm, ps);
  const float sd = tool_sdf_vox(c, ps);
  const float influence = fminf(expf(-sd / fmaxf(S.eps, c.softness)), 1.f);
  if (!(sd <= 0.f || influence > 0.1f)) return;
  float pn[3], qn[4], xn[3];
  tool_next_pose(c, S.dt, S.eps, pn, qn);
  rot(qn, pm, xn);
  float vc[3], rv[3];
  for (int k = 0; k < 3; ++k) {
    vc[k] = (xn[k] + pn[k] - x[k]) / S.dt;
    rv[k] = v[k] - vc[k];
  }
  // normal: central differences in voxel space (delta 1e-2), back to the mesh frame, then world
  float nv[3];
  for (int i = 0; i < 3; ++i) {
    float inc[3] = {ps[0], ps[1], ps[2]}, dec[3] = {ps[0], ps[1], ps[2]};
    inc[i] += 1e-2f;
    dec[i] -= 1e-2f;
    nv[i] = (tool_sdf_vox(c, inc) - tool_sdf_vox(c, dec)) / (2.f * 1e-2f);
  }
  float l = sqrtf(nv[0] * nv[0] + nv[1] * nv[1] + nv[2] * nv[2] + S.eps);
  for (int k = 0; k < 3; ++k) nv[k] /= l;
  float nm[3], n[3];
  for (int r = 0; r < 3; ++r) nm[r] = c.Rinv[r * 3 + 0] * nv[0] + c.Rinv[r * 3 + 1] * nv[1] + c.Rinv[r * 3 + 2] * nv[2];
  rot(c.quat, nm, n);
  l = sqrtf(n[0] * n[0] + n[1] * n[1] + n[2] * n[2] + S.eps);
  for (int k = 0; k < 3; ++k) n[k] /= l;
  const float rvn = rv[0] * n[0] + rv[1] * n[1] + rv[2] * n[2];
  if (!(rvn < 0.f)) return;
  float rt[3];
  for (int k = 0; k < 3; ++k) rt[k] = rv[k] - rvn * n[k];
  const float rtn = sqrtf(rt[0] * rt[0] + rt[1] * rt[1] + rt[2] * rt[2] + S.eps);
  const float mag = fmaxf(0.f, rtn + rvn * c.friction);
  for (int k = 0; k < 3; ++k) v[k] = vc[k] + rt[k] / rtn * mag * influence + rv[k] * (1.f - influence);
}

// _func_collide_in_rigid_geom (legacy_coupler.py:284-347) with its reaction: the velocity change
// of collide_in_velocity (mpm_colliders.cuh) gives the force and torque added to collider_acc.
__device__ void collide_in(const KParams& P, const SceneDev& S, int ci, const float* x, float* v, float m,
                           const float* n, float influence) {
  const ColliderDev& c = P.colliders[ci];
  const float v0[3] = {v[0], v[1], v[2]};
  if (!collide_in_velocity(c, S.eps, x, v, n, influence)) return;
  const float r[3] = {x[0] - c.com[0], x[1] - c.com[1], x[2] - c.com[2]};
  const float dv[3] = {v[0] - v0[0], v[1] - v0[1], v[2] - v0[2]};
  // particle -> rigid: force = -m dv / dt at x, torque (x - com) x force
  const float f[3] = {-m * dv[0] / S.dt, -m * dv[1] / S.dt, -m * dv[2] / S.dt};
  double* acc = P.collider_acc + (int64_t)ci * 6;
  atomicAdd(acc + 0, (double)f[0]);
  atomicAdd(acc + 1, (double)f[1]);
  atomicAdd(acc + 2, (double)f[2]);
  atomicAdd(acc + 3, (double)(r[1] * f[2] - r[2] * f[1]));
  atomicAdd(acc + 4, (double)(r[2] * f[0] - r[0] * f[2]));
  atomicAdd(acc + 5, (double)(r[0] * f[1] - r[1] * f[0]));
}

// _func_collide_with_rigid (legacy_coupler.py:134-218): every collider of the node's scene whose
// SDF influence exceeds 0.1 at x, in order.
// Tools come first (legacy_coupler.py:386-387 before :389-403).
__device__ void collide_node(const KParams& P, const SceneDev& S, int32_t scene, const float* x, float* v, float m) {
  for (int ci = 0; ci < P.n_colliders; ++ci) {
    const ColliderDev& c = P.colliders[ci];
    if (c.type == MPM_COLLIDER_TOOL && (c.scene < 0 || c.scene == scene)) collide_tool(c, S, x, v);
  }
  for (int ci = 0; ci < P.n_colliders; ++ci) {
    const ColliderDev& c = P.colliders[ci];
    if (c.type == MPM_COLLIDER_TOOL || (c.scene >= 0 && c.scene != scene)) continue;
    float n[3];
    const float sd = collider_sdf(c, x, S.eps, n);
    const float influence = fminf(expf(-sd / fmaxf(1e-10f, c.softness)), 1.f);
    if (!(influence > 0.1f)) continue;
    collide_in(P, S, ci, x, v, m, n, influence);
  }
}

// MPM <-> SPH, then MPM <-> PBD (legacy_coupler.py:404-498) at node address a with MPM mass m:
// when the set has particles in the node's cell, the node takes their mean velocity and each of
// them loses delta_mv / m_i, delta_mv = m (v_new - v_old) (PBD: only free particles).  The lists
// are acyclic by construction; a walk longer than the set still stops and flags the status.
__device__ void couple_ext(const KParams& P, int64_t a, float* v, float m) {
  for (int k = 0; k < 2; ++k) {
    const ExtSetDev& E = P.ext[k];
    if (E.n == 0) continue;
    const int64_t total = E.n * (int64_t)P.n_scenes;
    const int32_t h = E.head[a];
    if (h < 0) continue;
    float sv[3] = {0.f, 0.f, 0.f};
    int64_t cnt = 0;
    for (int32_t j = h; j >= 0 && j < total; j = E.next[j]) {
      if (++cnt > total) {
        atomicOr(P.status, MPM_STATUS_BAD_INDEX);
        return;
      }
      for (int d = 0; d < 3; ++d) sv[d] += E.vel[(int64_t)j * 3 + d];
    }
    float dmv[3];
    for (int d = 0; d < 3; ++d) {
      const float vn = sv[d] / (float)cnt;
      dmv[d] = m * (vn - v[d]);
      v[d] = vn;
    }
    int64_t left = cnt;
    for (int32_t j = h; j >= 0 && j < total && left > 0; j = E.next[j], --left) {
      if (k == 1 && E.free_ && !E.free_[j]) continue;
      const float mi = E.mass[j];
      for (int d = 0; d < 3; ++d) E.vel[(int64_t)j * 3 + d] -= dmv[d] / mi;
    }
  }
}

// CPIC (MPMOptions.enable_CPIC) for thin colliders.  Particle side, mpm_surface_to_particle
// (legacy_coupler.py:513-529): per collider the particle keeps the SDF normal at its position
// unless that normal turned against the stored one, so the stored normal remembers the side the
// particle is on; the normals ride with the particle in planes PF_CPIC + 3 * collider.  Node
// side (mpm_solver.py:389-411): a stencil node lies behind collider ci when the collider's
// normal at the node points against the particle's; the first such collider, in order, counts.
__device__ __forceinline__ bool collider_in_scene(const ColliderDev& c, int32_t scene) {
  return c.type != MPM_COLLIDER_TOOL && (c.scene < 0 || c.scene == scene);  // tools: no CPIC
}

__device__ int cpic_separating(const KParams& P, const SceneDev& S, int32_t scene, const float* D, int64_t i,
                               const float* xc) {
  const int64_t cap = P.cap;
  const int nc = P.n_colliders < P.cpic_slots ? P.n_colliders : P.cpic_slots;
  for (int ci = 0; ci < nc; ++ci) {
    const ColliderDev& c = P.colliders[ci];
    if (!collider_in_scene(c, scene)) continue;
    float n[3];
    collider_sdf(c, xc, S.eps, n);
    const float* pn = D + (int64_t)(PF_CPIC + 3 * ci) * cap + i;
    if (pn[0] * n[0] + pn[cap] * n[1] + pn[2 * cap] * n[2] < 0.f) return ci;
  }
  return -1;
}

// World position of stencil node o (= ox*9 + oy*3 + oz) of a particle in local cell tb of the
// block with node origin org: (base + offset) * dx as the reference computes it.
__device__ __forceinline__ void cpic_node_pos(const SceneDev& S, const int* org, const int* tb, int o, float* xc) {
  const int oo[3] = {o / 9, (o / 3) % 3, o % 3};
#pragma unroll
  for (int d = 0; d < 3; ++d) xc[d] = (float)(org[d] + tb[d] + oo[d] + S.offset[d]) * S.dx;
}

// P2G side: moves the particle's normals from its old slot (src) to its new one (dst), updating
// them when it is active, and returns the mask of its stencil nodes behind a collider
// (bit ox*9 + oy*3 + oz); 0 when inactive or outside the block.
__device__ __noinline__ uint32_t cpic_p2g(const KParams& P, const SceneDev& S, int32_t scene, const float* x,
                                          bool active, int64_t si, int64_t slot, const int* org, int cell) {
  const int64_t cap = P.cap;
  for (int ci = 0; ci < P.cpic_slots; ++ci) {
    float pn[3];
    for (int d = 0; d < 3; ++d) pn[d] = P.src[(int64_t)(PF_CPIC + 3 * ci + d) * cap + si];
    if (active && ci < P.n_colliders && collider_in_scene(P.colliders[ci], scene)) {
      float n[3];
      collider_sdf(P.colliders[ci], x, S.eps, n);
      if (n[0] * pn[0] + n[1] * pn[1] + n[2] * pn[2] >= 0.f)
        for (int d = 0; d < 3; ++d) pn[d] = n[d];
    }
    for (int d = 0; d < 3; ++d) P.dst[(int64_t)(PF_CPIC + 3 * ci + d) * cap + slot] = pn[d];
  }
  if (!active || cell >= BLK_NODES) return 0u;
  const int tb[3] = {cell >> 4, (cell >> 2) & 3, cell & 3};
  uint32_t mask = 0u;
  for (int o = 0; o < 27; ++o) {
    float xc[3];
    cpic_node_pos(S, org, tb, o, xc);
    if (cpic_separating(P, S, scene, P.dst, slot, xc) >= 0) mask |= 1u << o;
  }
  return mask;
}

// G2P side (mpm_solver.py:445-459): a node behind collider ci contributes, instead of its grid
// velocity, the particle's own velocity collided with ci (_func_collide_in_rigid_geom with the
// particle's stored normal, influence 1 and mass m_p w / 1e3), the reaction going to ci.
__device__ __noinline__ float4 cpic_g2p_node(const KParams& P, const SceneDev& S, int32_t scene, const float* D,
                                             int64_t i, const float* x, const int* org, const int* tb, int o,
                                             float weight, float4 g) {
  const int64_t cap = P.cap;
  float xc[3];
  cpic_node_pos(S, org, tb, o, xc);
  const int ci = cpic_separating(P, S, scene, D, i, xc);
  if (ci < 0) return g;
  float v[3], pn[3];
  for (int d = 0; d < 3; ++d) {
    v[d] = D[(int64_t)(PF_VEL + d) * cap + i];
    pn[d] = D[(int64_t)(PF_CPIC + 3 * ci + d) * cap + i];
  }
  const float m = P.mats[ld_info(D, cap, i) & INFO_MAT_MASK].mass * weight / 1e3f;
  collide_in(P, S, ci, x, v, m, pn, 1.f);
  return make_float4(v[0], v[1], v[2], g.w);
}
}  // namespace

// Bucket permutation of the sort; also the end-of-substep bookkeeping.
__global__ void k_perm(KParams P) {
  pdl_wait();
  const int64_t n = P.n_dev ? *P.n_dev : P.n;
  const int64_t stride = grid_stride_step();
  // four particles per thread and pass, their loads issued together
  for (int64_t i0 = grid_stride_begin(); i0 < n; i0 += 4 * stride) {
    int32_t key[4], rank[4];
    uint8_t cell[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int64_t i = i0 + u * stride;
      key[u] = i < n ? P.key[i] : 0;
      rank[u] = i < n ? P.rank[i] : 0;
      cell[u] = i < n ? P.cell8[i] : 0;
    }
    int32_t off[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) off[u] = i0 + u * stride < n ? P.offset[key[u]] : 0;
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int64_t i = i0 + u * stride;
      if (i >= n) break;
      const int64_t dst = (int64_t)off[u] + rank[u];
      P.perm[dst] = (int32_t)i;
      P.slot_cell[dst] = cell[u];  // P2G reads each slot's cell without gathering its position
    }
  }
  if (P.nlist_reset && blockIdx.x == 0 && threadIdx.x == 0) *P.nlist_reset = 0;  // cleared by the fused G2P
  if (P.ff_step && P.ff_step_advance && blockIdx.x == 0 && threadIdx.x == 0) *P.ff_step += 1;  // end of a substep
  if (P.colliders_rw && blockIdx.x == 0)  // end of a substep: tools move (tool_entity.py:193-206)
    for (int ci = threadIdx.x; ci < P.n_colliders; ci += blockDim.x) {
      ColliderDev& c = P.colliders_rw[ci];
      if (c.type != MPM_COLLIDER_TOOL) continue;
      const SceneDev& S = P.scenes[c.scene >= 0 ? c.scene : 0];
      float pn[3], qn[4];
      tool_next_pose(c, S.dt, S.eps, pn, qn);
      for (int k = 0; k < 3; ++k) c.pos[k] = pn[k];
      for (int k = 0; k < 4; ++k) c.quat[k] = qn[k];
    }
  if (P.steps && blockIdx.x == 0)  // end of a substep: count down per-scene substep budgets
    for (int s = threadIdx.x; s < P.n_scenes; s += blockDim.x)
      if (P.steps[s] > 0) P.steps[s] -= 1;
  pdl_trigger();
}

// ------------------------------------------------------------------ P2G
namespace {

// Loads one particle from the old order (planes of `S`, index si).
struct Particle {
  float x[3], v[3], C[9], F[9], Jp, pid, actu, mdir[3];
  uint32_t info;
};

__device__ __forceinline__ void load_particle(const KParams& P, const float* Sx, int64_t si, Particle& q) {
  const int64_t cap = P.cap;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    q.x[d] = Sx[(int64_t)(PF_POS + d) * cap + si];
    q.v[d] = Sx[(int64_t)(PF_VEL + d) * cap + si];
  }
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    q.C[k] = Sx[(int64_t)(PF_C + k) * cap + si];
    q.F[k] = Sx[(int64_t)(PF_F + k) * cap + si];
  }
  q.Jp = Sx[(int64_t)PF_JP * cap + si];
  q.info = __float_as_uint(Sx[(int64_t)PF_INFO * cap + si]);
  q.pid = Sx[(int64_t)PF_PID * cap + si];
  q.actu = 0.f;
  q.mdir[0] = 0.f, q.mdir[1] = 0.f, q.mdir[2] = 1.f;
  if (P.nf > NF_BASE) {
    q.actu = Sx[(int64_t)PF_ACTU * cap + si];
#pragma unroll
    for (int d = 0; d < 3; ++d) q.mdir[d] = Sx[(int64_t)(PF_MDIR + d) * cap + si];
  }
}

// Writes a particle to its sorted slot.  Velocity and C are left out: G2P of the same substep
// overwrites both for every particle of an active bucket before anything reads them.
__device__ __forceinline__ void store_particle(const KParams& P, float* Dx, int64_t slot, const Particle& q) {
  const int64_t cap = P.cap;
#pragma unroll
  for (int d = 0; d < 3; ++d) Dx[(int64_t)(PF_POS + d) * cap + slot] = q.x[d];
#pragma unroll
  for (int k = 0; k < 9; ++k) Dx[(int64_t)(PF_F + k) * cap + slot] = q.F[k];
  Dx[(int64_t)PF_JP * cap + slot] = q.Jp;
  Dx[(int64_t)PF_INFO * cap + slot] = __uint_as_float(q.info);
  Dx[(int64_t)PF_PID * cap + slot] = q.pid;
  if (P.nf > NF_BASE) {
    Dx[(int64_t)PF_ACTU * cap + slot] = q.actu;
#pragma unroll
    for (int d = 0; d < 3; ++d) Dx[(int64_t)(PF_MDIR + d) * cap + slot] = q.mdir[d];
  }
}

// Local cell (0..63) of a particle inside the block whose node origin is `org`, or 64.
__device__ __forceinline__ int local_cell(const SceneDev& S, const float* x, const int* org, int* tb) {
  bool inside = true;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const float t = __fmul_rn(x[d], S.inv_dx);
    const float f = floorf(__fsub_rn(t, 0.5f));
    const int b = (f > -1e9f && f < 1e9f) ? (int)f : -1000000;
    tb[d] = b - S.offset[d] - org[d];
    inside = inside && tb[d] >= 0 && tb[d] < BLK;
  }
  return inside ? (tb[0] * BLK + tb[1]) * BLK + tb[2] : BLK_NODES;
}

__device__ __forceinline__ void block_origin(const SceneDev& S, int64_t key, int* org) {
  const int64_t lb = key - S.block_base;
  org[2] = (int)(lb % S.bres[2]) * BLK;
  org[1] = (int)((lb / S.bres[2]) % S.bres[1]) * BLK;
  org[0] = (int)(lb / ((int64_t)S.bres[2] * S.bres[1])) * BLK;
}

// Particles per thread of a P2G item whose old slot and cell are loaded ahead (registers).
constexpr int P2G_PF = 4;

// The head of P2G work item `item`: its scene and, for the first P2G_PF particles of each thread
// (j = thread + k * T), the old slot (perm) and the cell in the block (slot_cell).  Loaded while
// the previous item scatters, so an item does not start with a chain of dependent global loads.
__device__ __forceinline__ void p2g_item_head(const KParams& P, int4 item, int T, int32_t* si, int32_t* cell,
                                              int32_t& sid) {
  const int cnt = item.z - item.y;
  const bool real = item.x < P.K && cnt > 0;
  sid = real ? P.block_scene[item.x] : 0;
#pragma unroll
  for (int k = 0; k < P2G_PF; ++k) {
    const int j = (int)threadIdx.x + k * T;
    const bool ok = real && j < cnt;
    si[k] = ok ? P.perm[item.y + j] : 0;
    cell[k] = ok ? (int32_t)P.slot_cell[item.y + j] : 0;
  }
}

}  // namespace

// Per work item (one grid block's bucket, up to `chunk` <= P2G_MAX_CHUNK particles):
//  1. counting-sort the item's particles by cell in shared memory (native integer atomics); the
//     cell of each slot comes from the G2P (or re-keying) that keyed the particle, in slot order
//     (k_perm), and its old slot is kept in shared memory for step 2;
//  2. in slot order (coalesced gathers through perm): compute_F_tmp + svd + material update
//     + stress (mpm_solver.py:293-307, 339-377), write the particle to its slot, and leave its
//     scatter parameters (fx, mass, q = m v - sum_k a_k fx_k, a_k = dx * affine[:,k]) in a
//     shared record at its cell-sorted position;
//  3. one thread per (cell, ox) walks its cell's records and sums the APIC mass/momentum
//     w_o (q + sum_k o_k a_k), w_o m (mpm_solver.py:379-418) of the 9 nodes (ox, *, *) in
//     registers, then adds them to its warp's private 6^3 shared tile (plain float4
//     read-modify-writes; no two lanes of a warp share a node): one tile update per cell and
//     node instead of one per particle and node;
//  4. sum the warp tiles and flush with one 16-byte vector reduction per node.
// With CPIC the nodes behind a thin collider get nothing from the particle (weight 0 in step 3).
template <bool CPIC>
__device__ __forceinline__ void p2g_body(const KParams& P) {
  extern __shared__ __align__(16) unsigned char p2g_smem[];
  __shared__ int s_cnt[BLK_NODES + 1];
  __shared__ int s_touch[8];
  // the item's scene record, read from shared memory: a reference into the global table would be
  // re-read after every particle store (the compiler cannot rule out aliasing)
  __shared__ SceneDev s_scene;
  pdl_wait();  // the sort's items and the particles' previous substep
  const int n_items = *P.n_items;
  const int T = blockDim.x, nw = T >> 5, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float4* s_tile = reinterpret_cast<float4*>(p2g_smem);
  float4* s_rec = s_tile + nw * TILE_NODES;
  uint32_t* s_cr = reinterpret_cast<uint32_t*>(s_rec + P2G_REC * P.chunk);
  int32_t* s_si = reinterpret_cast<int32_t*>(s_cr + P.chunk);  // old slot of each item particle
  const int64_t cap = P.cap;
  const float* Sx = P.src;
  float* Dx = P.dst;
  float4* my_tile = s_tile + warp * TILE_NODES;
  // tiles, cell counts and touch flags start zeroed; each item leaves them zeroed again
  for (int t = threadIdx.x; t < nw * TILE_NODES; t += T) s_tile[t] = make_float4(0.f, 0.f, 0.f, 0.f);
  if (threadIdx.x <= BLK_NODES) s_cnt[threadIdx.x] = 0;
  if (threadIdx.x < 8) s_touch[threadIdx.x] = 0;
  __syncthreads();
  int4 nitem = (int)blockIdx.x < n_items ? P.items[blockIdx.x] : make_int4(0, 0, 0, 0);
  int32_t nsi[P2G_PF], ncell[P2G_PF], nsid;
  p2g_item_head(P, nitem, T, nsi, ncell, nsid);
  for (int it = blockIdx.x; it < n_items; it += gridDim.x) {
    const int4 item = nitem;
    const int32_t sid = nsid;
    int32_t pf_si[P2G_PF], pf_cell[P2G_PF];
#pragma unroll
    for (int k = 0; k < P2G_PF; ++k) {
      pf_si[k] = nsi[k];
      pf_cell[k] = ncell[k];
    }
    const int nit = it + (int)gridDim.x;
    const int cnt = item.z - item.y;
    const bool frozen = item.x < P.K && P.steps && P.steps[sid] == 0;
    if (item.x >= P.K || frozen) {  // inactive bucket or frozen scene: carry over unchanged (uniform)
      for (int j = threadIdx.x; j < cnt; j += T) {
        const int64_t si = P.perm[item.y + j];
        for (int k = 0; k < P.nf; ++k) Dx[(int64_t)k * cap + item.y + j] = Sx[(int64_t)k * cap + si];
      }
      nitem = nit < n_items ? P.items[nit] : make_int4(0, 0, 0, 0);
      p2g_item_head(P, nitem, T, nsi, ncell, nsid);
      continue;
    }
    int org[3];
    block_origin(P.scenes[sid], item.x, org);
    if (threadIdx.x == 0) s_scene = P.scenes[sid];  // published by the barrier after step 1
    const SceneDev& S = s_scene;
    // 1. cell ranks (old slot and cell of the first P2G_PF particles per thread were loaded ahead;
    //    the cell comes from the G2P, or re-keying, that keyed the particle)
#pragma unroll
    for (int k = 0; k < P2G_PF; ++k) {
      const int j = (int)threadIdx.x + k * T;
      if (j < cnt) {
        s_si[j] = pf_si[k];
        const int r = atomicAdd(&s_cnt[pf_cell[k]], 1);
        s_cr[j] = ((uint32_t)pf_cell[k] << 16) | (uint32_t)r;
      }
    }
    for (int j = (int)threadIdx.x + P2G_PF * T; j < cnt; j += T) {
      s_si[j] = P.perm[item.y + j];
      const int cell = P.slot_cell[item.y + j];
      const int r = atomicAdd(&s_cnt[cell], 1);
      s_cr[j] = ((uint32_t)cell << 16) | (uint32_t)r;
    }
    __syncthreads();
    // every warp scans the 64 cell counts into registers: lane l holds the start of cells l and
    // l + 32 (no extra barrier; starts are fetched by shuffles, a cell ends where the next starts)
    int offA, offB, tot_in;
    {
      const int a = s_cnt[lane], b = s_cnt[lane + 32];
      int ia = a, ib = b;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int ta = __shfl_up_sync(0xffffffffu, ia, o), tbv = __shfl_up_sync(0xffffffffu, ib, o);
        if (lane >= o) {
          ia += ta;
          ib += tbv;
        }
      }
      const int tot_a = __shfl_sync(0xffffffffu, ia, 31);
      offA = ia - a;
      offB = tot_a + ib - b;
      tot_in = __shfl_sync(0xffffffffu, tot_a + ib, 31);  // start of the particles outside the block's cells
    }
    // 2. material + stress in slot order; scatter parameters to the sorted record (lanes of a warp
    //    iterate together so the offset shuffles see the whole warp)
    for (int jb = threadIdx.x - lane; jb < cnt; jb += T) {
      const int j = jb + lane;
      const uint32_t cr = j < cnt ? s_cr[j] : 0u;
      const int cell = (int)(cr >> 16);
      const int oa = __shfl_sync(0xffffffffu, offA, cell & 31), ob = __shfl_sync(0xffffffffu, offB, cell & 31);
      if (j >= cnt) continue;
      const int p = (cell < 32 ? oa : (cell < BLK_NODES ? ob : tot_in)) + (int)(cr & 0xffffu);
      const int64_t slot = item.y + j;
      const int64_t si = s_si[j];
      Particle pt;
      load_particle(P, Sx, si, pt);
      bool scattered = false;
      uint32_t cmask = 0u;
      if constexpr (CPIC) {
        cmask = cpic_p2g(P, S, sid, pt.x, (pt.info & INFO_ACTIVE) != 0, si, slot, org, cell);
        P.cpic_mask[slot] = cmask;
#pragma unroll
        for (int d = 0; d < 3; ++d) Dx[(int64_t)(PF_VEL + d) * cap + slot] = pt.v[d];  // G2P collides it
      }
      if (pt.info & INFO_ACTIVE) {
        const MaterialDev& M = P.mats[pt.info & INFO_MAT_MASK];
        // F_tmp = (I + dt C) F   (compute_F_tmp, mpm_solver.py:293-299)
        float A[9], Ft[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) A[k] = ((k % 4 == 0) ? 1.f : 0.f) + S.dt * pt.C[k];
        mat_mul(A, pt.F, Ft);
        float Pk[9], Jpn = pt.Jp;
        if (M.type == MT_LIQUID && M.mu == 0.f) {
          // Non-viscous liquid (liquid.py:36-49 with mu = 0) uses only J = sigma0 sigma1 sigma2 of the
          // SVD, which equals det F_tmp (det U = det V = 1): F_new = J^(1/3) I, stress = lam J (J-1) I.
          const float J = Ft[0] * (Ft[4] * Ft[8] - Ft[5] * Ft[7]) - Ft[1] * (Ft[3] * Ft[8] - Ft[5] * Ft[6]) +
                          Ft[2] * (Ft[3] * Ft[7] - Ft[4] * Ft[6]);
          const float j3 = powf(J, 1.f / 3.f);
          const float pr = M.lam * J * (J - 1.f);
#pragma unroll
          for (int k = 0; k < 9; ++k) {
            pt.F[k] = (k % 4 == 0) ? j3 : 0.f;
            Pk[k] = (k % 4 == 0) ? pr : 0.f;
          }
        } else {
          float U[9], sig[3], V[9];
          const float res = svd3<float, SVD_SWEEPS>(Ft, U, sig, V);
          if (!svd_accurate(res, sig, SVD_FP64_TOL)) {
            svd3_fp64(Ft, U, sig, V);
            atomicAdd(P.fp64_count, 1ull);
          }
          material_update<float>(M, Ft, U, sig, V, pt.Jp, pt.actu, pt.mdir, P.eps_norm, pt.F, Jpn, Pk);
        }
        pt.Jp = Jpn;
        if (cell < BLK_NODES) {
          const int tb0 = cell >> 4, tb1 = (cell >> 2) & 3, tb2 = cell & 3;
          const float mass = M.mass;
          float fx[3];
          const int tbv[3] = {tb0, tb1, tb2};
#pragma unroll
          for (int d = 0; d < 3; ++d) fx[d] = __fmul_rn(pt.x[d], S.inv_dx) - (float)(tbv[d] + S.offset[d] + org[d]);
          float a[9];  // a[k*3 + r] = dx * affine[r][k]
#pragma unroll
          for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int k = 0; k < 3; ++k) a[k * 3 + r] = S.dx * (S.stress_scale * Pk[r * 3 + k] + mass * pt.C[r * 3 + k]);
          float qv[3];
#pragma unroll
          for (int r = 0; r < 3; ++r) qv[r] = mass * pt.v[r] - (a[r] * fx[0] + a[3 + r] * fx[1] + a[6 + r] * fx[2]);
          float4* rec = s_rec + P2G_REC * p;  // layout: P2G_REC
          rec[0] = make_float4(qv[0], qv[1], qv[2], mass);
          rec[1] = make_float4(a[0], a[1], a[3], a[4]);
          rec[2] = make_float4(a[6], a[7], a[2], a[5]);
          rec[3] = make_float4(a[8], fx[0], fx[1], fx[2]);
          if constexpr (CPIC) rec[4] = make_float4(__uint_as_float(cmask), 0.f, 0.f, 0.f);
          scattered = true;
          if (!(pt.info & INFO_FREE) && P.pin) {  // its 27 nodes lose all momentum (mpm_solver.py:420-421)
            for (int o = 0; o < 27; ++o) {
              const int64_t ad = node_addr(S, org[0] + tb0 + o / 9, org[1] + tb1 + (o / 3) % 3, org[2] + tb2 + o % 3);
              atomicOr(&P.pin[ad >> 5], 1u << (ad & 31));
            }
          }
        } else {
          atomicOr(P.status, 2u);  // cannot happen for a correctly keyed particle; never touches memory
        }
      }
      if (!scattered && cell < BLK_NODES) {  // holds a place in its cell's run: contributes nothing
        float4* rec = s_rec + P2G_REC * p;
        rec[0] = rec[1] = rec[2] = make_float4(0.f, 0.f, 0.f, 0.f);
        rec[3] = make_float4(0.f, 0.5f, 0.5f, 0.5f);
        if constexpr (CPIC) rec[4] = make_float4(0.f, 0.f, 0.f, 0.f);
      }
      store_particle(P, Dx, slot, pt);
    }
    nitem = nit < n_items ? P.items[nit] : make_int4(0, 0, 0, 0);  // arrives during the barrier wait
    __syncthreads();
    p2g_item_head(P, nitem, T, nsi, ncell, nsid);  // consumed by the next item's step 1
    // 3. cell-major scatter: unit u = (cell, ox) sums the 9 nodes (ox, *, *) of the stencils of
    //    all particles of its cell in registers and adds them to the warp tile once.  A warp's
    //    32 units span fewer than 16 consecutive cells, so no two of its lanes share a node.
    for (int u0 = 0; u0 < 3 * BLK_NODES; u0 += T) {
      const int u = u0 + threadIdx.x;
      const bool has = u < 3 * BLK_NODES;
      const int cell = has ? u / 3 : 0, ox = has ? u - 3 * (u / 3) : 0;
      const int nx = (cell + 1) & 31;
      const int oa = __shfl_sync(0xffffffffu, offA, cell & 31), ob = __shfl_sync(0xffffffffu, offB, cell & 31);
      const int na = __shfl_sync(0xffffffffu, offA, nx), nb = __shfl_sync(0xffffffffu, offB, nx);
      const int beg = cell < 32 ? oa : ob;
      const int end = cell + 1 < 32 ? na : (cell + 1 < BLK_NODES ? nb : tot_in);
      const int len = has ? end - beg : 0;
      const int nmax = __reduce_max_sync(0xffffffffu, len);
      if (nmax == 0) continue;  // warp-uniform
      // node sums in channel pairs (momentum x, y) and (momentum z, mass), accumulated with the
      // paired FP32 operations (__ffma2_rn etc.: each half rounds as fmaf does, so the sums are
      // those of the scalar form, at half the instructions)
      float2 acc01[3][3], acc2m[3][3];
#pragma unroll
      for (int oy = 0; oy < 3; ++oy)
#pragma unroll
        for (int oz = 0; oz < 3; ++oz) acc01[oy][oz] = acc2m[oy][oz] = make_float2(0.f, 0.f);
      const float2 fod = make_float2((float)ox, (float)ox), two = make_float2(2.f, 2.f);
      // the quadratic B-spline weights (mpm_solver.py:381) as polynomials in Horner form,
      // w_o(f) = (p2_o f + p1_o) f + p0_o, each held twice (a pair) for the paired products;
      // this lane's x weight needs only its own o = ox
      const float px2 = ox == 1 ? -1.f : 0.5f, px1 = ox == 0 ? -1.5f : (ox == 1 ? 2.f : -0.5f),
                  px0 = ox == 0 ? 1.125f : (ox == 1 ? -0.25f : 0.125f);
      const float2 px2d = make_float2(px2, px2), px1d = make_float2(px1, px1), px0d = make_float2(px0, px0);
      for (int j = 0; j < nmax; ++j) {
        if (j < len) {
          const float4* rec = s_rec + P2G_REC * (beg + j);
          const float4 r0 = rec[0], r1 = rec[1], r2 = rec[2], r3 = rec[3];
          uint32_t m9 = 0u;  // CPIC: the record's separated nodes of this ox
          if constexpr (CPIC) m9 = __float_as_uint(rec[4].x) >> (9 * ox);
          const float2 fxd = make_float2(r3.y, r3.y), fyd = make_float2(r3.z, r3.z), fzd = make_float2(r3.w, r3.w);
          const float2 wxd = __ffma2_rn(__ffma2_rn(px2d, fxd, px1d), fxd, px0d);
          const float2 wyd[3] = {
              __ffma2_rn(__ffma2_rn(make_float2(0.5f, 0.5f), fyd, make_float2(-1.5f, -1.5f)), fyd,
                         make_float2(1.125f, 1.125f)),
              __ffma2_rn(__ffma2_rn(make_float2(-1.f, -1.f), fyd, make_float2(2.f, 2.f)), fyd,
                         make_float2(-0.25f, -0.25f)),
              __ffma2_rn(__ffma2_rn(make_float2(0.5f, 0.5f), fyd, make_float2(-0.5f, -0.5f)), fyd,
                         make_float2(0.125f, 0.125f))};
          const float2 wzd[3] = {
              __ffma2_rn(__ffma2_rn(make_float2(0.5f, 0.5f), fzd, make_float2(-1.5f, -1.5f)), fzd,
                         make_float2(1.125f, 1.125f)),
              __ffma2_rn(__ffma2_rn(make_float2(-1.f, -1.f), fzd, make_float2(2.f, 2.f)), fzd,
                         make_float2(-0.25f, -0.25f)),
              __ffma2_rn(__ffma2_rn(make_float2(0.5f, 0.5f), fzd, make_float2(-0.5f, -0.5f)), fzd,
                         make_float2(0.125f, 0.125f))};
          // node value (q + ox a_x + oy a_y + oz a_z, m): the offsets 0, 1, 2 spelled out (without
          // fast math a product by 0 or 1 is not folded away); the mass half takes a zero step
          const float2 ax01 = make_float2(r1.x, r1.y), ay01 = make_float2(r1.z, r1.w), az01 = make_float2(r2.x, r2.y);
          const float2 ax2z = make_float2(r2.z, 0.f), ay2z = make_float2(r2.w, 0.f), az2z = make_float2(r3.x, 0.f);
          const float2 s01 = __ffma2_rn(fod, ax01, make_float2(r0.x, r0.y));
          const float2 s2m = __ffma2_rn(fod, ax2z, make_float2(r0.z, r0.w));
#pragma unroll
          for (int oy = 0; oy < 3; ++oy) {
            const float2 u01 = oy == 0 ? s01 : (oy == 1 ? __fadd2_rn(s01, ay01) : __ffma2_rn(two, ay01, s01));
            const float2 u2m = oy == 0 ? s2m : (oy == 1 ? __fadd2_rn(s2m, ay2z) : __ffma2_rn(two, ay2z, s2m));
            const float2 w01 = __fmul2_rn(wxd, wyd[oy]);
#pragma unroll
            for (int oz = 0; oz < 3; ++oz) {
              const float2 v01 = oz == 0 ? u01 : (oz == 1 ? __fadd2_rn(u01, az01) : __ffma2_rn(two, az01, u01));
              const float2 v2m = oz == 0 ? u2m : (oz == 1 ? __fadd2_rn(u2m, az2z) : __ffma2_rn(two, az2z, u2m));
              float2 wt = __fmul2_rn(w01, wzd[oz]);
              if constexpr (CPIC) {
                if ((m9 >> (oy * 3 + oz)) & 1u) wt = make_float2(0.f, 0.f);
              }
              acc01[oy][oz] = __ffma2_rn(wt, v01, acc01[oy][oz]);
              acc2m[oy][oz] = __ffma2_rn(wt, v2m, acc2m[oy][oz]);
            }
          }
        }
      }
      // Lanes of neighbouring cells reach the same node at different (oy, oz) steps: a
      // __syncwarp between steps orders those read-modify-writes.
      const int tb0 = cell >> 4, tb1 = (cell >> 2) & 3, tb2 = cell & 3;
#pragma unroll
      for (int oy = 0; oy < 3; ++oy)
#pragma unroll
        for (int oz = 0; oz < 3; ++oz) {
          if (len > 0) {
            float4* g = my_tile + ((tb0 + ox) * TILE + (tb1 + oy)) * TILE + (tb2 + oz);
            float4 h = *g;
            h.x += acc01[oy][oz].x;
            h.y += acc01[oy][oz].y;
            h.z += acc2m[oy][oz].x;
            h.w += acc2m[oy][oz].y;
            *g = h;
          }
          __syncwarp();
        }
    }
    __syncthreads();
    // 4. flush
    if (threadIdx.x <= BLK_NODES) s_cnt[threadIdx.x] = 0;  // every warp's scan read it before phase 2 ended
    for (int t = threadIdx.x; t < TILE_NODES; t += T) {
      float4 g = s_tile[t];
      s_tile[t] = make_float4(0.f, 0.f, 0.f, 0.f);
      for (int ww = 1; ww < nw; ++ww) {
        const float4 h = s_tile[ww * TILE_NODES + t];
        s_tile[ww * TILE_NODES + t] = make_float4(0.f, 0.f, 0.f, 0.f);
        g.x += h.x;
        g.y += h.y;
        g.z += h.z;
        g.w += h.w;
      }
      if (g.w == 0.f) continue;
      const int tx = t / (TILE * TILE), ty = (t / TILE) % TILE, tz = t % TILE;
      const int gx = org[0] + tx, gy = org[1] + ty, gz = org[2] + tz;
      if (gx >= S.res[0] || gy >= S.res[1] || gz >= S.res[2]) continue;
      atomicAdd(reinterpret_cast<float4*>(&P.grid[node_addr(S, gx, gy, gz)]), g);
      s_touch[(tx >> 2) * 4 + (ty >> 2) * 2 + (tz >> 2)] = 1;
    }
    // what the block flags need of the scene, read before the barrier (the next item's thread 0
    // rewrites s_scene after it)
    const int bres0 = S.bres[0], bres1 = S.bres[1], bres2 = S.bres[2];
    const int64_t bbase = S.block_base;
    __syncthreads();
    if (threadIdx.x < 8 && s_touch[threadIdx.x]) {
      s_touch[threadIdx.x] = 0;
      const int bx = org[0] / BLK + (threadIdx.x >> 2), by = org[1] / BLK + ((threadIdx.x >> 1) & 1),
                bz = org[2] / BLK + (threadIdx.x & 1);
      if (bx < bres0 && by < bres1 && bz < bres2) {
        const int64_t blk = bbase + ((int64_t)bx * bres1 + by) * bres2 + bz;
        if (atomicExch(&P.flags[blk], 1) == 0) P.list[atomicAdd(P.nlist, 1)] = (int32_t)blk;
      }
    }
  }
  pdl_trigger();
}

// Capped at 96 registers: five 128-thread CTAs per SM instead of four at 128 registers, which
// measured 5% faster despite a small spill.
__global__ void __maxnreg__(96) k_p2g(KParams P) { p2g_body<false>(P); }
__global__ void __launch_bounds__(P2G_MAX_THREADS) k_p2g_cpic(KParams P) { p2g_body<true>(P); }

// ------------------------------------------------------------------ G2P
// mpm_solver.py:423-481 (g2p) with the particle boundary of boundaries.py:22-32, over the
// same work items as the P2G that wrote the particles (so every item's particles read one
// 6^3 node tile, staged once in shared memory), followed by the bucket key of the new
// position and a warp-aggregated rank within the bucket.
__device__ __forceinline__ void add_rank(const KParams& P, bool valid, int32_t key, int64_t i, int lane, int cell) {
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
    P.cell8[i] = (uint8_t)cell;
  }
}

template <bool CPIC>
__device__ __forceinline__ void g2p_body(const KParams& P) {
  __shared__ float4 s_v[TILE_NODES];
  __shared__ SceneDev s_scene;  // the item's scene record (see p2g_body)
  pdl_wait();
  if (P.fuse_grid) {
    // the grid op's other duty: zero the blocks the previous substep left in the other buffer
    // (the next P2G adds into it); k_perm resets that list's length after this kernel
    const int64_t n_other = (int64_t)*P.nlist_other * BLK_NODES;
    for (int64_t i = grid_stride_begin(); i < n_other; i += grid_stride_step()) {
      const int32_t blk = P.list_other[i / BLK_NODES];
      P.grid_other[(int64_t)blk * BLK_NODES + (i % BLK_NODES)] = make_float4(0.f, 0.f, 0.f, 0.f);
      if (i % BLK_NODES == 0) P.flags_other[blk] = 0;
    }
  } else if (blockIdx.x == 0 && threadIdx.x == 0) {
    *P.nlist_other = 0;
  }
  const int n_items = *P.n_items;
  const int T = blockDim.x, lane = threadIdx.x & 31;
  const int64_t cap = P.cap;
  float* D = P.dst;
  const int32_t kInactive = (int32_t)P.K, kDead = (int32_t)P.K + 1;
  for (int it = blockIdx.x; it < n_items; it += gridDim.x) {
    const int4 item = P.items[it];
    const int cnt = item.z - item.y;
    const int total = (cnt + 31) & ~31;
    const bool frozen = item.x < P.K && P.steps && P.steps[P.block_scene[item.x]] == 0;
    if (item.x >= P.K || frozen) {  // inactive bucket or frozen scene: keys only (uniform branch)
      for (int q = threadIdx.x; q < total; q += T) {
        const bool valid = q < cnt;
        const int64_t i = item.y + q;
        int32_t key = kInactive;
        int cellk = BLK_NODES;
        if (valid) {
          const uint32_t info = ld_info(D, cap, i);
          if (info & INFO_DEAD) key = kDead;
          else if (info & INFO_ACTIVE) {
            const SceneDev& Sc = P.scenes[scene_of(P, info)];
            float x[3];
            int b[3];
            for (int d = 0; d < 3; ++d) x[d] = D[(int64_t)(PF_POS + d) * cap + i];
            if (stencil_origin(Sc, x, b)) {
              key = (int32_t)block_of(Sc, b[0], b[1], b[2]);
              cellk = ((b[0] & 3) * 4 + (b[1] & 3)) * 4 + (b[2] & 3);
            }
          }
        }
        add_rank(P, valid, key, i, lane, cellk);
      }
      continue;
    }
    const SceneDev& Sg = P.scenes[P.block_scene[item.x]];
    if (threadIdx.x == 0) s_scene = Sg;  // published by the barrier after the staging
    int org[3];
    block_origin(Sg, item.x, org);
    // positions are software-pipelined one particle ahead; the first load overlaps the staging
    float xn[3] = {0.f, 0.f, 0.f};
    if ((int)threadIdx.x < cnt) {
#pragma unroll
      for (int d = 0; d < 3; ++d) xn[d] = D[(int64_t)(PF_POS + d) * cap + item.y + threadIdx.x];
    }
    for (int t = threadIdx.x; t < TILE_NODES; t += T) {
      const int gx = org[0] + t / (TILE * TILE), gy = org[1] + (t / TILE) % TILE, gz = org[2] + t % TILE;
      float4 g = make_float4(0.f, 0.f, 0.f, 0.f);
      if (gx < Sg.res[0] && gy < Sg.res[1] && gz < Sg.res[2]) {
        g = P.grid[node_addr(Sg, gx, gy, gz)];
        if (P.fuse_grid) g = grid_velocity(Sg, g, gx, gy, gz);
      }
      s_v[t] = g;
    }
    __syncthreads();
    const SceneDev& S = s_scene;
    for (int q = threadIdx.x; q < total; q += T) {
      const bool valid = q < cnt;
      const int64_t i = item.y + q;
      int32_t key = kInactive;
      int cellk = BLK_NODES;
      float x[3] = {xn[0], xn[1], xn[2]};
      if (q + T < cnt) {
#pragma unroll
        for (int d = 0; d < 3; ++d) xn[d] = D[(int64_t)(PF_POS + d) * cap + i + T];
      }
      if (valid) {
        int tb[3];
        const int cell = local_cell(S, x, org, tb);
        if (cell < BLK_NODES) {
          float fx[3], w[3][3];
#pragma unroll
          for (int d = 0; d < 3; ++d) {
            const float t = __fmul_rn(x[d], S.inv_dx);
            fx[d] = t - (float)(tb[d] + S.offset[d] + org[d]);
            bspline_w(fx[d], w[d]);
          }
          // v = sum w v_i;  C = 4 inv_dx sum w v_i (o - fx)^T = 4 inv_dx (M - v fx^T), M = sum w v_i o^T,
          // accumulated along the separable stencil (z innermost)
          uint32_t cm = 0u;  // CPIC: nodes behind a collider, from this substep's P2G
          if constexpr (CPIC) cm = P.cpic_mask[i];
          float v[3] = {0.f, 0.f, 0.f}, M[9];
#pragma unroll
          for (int k = 0; k < 9; ++k) M[k] = 0.f;
#pragma unroll
          for (int ox = 0; ox < 3; ++ox)
#pragma unroll
            for (int oy = 0; oy < 3; ++oy) {
              float a[3] = {0.f, 0.f, 0.f}, bz[3] = {0.f, 0.f, 0.f};
#pragma unroll
              for (int oz = 0; oz < 3; ++oz) {
                float4 g = s_v[((tb[0] + ox) * TILE + (tb[1] + oy)) * TILE + (tb[2] + oz)];
                if constexpr (CPIC) {
                  if ((cm >> (ox * 9 + oy * 3 + oz)) & 1u)
                    g = cpic_g2p_node(P, S, P.block_scene[item.x], D, i, x, org, tb, ox * 9 + oy * 3 + oz,
                                      w[0][ox] * w[1][oy] * w[2][oz], g);
                }
                const float wz = w[2][oz];
                a[0] += wz * g.x;
                a[1] += wz * g.y;
                a[2] += wz * g.z;
                if (oz > 0) {
                  const float wo = wz * (float)oz;
                  bz[0] += wo * g.x;
                  bz[1] += wo * g.y;
                  bz[2] += wo * g.z;
                }
              }
              const float wxy = w[0][ox] * w[1][oy];
#pragma unroll
              for (int r = 0; r < 3; ++r) {  // offsets 0 spelled out: a product by 0 is not folded away
                const float t = wxy * a[r];
                v[r] += t;
                if (ox > 0) M[r * 3 + 0] = fmaf((float)ox, t, M[r * 3 + 0]);
                if (oy > 0) M[r * 3 + 1] = fmaf((float)oy, t, M[r * 3 + 1]);
                M[r * 3 + 2] = fmaf(wxy, bz[r], M[r * 3 + 2]);
              }
            }
          float Cn[9];
#pragma unroll
          for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int c = 0; c < 3; ++c) Cn[r * 3 + c] = 4.f * S.inv_dx * (M[r * 3 + c] - v[r] * fx[c]);
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
          int b[3];
          if (!finite) atomicOr(P.status, 1u);
          else if (stencil_origin(S, xn, b)) {
            key = (int32_t)block_of(S, b[0], b[1], b[2]);
            cellk = ((b[0] & 3) * 4 + (b[1] & 3)) * 4 + (b[2] & 3);
          } else {
            atomicOr(P.status, 2u);
          }
        } else {
          atomicOr(P.status, 2u);
        }
      }
      add_rank(P, valid, key, i, lane, cellk);
    }
    __syncthreads();
  }
  pdl_trigger();
}

__global__ void __launch_bounds__(256) k_g2p(KParams P) { g2p_body<false>(P); }
__global__ void __launch_bounds__(256) k_g2p_cpic(KParams P) { g2p_body<true>(P); }

// ------------------------------------------------------------------ grid op
// legacy_coupler.py:356-501 without coupling partners: for nodes with mass > eps,
// v = (1/m) p + dt g, then CubeBoundary.impose_pos_vel at the node position; 0 otherwise.
// Also clears the other grid buffer's blocks touched in the previous substep.
// Staged (KParams::grid_stage > 0) for callers that act on the node velocities between the
// built-in force fields and the rest of the grid op (Custom force fields): stage 1 turns momentum
// into velocity and applies fields [ff_begin, ff_end), stage 2 applies more fields to the
// velocities, stage 3 applies colliders, coupled particle sets and the boundary.
__global__ void __launch_bounds__(256) k_grid_op(KParams P) {
  const int sub = threadIdx.x >> 6, ln = threadIdx.x & 63;
  const int per_iter = (int)gridDim.x * (blockDim.x >> 6);
  const int stage = P.grid_stage;
  if (stage <= 1) {
    const int n_other = *P.nlist_other;
    for (int i = blockIdx.x * (blockDim.x >> 6) + sub; i < n_other; i += per_iter) {
      const int32_t blk = P.list_other[i];
      P.grid_other[(int64_t)blk * BLK_NODES + ln] = make_float4(0.f, 0.f, 0.f, 0.f);
      if (ln == 0) P.flags_other[blk] = 0;
    }
  }
  const int n_cur = *P.nlist;
  const unsigned long long step = P.ff_step ? *P.ff_step : 0ull;
  for (int i = blockIdx.x * (blockDim.x >> 6) + sub; i < n_cur; i += per_iter) {
    const int32_t blk = P.list[i];
    const SceneDev& S = P.scenes[P.block_scene[blk]];
    const int64_t lb = (int64_t)blk - S.block_base;
    const int bz = (int)(lb % S.bres[2]), by = (int)((lb / S.bres[2]) % S.bres[1]),
              bx = (int)(lb / ((int64_t)S.bres[2] * S.bres[1]));
    const int g[3] = {bx * BLK + (ln >> 4), by * BLK + ((ln >> 2) & 3), bz * BLK + (ln & 3)};
    float4* node = &P.grid[(int64_t)blk * BLK_NODES + ln];
    float4 q = *node;
    if (stage <= 1 && P.pin) {  // nodes touched by a non-free particle keep no momentum (mpm_solver.py:420-421)
      const int64_t a = (int64_t)blk * BLK_NODES + ln;
      const uint32_t bit = 1u << (a & 31);
      if (P.pin[a >> 5] & bit) {
        q.x = q.y = q.z = 0.f;
        atomicAnd(&P.pin[a >> 5], ~bit);
      }
    }
    if (stage == 0 && P.n_colliders == 0 && P.n_ffs == 0 && P.ext[0].n == 0 && P.ext[1].n == 0) {
      *node = grid_velocity(S, q, g[0], g[1], g[2]);
    } else {  // gravity, force fields (:381-383), colliders (:389-403), SPH / PBD (:404-498), boundary
      float v[3] = {0.f, 0.f, 0.f};
      bool has;
      if (stage <= 1) {
        has = grid_free_velocity(S, q, v);
      } else {  // the node already holds its velocity
        has = q.w > S.eps;
        if (has) v[0] = q.x, v[1] = q.y, v[2] = q.z;
      }
      if (has) {
        const float x[3] = {(float)(g[0] + S.offset[0]) * S.dx, (float)(g[1] + S.offset[1]) * S.dx,
                            (float)(g[2] + S.offset[2]) * S.dx};
        if (stage != 3) {
          for (int fi = P.ff_begin; fi < P.ff_end; ++fi) {
            if (!P.ffs[fi].active) continue;
            float a[3];
            const int gw[3] = {g[0] + S.offset[0], g[1] + S.offset[1], g[2] + S.offset[2]};
            ff_acc(P.ffs[fi], x, v, S.eps, a, P.block_scene[blk], gw, step);
            for (int k = 0; k < 3; ++k) v[k] += a[k] * S.dt;
          }
        }
        if (stage == 0 || stage == 3) {
          collide_node(P, S, P.block_scene[blk], x, v, q.w / 1e3f);
          couple_ext(P, (int64_t)blk * BLK_NODES + ln, v, q.w / 1e3f);
          grid_boundary(S, v, g[0], g[1], g[2]);
        }
      }
      *node = make_float4(v[0], v[1], v[2], q.w);
    }
  }
}

// World position of every node of the grid buffer ([K * 64][3], block-major like the grid) and
// its scene (-1 for the padding of a block past the scene's grid).
__global__ void k_node_positions(KParams P, float* pos, int32_t* scene) {
  const int64_t total = P.K * BLK_NODES;
  for (int64_t i = grid_stride_begin(); i < total; i += grid_stride_step()) {
    const int64_t blk = i / BLK_NODES;
    const int ln = (int)(i % BLK_NODES);
    const int32_t sid = P.block_scene[blk];
    const SceneDev& S = P.scenes[sid];
    const int64_t lb = blk - S.block_base;
    const int bz = (int)(lb % S.bres[2]), by = (int)((lb / S.bres[2]) % S.bres[1]),
              bx = (int)(lb / ((int64_t)S.bres[2] * S.bres[1]));
    const int g[3] = {bx * BLK + (ln >> 4), by * BLK + ((ln >> 2) & 3), bz * BLK + (ln & 3)};
    const bool in = g[0] < S.res[0] && g[1] < S.res[1] && g[2] < S.res[2];
#pragma unroll
    for (int d = 0; d < 3; ++d) pos[i * 3 + d] = (float)(g[d] + S.offset[d]) * S.dx;
    if (scene) scene[i] = in ? sid : -1;
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
    float4 q = P.grid[node_addr(S, gx, gy, gz)];
    if (P.fuse_grid) q = grid_velocity(S, q, gx, gy, gz);  // the buffer holds P2G momentum
    out[i * 4 + 0] = q.x;
    out[i * 4 + 1] = q.y;
    out[i * 4 + 2] = q.z;
    out[i * 4 + 3] = q.w;
  }
}

// ------------------------------------------------------------------ particle constraints
namespace {
// gu.qd_transform_by_quat (utils/geom.py:256-271) for q = (w, x, y, z), unnormalised as there.
__device__ __forceinline__ void quat_rotate(const float* q, const float* v, float* o) {
  const float w = q[0], x = q[1], y = q[2], z = q[3];
  const float xx = x * x, xy = x * y, xz = x * z, wx = x * w, yy = y * y, yz = y * z, wy = y * w, zz = z * z,
              wz = z * w, ww = w * w;
  o[0] = v[0] * (xx + ww - yy - zz) + v[1] * (2.f * xy - 2.f * wz) + v[2] * (2.f * xz + 2.f * wy);
  o[1] = v[0] * (2.f * wz + 2.f * xy) + v[1] * (ww - xx + yy - zz) + v[2] * (-2.f * wx + 2.f * yz);
  o[2] = v[0] * (-2.f * wy + 2.f * xz) + v[1] * (2.f * wx + 2.f * yz) + v[2] * (ww - xx - yy + zz);
}

// Reference row of a particle slot of scenes [s0, s1) that lies in [start, start + n) of its
// scene, or -1.
__device__ __forceinline__ int64_t masked_local(const KParams& P, int64_t i, int64_t s0, int64_t s1, int64_t start,
                                                int64_t n, int32_t& s, uint32_t& pid) {
  const uint32_t info = ld_info(P.dst, P.cap, i);
  if (info & INFO_DEAD) return -1;
  s = scene_of(P, info);
  if (s < s0 || s >= s1) return -1;
  pid = __float_as_uint(P.dst[(int64_t)PF_PID * P.cap + i]);
  const int64_t l = (int64_t)pid - start;
  return (l >= 0 && l < n) ? l : -1;
}
}  // namespace

// _kernel_set_particle_constraints (mpm_solver.py:1052-1084): the target is the particle's
// current position; its offset in the link frame is kept for later link poses.
__global__ void k_set_constraints(KParams P, int64_t s0, int64_t s1, int64_t start, int64_t n, const uint8_t* mask,
                                  float stiffness, int32_t link, const float* link_pos, const float* link_quat,
                                  ConstraintDev* cons) {
  for (int64_t i = grid_stride_begin(); i < P.n; i += grid_stride_step()) {
    int32_t s;
    uint32_t pid;
    const int64_t l = masked_local(P, i, s0, s1, start, n, s, pid);
    if (l < 0 || !mask[(s - s0) * n + l]) continue;
    float x[3], d[3], loc[3];
    const float* lp = link_pos + (s - s0) * 3;
    const float* lq = link_quat + (s - s0) * 4;
    for (int k = 0; k < 3; ++k) {
      x[k] = P.dst[(int64_t)(PF_POS + k) * P.cap + i];
      d[k] = x[k] - lp[k];
    }
    const float qi[4] = {lq[0], -lq[1], -lq[2], -lq[3]};
    quat_rotate(qi, d, loc);
    ConstraintDev& c = cons[P.scenes[s].p_begin + pid];
    for (int k = 0; k < 3; ++k) {
      c.local[k] = loc[k];
      c.target[k] = x[k];
    }
    c.stiffness = stiffness;
    c.link = link;
    c.on = 1;
  }
}

// _kernel_remove_particle_constraints (mpm_solver.py:1086-1097)
__global__ void k_remove_constraints(KParams P, int64_t s0, int64_t s1, int64_t start, int64_t n,
                                     const uint8_t* mask, ConstraintDev* cons) {
  for (int64_t i = grid_stride_begin(); i < P.n; i += grid_stride_step()) {
    int32_t s;
    uint32_t pid;
    const int64_t l = masked_local(P, i, s0, s1, start, n, s, pid);
    if (l < 0 || !mask[(s - s0) * n + l]) continue;
    ConstraintDev& c = cons[P.scenes[s].p_begin + pid];
    c.on = 0;
    c.link = -1;
  }
}

// apply_particle_constraints (mpm_solver.py:1099-1128), after G2P: the target follows its link's
// pose; a critically damped spring changes the velocity,
// dv = dt (-k (x - target) - 2 sqrt(k m) v) / m with m the particle's real mass.
__global__ void k_constraints(KParams P, ConstraintDev* cons, const float* links, int32_t n_links) {
  const int64_t n = P.n_dev ? *P.n_dev : P.n;
  for (int64_t i = grid_stride_begin(); i < n; i += grid_stride_step()) {
    const uint32_t info = ld_info(P.dst, P.cap, i);
    if (info & INFO_DEAD) continue;
    const MaterialDev& M = P.mats[info & INFO_MAT_MASK];
    const int32_t s = M.scene;
    if (P.steps && P.steps[s] == 0) continue;  // frozen scene
    const uint32_t pid = __float_as_uint(P.dst[(int64_t)PF_PID * P.cap + i]);
    ConstraintDev& c = cons[P.scenes[s].p_begin + pid];
    if (!c.on) continue;
    if (c.link >= 0 && c.link < n_links) {
      const float* L = links + ((int64_t)s * n_links + c.link) * 7;
      float t[3];
      quat_rotate(L + 3, c.local, t);
      for (int k = 0; k < 3; ++k) c.target[k] = t[k] + L[k];
    }
    const float m = M.mass / 1e3f;  // particles_info.mass / particle_volume_scale
    const float k = c.stiffness;
    const float damp = 2.f * sqrtf(k * m);
    for (int d = 0; d < 3; ++d) {
      const float x = P.dst[(int64_t)(PF_POS + d) * P.cap + i];
      float& v = P.dst[(int64_t)(PF_VEL + d) * P.cap + i];
      const float f = -k * (x - c.target[d]) - damp * v;
      v = v + P.scenes[s].dt * f / m;
    }
  }
}

// ------------------------------------------------------------------ lattice sampling
namespace {
// np.linspace(lo, hi, n)[i]: i * step + lo, the last point exactly hi.
__device__ __forceinline__ double lattice_coord(const LatticeDev& L, int d, int64_t i) {
  return (L.n[d] > 1 && i == L.n[d] - 1) ? L.hi[d] : (double)i * L.step[d] + L.lo[d];
}

// The reference's rejection tests (particle.py:249-250, 273-274): numpy norm in float64.
__device__ __forceinline__ bool lattice_keep(const LatticeDev& L, double x, double y, double z) {
  if (L.shape == 0) return true;
  const double dx = x - L.center[0], dy = y - L.center[1];
  if (L.shape == 2) return sqrt(dx * dx + dy * dy) <= L.radius;
  const double dz = z - L.center[2];
  return sqrt(dx * dx + dy * dy + dz * dz) <= L.radius;
}
}  // namespace

// Kept points of each (ix, iy) row of the lattice.
__global__ void k_lattice_rows(LatticeDev L, int64_t* row_count) {
  const int64_t rows = L.n[0] * L.n[1];
  for (int64_t r = grid_stride_begin(); r < rows; r += grid_stride_step()) {
    const double x = lattice_coord(L, 0, r / L.n[1]), y = lattice_coord(L, 1, r % L.n[1]);
    int64_t c = 0;
    for (int64_t iz = 0; iz < L.n[2]; ++iz) c += lattice_keep(L, x, y, lattice_coord(L, 2, iz)) ? 1 : 0;
    row_count[r] = c;
  }
}

// Kept points in row-major (ix, iy, iz) order, as np.meshgrid(..., indexing='ij').reshape(-1, 3)
// followed by the boolean mask; row_offset is the exclusive scan of k_lattice_rows.
__global__ void k_lattice_fill(LatticeDev L, const int64_t* row_offset, float* out) {
  const int64_t rows = L.n[0] * L.n[1];
  for (int64_t r = grid_stride_begin(); r < rows; r += grid_stride_step()) {
    const double x = lattice_coord(L, 0, r / L.n[1]), y = lattice_coord(L, 1, r % L.n[1]);
    int64_t o = row_offset[r];
    for (int64_t iz = 0; iz < L.n[2]; ++iz) {
      const double z = lattice_coord(L, 2, iz);
      if (!lattice_keep(L, x, y, z)) continue;
      out[o * 3 + 0] = (float)x;
      out[o * 3 + 1] = (float)y;
      out[o * 3 + 2] = (float)z;
      ++o;
    }
  }
}

// Visual vertices of _kernel_update_render_fields (mpm_solver.py:795-803): support-weighted sum
// of the particles' positions (`pos` holds the rows of scenes [s0, s1) in get_state order).
__global__ void k_render_vverts(KParams P, int64_t s0, int64_t s1, const float* pos, const uint8_t* active,
                                int64_t n_vverts, int32_t n_supports, const int32_t* support_idx,
                                const float* support_w, float* vpos, uint8_t* vactive) {
  const int64_t total = (s1 - s0) * n_vverts;
  for (int64_t i = grid_stride_begin(); i < total; i += grid_stride_step()) {
    const int64_t b = i / n_vverts, v = i % n_vverts;
    const SceneDev& S = P.scenes[s0 + b];
    const int64_t base = S.p_begin - P.scenes[s0].p_begin, n_s = S.n_particles;
    float acc[3] = {0.f, 0.f, 0.f};
    for (int j = 0; j < n_supports; ++j) {
      const int64_t k = support_idx[v * n_supports + j];
      if (k < 0 || k >= n_s) {
        atomicOr(P.status, MPM_STATUS_BAD_INDEX);
        continue;
      }
      const float w = support_w[v * n_supports + j];
#pragma unroll
      for (int d = 0; d < 3; ++d) acc[d] += pos[(base + k) * 3 + d] * w;
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) vpos[i * 3 + d] = acc[d];
    const int64_t k0 = n_supports > 0 ? support_idx[v * n_supports] : -1;
    if (vactive) vactive[i] = (k0 >= 0 && k0 < n_s) ? active[base + k0] : 0;
  }
}

// particles_render.pos of an inactive particle is gu.qd_nowhere() (utils/geom.py:355-357).
__global__ void k_render_nowhere(int64_t rows, const uint8_t* active, float* pos) {
  for (int64_t r = grid_stride_begin(); r < rows; r += grid_stride_step()) {
    if (active[r]) continue;
    pos[r * 3 + 0] = -2333333.f;
    pos[r * 3 + 1] = -6666666.f;
    pos[r * 3 + 2] = -5201314.f;
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

// Sets n floats of one particle plane to v (planes added to a live context).
__global__ void k_fill_plane(float* p, int64_t n, float v) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) p[i] = v;
}

// Bins coupled set k by grid node before the grid op (unbin = 0) and empties those lists after it
// (unbin = 1).  A particle belongs to the node whose cell holds it, |x_node - p|_inf < dx / 2
// (legacy_coupler.py:417-420); only the nearest node can pass that test, so it alone is tried.
__global__ void k_ext_bin(KParams P, int k, int unbin) {
  const ExtSetDev& E = P.ext[k];
  const int64_t total = E.n * (int64_t)P.n_scenes;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    if (unbin) {
      const int64_t a = E.node[i];
      if (a >= 0) E.head[a] = -1;
      continue;
    }
    const SceneDev& S = P.scenes[i / E.n];
    int g[3];
    bool ok = true;
    for (int d = 0; d < 3 && ok; ++d) {
      const float p = E.pos[i * 3 + d];
      const float t = floorf(__fadd_rn(__fmul_rn(p, S.inv_dx), 0.5f));
      if (!(t > -1e9f && t < 1e9f)) {
        ok = false;
        break;
      }
      const int gi = (int)t;
      ok = fabsf(__fsub_rn(__fmul_rn((float)gi, S.dx), p)) < __fmul_rn(0.5f, S.dx);
      g[d] = gi - S.offset[d];
      ok = ok && g[d] >= 0 && g[d] < S.res[d];
    }
    int64_t a = -1;
    if (ok) {
      a = node_addr(S, g[0], g[1], g[2]);
      E.next[i] = atomicExch(&E.head[a], (int32_t)i);
    }
    E.node[i] = a;
  }
}

}  // namespace gbmpm
