// mpm_capi.cu - host runtime of libgbmpm.so: context (device memory pool, scene and
// material tables), launch sequencing, CUDA-graph capture of the substep loop, per-kernel
// event timing, and the extern "C" entry points declared in include/gbmpm.h.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "gbmpm.h"
#include "mpm_kernels.cuh"

using namespace gbmpm;

namespace {
std::mutex g_err_mu;
std::string g_create_err;

// Kernel groups timed in profiling mode.
enum { KT_P2G = 0, KT_GRID = 1, KT_G2P = 2, KT_SCAN = 3, KT_PERM = 4, KT_N = 5 };

struct TimedPair {
  int kind;
  cudaEvent_t a, b;
};
}  // namespace

struct mpm_ctx {
  int device = 0;
  int n_sm = 1;
  std::string err;

  // tables
  int64_t n_scenes = 0, n_mats = 0;
  std::vector<SceneDev> scenes_h;
  std::vector<MaterialDev> mats_h;
  std::vector<int64_t> pbegin_h;
  std::vector<int32_t> first_mat_h;
  std::vector<int32_t> mat_count_h;
  int64_t cap = 0, n = 0, K = 0;
  int64_t n_phys = 0;  // extent of the current particle buffer (> n after a retire, until the next substep)
  int nf = NF_BASE;
  // pool mode (serving): slots configured and retired at run time
  bool pool = false;
  int64_t max_blocks = 0;
  int32_t max_mats = 0;
  std::vector<int64_t> slot_n;
  std::vector<char> slot_live;
  float eps_norm = 1.1920929e-7f;

  // device memory
  SceneDev* d_scenes = nullptr;
  MaterialDev* d_mats = nullptr;
  int32_t* d_block_scene = nullptr;
  int64_t* d_pbegin = nullptr;
  int32_t* d_first_mat = nullptr;
  float* d_pbuf[2] = {nullptr, nullptr};
  float4* d_grid[2] = {nullptr, nullptr};
  int32_t* d_flags[2] = {nullptr, nullptr};
  int32_t* d_list[2] = {nullptr, nullptr};
  int32_t* d_nlist = nullptr;  // [2]
  int32_t* d_key = nullptr;
  int32_t* d_rank = nullptr;
  int32_t* d_count = nullptr;
  int32_t* d_offset = nullptr;
  int32_t* d_perm = nullptr;
  uint8_t* d_cell8 = nullptr;
  uint8_t* d_slot_cell = nullptr;
  int4* d_items = nullptr;
  int32_t* d_nitems = nullptr;
  int2* d_partials = nullptr;
  int2* d_scan_tiles = nullptr;                // one-pass scan: bucket range of each live tile
  int32_t* d_n_scan_tiles = nullptr;           // live tile count
  unsigned long long* d_scan_state = nullptr;  // one-pass scan: per-tile (flag, count, items) words
  int32_t* d_scan_sync = nullptr;              // one-pass scan: tile ticket, finished tiles
  uint32_t* d_status = nullptr;
  unsigned long long* d_fp64 = nullptr;
  unsigned long long* d_tmp64 = nullptr;
  uint32_t* d_pin = nullptr;
  ConstraintDev* d_cons = nullptr;  // particle constraints by reference row (allocated on first use)
  ForceFieldDev* d_ffs = nullptr;      // force fields (capacity MAX_FORCE_FIELDS once allocated)
  unsigned long long* d_ff_step = nullptr;  // substeps since the force fields were set
  int32_t n_ffs = 0;
  ColliderDev* d_colliders = nullptr;  // kinematic colliders (capacity MAX_COLLIDERS once allocated)
  double* d_collider_acc = nullptr;    // [MAX_COLLIDERS][6]
  int32_t n_colliders = 0;
  int32_t n_tools = 0;               // MPM_COLLIDER_TOOL colliders among them (k_perm moves them)
  struct SdfGrid {                   // voxel SDF grids of MPM_COLLIDER_SDF / MPM_COLLIDER_TOOL colliders
    float* val = nullptr;
    float* grad = nullptr;
    int32_t res[3] = {0, 0, 0};
    double T[16] = {};
    double cell_size = 0, sdf_max = 0;
  };
  std::vector<SdfGrid> sdf_grids;
  int32_t cpic_slots = 0;            // CPIC collider slots (normal planes); 0: CPIC off
  uint32_t* d_cpic_mask = nullptr;   // CPIC: per particle slot, the stencil nodes behind a collider
  ExtSetDev ext[2] = {};             // coupled SPH / PBD particle sets (caller-owned arrays, own bins)
  int64_t ext_cap[2] = {0, 0};       // particles the bin arrays of each set hold
  float* d_links = nullptr;         // kinematic link poses [scene][link] (pos xyz, quat wxyz)
  int32_t n_links = 0;
  int32_t* d_steps = nullptr;
  int64_t* d_n = nullptr;  // live particle count, read by k_perm inside captured substeps
  int64_t max_items = 0;
  int n_tiles = 0;
  std::vector<void*> allocs;

  // state machine
  int cur = 0;          // particle buffer holding the current state; grid parity of the next P2G
  bool sorted = false;  // perm/items valid for pbuf[cur]
  int phase = 0;        // 0 ready, 1 after P2G, 2 after grid op, 3 inside a staged grid op

  // tuning / launch
  // defaults: the fastest shape on the ~1M-particle plain scene and on the served pool (measured)
  int p2g_threads = 128, ppt = 2, g2p_threads = 128;
  bool use_graph = true;
  int p2g_blocks = 0, g2p_blocks = 0, keys_blocks = 0, grid_blocks = 0, io_blocks = 0;
  int p2g_cpic_blocks = 0, g2p_cpic_blocks = 0;

  // streams, graph, timing
  cudaStream_t cs = nullptr;
  cudaEvent_t ev_in = nullptr, ev_out = nullptr;
  cudaGraphExec_t gexec = nullptr;
  bool graph_valid = false;
  bool grid_momentum[2] = {false, false};  // grid buffer holds P2G momentum (grid op fused into G2P)
  bool profiling = false;
  std::vector<TimedPair> pending;
  std::vector<cudaEvent_t> ev_pool;
  double ktime_ms[KT_N] = {0, 0, 0, 0, 0};
  int64_t kcount[KT_N] = {0, 0, 0, 0, 0};
};

namespace {

// NVTX range over an entry point (visible in Nsight timelines; a no-op without a tool attached).
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
};

int fail(mpm_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  else {
    std::lock_guard<std::mutex> lk(g_err_mu);
    g_create_err = msg;
  }
  return code;
}

#define CK(call)                                                                                    \
  do {                                                                                              \
    cudaError_t e_ = (call);                                                                        \
    if (e_ != cudaSuccess)                                                                          \
      return fail(ctx, MPM_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));           \
  } while (0)

#define CKL()                                                                                       \
  do {                                                                                              \
    cudaError_t e_ = cudaGetLastError();                                                            \
    if (e_ != cudaSuccess) return fail(ctx, MPM_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e_)); \
  } while (0)

// Launch with programmatic stream serialisation: the kernel may begin launching while the previous
// kernel of the stream drains; every kernel launched this way calls pdl_wait() before it reads
// what its predecessor wrote.
template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*kernel)(KArgs...), int grid, int block, size_t smem, cudaStream_t s, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3((unsigned)block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, args...);
}

template <typename T>
int dalloc(mpm_ctx* ctx, T** p, size_t count) {
  *p = nullptr;
  if (count == 0) count = 1;
  cudaError_t e = cudaMalloc((void**)p, count * sizeof(T));
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(ctx, MPM_ERR_OOM, std::string("cudaMalloc of ") + std::to_string(count * sizeof(T)) + " bytes: " +
                                      cudaGetErrorString(e));
  }
  ctx->allocs.push_back((void*)*p);
  return MPM_OK;
}

KParams make_params(mpm_ctx* ctx, int src, int dst, int g) {
  KParams P;
  std::memset(&P, 0, sizeof(P));
  P.scenes = ctx->d_scenes;
  P.mats = ctx->d_mats;
  P.block_scene = ctx->d_block_scene;
  P.src = ctx->d_pbuf[src];
  P.dst = ctx->d_pbuf[dst];
  P.cap = ctx->cap;
  P.nf = ctx->nf;
  P.chunk = ctx->p2g_threads * ctx->ppt;
  P.n = ctx->n_phys;
  P.K = ctx->K;
  P.n_scenes = (int32_t)ctx->n_scenes;
  P.grid = ctx->d_grid[g];
  P.grid_other = ctx->d_grid[1 - g];
  P.flags = ctx->d_flags[g];
  P.flags_other = ctx->d_flags[1 - g];
  P.list = ctx->d_list[g];
  P.nlist = ctx->d_nlist + g;
  P.list_other = ctx->d_list[1 - g];
  P.nlist_other = ctx->d_nlist + (1 - g);
  P.key = ctx->d_key;
  P.rank = ctx->d_rank;
  P.count = ctx->d_count;
  P.offset = ctx->d_offset;
  P.perm = ctx->d_perm;
  P.cell8 = ctx->d_cell8;
  P.slot_cell = ctx->d_slot_cell;
  P.items = ctx->d_items;
  P.n_items = ctx->d_nitems;
  P.partials = ctx->d_partials;
  P.scan_state = ctx->d_scan_state;
  P.ffs = ctx->d_ffs;
  P.n_ffs = ctx->n_ffs;
  P.grid_stage = 0;
  P.ff_begin = 0;
  P.ff_end = ctx->n_ffs;
  P.colliders = ctx->d_colliders;
  P.n_colliders = ctx->n_colliders;
  P.collider_acc = ctx->d_collider_acc;
  P.cpic_slots = ctx->cpic_slots;
  P.cpic_mask = ctx->d_cpic_mask;
  P.ext[0] = ctx->ext[0];
  P.ext[1] = ctx->ext[1];
  P.ff_step = ctx->d_ff_step;
  P.scan_sync = ctx->d_scan_sync;
  P.n_tiles = ctx->n_tiles;
  P.scan_tiles = ctx->d_scan_tiles;
  P.n_scan_tiles = ctx->d_n_scan_tiles;
  P.pin = ctx->d_pin;
  P.eps_norm = ctx->eps_norm;
  P.status = ctx->d_status;
  P.fp64_count = ctx->d_fp64;
  return P;
}

cudaEvent_t pool_event(mpm_ctx* ctx) {
  if (!ctx->ev_pool.empty()) {
    cudaEvent_t e = ctx->ev_pool.back();
    ctx->ev_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

struct Timer {
  mpm_ctx* ctx;
  cudaStream_t s;
  int kind;
  cudaEvent_t a = nullptr;
  Timer(mpm_ctx* c, cudaStream_t st, int k) : ctx(c), s(st), kind(k) {
    if (ctx->profiling) {
      a = pool_event(ctx);
      cudaEventRecord(a, s);
    }
  }
  ~Timer() {
    if (ctx->profiling) {
      cudaEvent_t b = pool_event(ctx);
      cudaEventRecord(b, s);
      ctx->pending.push_back({kind, a, b});
    }
  }
};

int launch_sort(mpm_ctx* ctx, const KParams& P, cudaStream_t s) {
  {
    Timer t(ctx, s, KT_SCAN);
    if (ctx->K + 2 <= SCAN_SINGLE_MAX) {
      CK(launch_pdl(k_scan_single, 1, 1024, 0, s, P));
    } else {
      CK(launch_pdl(k_scan_onepass, ctx->n_tiles, SCAN_THREADS, 0, s, P));
    }
  }
  CKL();
  if (P.n > 0 || P.steps || P.nlist_reset || P.colliders_rw) {
    Timer t(ctx, s, KT_PERM);
    CK(launch_pdl(k_perm, ctx->n_sm * 8, 256, 0, s, P));  // one wave; four particles per thread and pass
  }
  CKL();
  return MPM_OK;
}

// Keys of the current state (after load / set_state), then the sort.
int launch_rekey(mpm_ctx* ctx, cudaStream_t s) {
  KParams P = make_params(ctx, ctx->cur, ctx->cur, ctx->cur);
  if (ctx->n_phys > 0) {
    k_keys<<<ctx->keys_blocks, 256, 0, s>>>(P);
    CKL();
  }
  int r = launch_sort(ctx, P, s);
  if (r) return r;
  ctx->sorted = true;
  return MPM_OK;
}

int launch_pre(mpm_ctx* ctx, int c, cudaStream_t s) {
  KParams P = make_params(ctx, c, 1 - c, c);
  P.n = ctx->n;
  P.steps = ctx->d_steps;
  Timer t(ctx, s, KT_P2G);
  if (ctx->cpic_slots > 0 && ctx->n_colliders > 0)
    CK(launch_pdl(k_p2g_cpic, ctx->p2g_cpic_blocks, ctx->p2g_threads, p2g_dyn_smem(ctx->p2g_threads, P.chunk), s, P));
  else
    CK(launch_pdl(k_p2g, ctx->p2g_blocks, ctx->p2g_threads, p2g_dyn_smem(ctx->p2g_threads, P.chunk), s, P));
  CKL();
  return MPM_OK;
}

// The grid op, whole (stage 0) or one of its stages (see KParams::grid_stage); the coupled
// particle sets are binned around the stages that apply them (0 and 3).
int launch_grid(mpm_ctx* ctx, int c, cudaStream_t s, int stage = 0, int ff_begin = 0, int ff_end = -1) {
  KParams P = make_params(ctx, c, 1 - c, c);
  P.grid_stage = stage;
  P.ff_begin = ff_begin;
  P.ff_end = ff_end < 0 ? ctx->n_ffs : ff_end;
  ctx->grid_momentum[c] = false;
  const bool ext = stage == 0 || stage == 3;
  for (int k = 0; k < 2; ++k)
    if (ext && ctx->ext[k].n > 0) k_ext_bin<<<ctx->io_blocks, 256, 0, s>>>(P, k, 0);
  {
    Timer t(ctx, s, KT_GRID);
    k_grid_op<<<ctx->grid_blocks, 256, 0, s>>>(P);
  }
  for (int k = 0; k < 2; ++k)
    if (ext && ctx->ext[k].n > 0) k_ext_bin<<<ctx->io_blocks, 256, 0, s>>>(P, k, 1);
  CKL();
  return MPM_OK;
}

int launch_post(mpm_ctx* ctx, int c, cudaStream_t s, bool fuse_grid = false) {
  KParams P = make_params(ctx, c, 1 - c, c);
  P.n = ctx->n;
  P.n_dev = ctx->d_n;
  P.steps = ctx->d_steps;
  P.fuse_grid = fuse_grid ? 1 : 0;
  P.nlist_reset = fuse_grid ? P.nlist_other : nullptr;
  P.ff_step_advance = 1;
  P.colliders_rw = ctx->n_tools > 0 ? ctx->d_colliders : nullptr;
  ctx->grid_momentum[c] = fuse_grid;
  {
    Timer t(ctx, s, KT_G2P);
    if (ctx->cpic_slots > 0 && ctx->n_colliders > 0)
      CK(launch_pdl(k_g2p_cpic, ctx->g2p_cpic_blocks, ctx->g2p_threads, 0, s, P));
    else
      CK(launch_pdl(k_g2p, ctx->g2p_blocks, ctx->g2p_threads, 0, s, P));
  }
  CKL();
  if (ctx->d_cons) {  // after g2p, as substep_post_coupling does (mpm_solver.py:538-540)
    k_constraints<<<ctx->io_blocks, 256, 0, s>>>(P, ctx->d_cons, ctx->d_links, ctx->n_links);
    CKL();
  }
  return launch_sort(ctx, P, s);
}

// Without pinned particles the grid op is folded into G2P (k_grid_op is not launched); the
// split-phase entry points keep it separate so a coupler can act on the velocity grid.
int launch_substep(mpm_ctx* ctx, int c, cudaStream_t s) {
  const bool fuse = ctx->d_pin == nullptr && ctx->n_colliders == 0 && ctx->n_ffs == 0 && ctx->ext[0].n == 0 &&
                    ctx->ext[1].n == 0;
  int r = launch_pre(ctx, c, s);
  if (!r && !fuse) r = launch_grid(ctx, c, s);
  if (!r) r = launch_post(ctx, c, s, fuse);
  return r;
}

// The bucket ranges the one-pass scan covers, in tiles of SCAN_TILE: every bucket of a plain
// context; in a pool only the blocks of each live slot's own grid, then the inactive and dead
// buckets.  Synchronises the context stream (the host table must outlive the copy).
int upload_scan_tiles(mpm_ctx* ctx) {
  std::vector<int2> t;
  auto add = [&](int64_t b, int64_t e) {
    for (int64_t k = b; k < e; k += SCAN_TILE) t.push_back(make_int2((int)k, (int)(k + SCAN_TILE < e ? k + SCAN_TILE : e)));
  };
  if (!ctx->pool) {
    add(0, ctx->K + 2);
  } else {
    for (int64_t s = 0; s < ctx->n_scenes; ++s)
      if (ctx->slot_live[s]) {
        const SceneDev& S = ctx->scenes_h[s];
        add(S.block_base, S.block_base + (int64_t)S.bres[0] * S.bres[1] * S.bres[2]);
      }
    add(ctx->K, ctx->K + 2);
  }
  if ((int64_t)t.size() > ctx->n_tiles) return fail(ctx, MPM_ERR_STATE, "scan tile table overflow");
  const int32_t nt = (int32_t)t.size();
  CK(cudaMemcpyAsync(ctx->d_scan_tiles, t.data(), sizeof(int2) * t.size(), cudaMemcpyHostToDevice, ctx->cs));
  CK(cudaMemcpyAsync(ctx->d_n_scan_tiles, &nt, sizeof(int32_t), cudaMemcpyHostToDevice, ctx->cs));
  CK(cudaStreamSynchronize(ctx->cs));
  return MPM_OK;
}

int compute_launch_shapes(mpm_ctx* ctx) {
  int occ = 0;
  CK(cudaFuncSetAttribute(k_p2g, cudaFuncAttributeMaxDynamicSharedMemorySize,
                          (int)p2g_dyn_smem(P2G_MAX_THREADS, P2G_MAX_CHUNK)));
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_p2g, ctx->p2g_threads,
                                                   p2g_dyn_smem(ctx->p2g_threads, ctx->p2g_threads * ctx->ppt)));
  ctx->p2g_blocks = ctx->n_sm * (occ > 0 ? occ : 1);
  int occ2 = 0;
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ2, k_g2p, ctx->g2p_threads, 0));
  ctx->g2p_blocks = ctx->n_sm * (occ2 > 0 ? occ2 : 1);  // persistent over the work items
  if (ctx->cpic_slots > 0) {
    CK(cudaFuncSetAttribute(k_p2g_cpic, cudaFuncAttributeMaxDynamicSharedMemorySize,
                            (int)p2g_dyn_smem(P2G_MAX_THREADS, P2G_MAX_CHUNK)));
    int oc = 0;
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&oc, k_p2g_cpic, ctx->p2g_threads,
                                                     p2g_dyn_smem(ctx->p2g_threads, ctx->p2g_threads * ctx->ppt)));
    ctx->p2g_cpic_blocks = ctx->n_sm * (oc > 0 ? oc : 1);
    oc = 0;
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&oc, k_g2p_cpic, ctx->g2p_threads, 0));
    ctx->g2p_cpic_blocks = ctx->n_sm * (oc > 0 ? oc : 1);
  }
  int occ3 = 0;
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ3, k_keys, 256, 0));
  const int64_t ext = ctx->n_phys > ctx->n ? ctx->n_phys : ctx->n;
  int64_t want = (ext + 255) / 256;
  int64_t lim = (int64_t)ctx->n_sm * (occ3 > 0 ? occ3 : 1);
  ctx->keys_blocks = (int)(want < 1 ? 1 : (want < lim ? want : lim));
  ctx->grid_blocks = ctx->n_sm * 8;
  (void)ext;
  ctx->io_blocks = ctx->n_sm * 16;  // grid-stride; independent of n so captured graphs stay valid
  return MPM_OK;
}

void drop_graph(mpm_ctx* ctx) {
  if (ctx->gexec) cudaGraphExecDestroy(ctx->gexec);
  ctx->gexec = nullptr;
  ctx->graph_valid = false;
}

// Two substeps (parity 0 then 1) captured once; replays keep `cur` at 0.
int ensure_graph(mpm_ctx* ctx) {
  if (ctx->graph_valid) return MPM_OK;
  drop_graph(ctx);
  cudaGraph_t g = nullptr;
  CK(cudaStreamBeginCapture(ctx->cs, cudaStreamCaptureModeThreadLocal));
  int r = launch_substep(ctx, 0, ctx->cs);
  if (!r) r = launch_substep(ctx, 1, ctx->cs);
  cudaError_t e = cudaStreamEndCapture(ctx->cs, &g);
  if (r) {
    if (g) cudaGraphDestroy(g);
    return r;
  }
  if (e != cudaSuccess) return fail(ctx, MPM_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
  e = cudaGraphInstantiate(&ctx->gexec, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return fail(ctx, MPM_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
  ctx->graph_valid = true;
  return MPM_OK;
}

int enter(mpm_ctx* ctx, void* stream) {
  CK(cudaSetDevice(ctx->device));
  CK(cudaEventRecord(ctx->ev_in, (cudaStream_t)stream));
  CK(cudaStreamWaitEvent(ctx->cs, ctx->ev_in, 0));
  return MPM_OK;
}

int leave(mpm_ctx* ctx, void* stream) {
  CK(cudaEventRecord(ctx->ev_out, ctx->cs));
  CK(cudaStreamWaitEvent((cudaStream_t)stream, ctx->ev_out, 0));
  return MPM_OK;
}


}  // namespace

namespace gbmpm {
// Scene constants exactly as MPMSolver.__init__ (mpm_solver.py:32-80); fills everything but
// the block/material/particle bases.
int derive_scene(const mpm_scene_config& c, SceneDev& S, std::string& err) {
  std::memset(&S, 0, sizeof(S));
  if (!(c.grid_density > 0) || !(c.particle_size > 0) || !(c.substep_dt > 0) || c.n_particles < 0) {
    err = "invalid grid_density/particle_size/substep_dt/n_particles";
    return MPM_ERR_BAD_ARG;
  }
  const double dx = 1.0 / c.grid_density;
  const double inv_dx = c.grid_density;
  int64_t lo_cell[3], hi_cell[3], res[3];
  double nodes = 1.0;
  for (int d = 0; d < 3; ++d) {
    if (!(c.upper_bound[d] > c.lower_bound[d])) {
      err = "Invalid pair of upper_bound and lower_bound.";
      return MPM_ERR_BAD_ARG;
    }
    lo_cell[d] = (int64_t)std::nearbyint(c.grid_density * c.lower_bound[d]);
    hi_cell[d] = (int64_t)std::nearbyint(c.grid_density * c.upper_bound[d]);
    res[d] = hi_cell[d] - lo_cell[d] + 1;
    nodes *= (double)res[d];
  }
  if (nodes > 1e9) {
    err = "Grid size larger than 1e9 not supported by MPM solver. Please reduce 'grid_density', or set tighter "
          "boundaries via 'lower_bound' / 'upper_bound'.";
    return MPM_ERR_BAD_ARG;
  }
  const double pvol = c.particle_size * c.particle_size * c.particle_size * 1e3;
  S.dx = (float)dx;
  S.inv_dx = (float)inv_dx;
  S.dt = (float)c.substep_dt;
  S.stress_scale = (float)(-c.substep_dt * pvol * 4.0 * inv_dx * inv_dx);
  for (int d = 0; d < 3; ++d) {
    S.grav[d] = (float)c.gravity[d];
    S.lo[d] = (float)(c.lower_bound[d] + 3.0 * dx);
    S.hi[d] = (float)(c.upper_bound[d] - 3.0 * dx);
    S.res[d] = (int32_t)res[d];
    S.offset[d] = (int32_t)lo_cell[d];
    S.bres[d] = (int32_t)((res[d] + BLK - 1) / BLK);
  }
  S.eps = (float)c.mass_eps;
  S.restitution = (float)c.restitution;
  S.n_particles = c.n_particles;
  return MPM_OK;
}

// Material record with the constants the reference folds in Python before compiling its
// kernels (sand.py:70, snow.py:60, elasto_plastic.py:56) and the fp32 particle mass
// particle_volume * rho (mpm_solver.py:822).
MaterialDev derive_material(const mpm_material& m, const mpm_scene_config& c) {
  MaterialDev M;
  std::memset(&M, 0, sizeof(M));
  M.type = m.type;
  M.flags = m.flags;
  M.scene = m.scene;
  M.mu = (float)m.mu;
  M.lam = (float)m.lam;
  const float pvol = (float)(c.particle_size * c.particle_size * c.particle_size * 1e3);
  M.mass = pvol * (float)m.rho;
  M.default_Jp = (float)m.default_Jp;
  M.alpha = (float)m.friction_alpha;
  M.sand_coef = m.mu != 0.0 ? (float)((3.0 * m.lam + 2.0 * m.mu) / (2.0 * m.mu)) : 0.f;
  M.clamp_lo = (float)(1.0 - m.yield_lower);
  M.clamp_hi = (float)(1.0 + m.yield_higher);
  M.vm_ratio = m.mu != 0.0 ? (float)(m.von_mises_yield_stress / (2.0 * m.mu)) : 0.f;
  M.stiffness = (float)m.stiffness;
  return M;
}

// A force field as the grid op reads it (float copies of the ABI record); false for an unknown type.
bool force_field_dev(const mpm_force_field& f, ForceFieldDev& d) {
  if (f.type < MPM_FF_CONSTANT || f.type > MPM_FF_TURBULENCE) return false;
  std::memset(&d, 0, sizeof(d));
  d.type = f.type;
  d.active = f.active ? 1 : 0;
  for (int k = 0; k < 3; ++k) {
    d.dir[k] = (float)f.direction[k];
    d.center[k] = (float)f.center[k];
  }
  d.strength = (float)f.strength;
  d.radius = (float)f.radius;
  d.falloff_pow = (float)f.falloff_pow;
  d.flow = (float)f.flow;
  d.linear = (float)f.linear;
  d.quadratic = (float)f.quadratic;
  d.s_perp = (float)f.strength_perpendicular;
  d.s_radial = (float)f.strength_radial;
  d.falloff_min = (float)f.falloff_min;
  d.falloff_max = (float)f.falloff_max;  // +inf stays +inf
  d.damping = (float)f.damping;
  d.frequency = (float)f.frequency;
  d.seed = (unsigned long long)f.seed;
  std::memcpy(d.perm, f.perm, sizeof(d.perm));
  return true;
}

// A collider as the grid op reads it (float copies; SDF grids from ctx's table); null on success,
// else what is wrong with the record.
const char* collider_dev(const mpm_ctx* ctx, const mpm_collider& c, ColliderDev& d) {
  if (c.type < MPM_COLLIDER_SPHERE || c.type > MPM_COLLIDER_TOOL) return "unknown collider type";
  const bool gridded = c.type == MPM_COLLIDER_SDF || c.type == MPM_COLLIDER_TOOL;
  if (gridded && (!ctx || c.sdf_grid < 0 || c.sdf_grid >= (int32_t)ctx->sdf_grids.size()))
    return "collider SDF grid id out of range (mpm_add_sdf_grid)";
  if (c.type == MPM_COLLIDER_SDF && !ctx->sdf_grids[(size_t)c.sdf_grid].grad)
    return "an SDF collider needs a grid with gradients";
  std::memset(&d, 0, sizeof(d));
  d.type = c.type;
  d.scene = c.scene;
  for (int k = 0; k < 3; ++k) {
    d.pos[k] = (float)c.pos[k];
    d.size[k] = (float)c.size[k];
    d.com[k] = (float)c.com[k];
    d.lin[k] = (float)c.lin_vel[k];
    d.ang[k] = (float)c.ang_vel[k];
  }
  for (int k = 0; k < 4; ++k) d.quat[k] = (float)c.quat[k];
  d.friction = (float)c.friction;
  d.softness = (float)c.softness;
  d.restitution = (float)c.restitution;
  if (gridded) {
    const mpm_ctx::SdfGrid& g = ctx->sdf_grids[(size_t)c.sdf_grid];
    d.pad0 = c.sdf_grid;
    d.val = g.val;
    d.grad = g.grad;
    for (int k = 0; k < 3; ++k) d.res[k] = g.res[k];
    for (int k = 0; k < 12; ++k) d.T[k] = (float)g.T[k];
    // inverse of the 3x3 block (tool normals: voxel frame -> mesh frame), by cofactors in double
    const double* T = g.T;
    const double a = T[0], b = T[1], cc = T[2], e = T[4], f = T[5], gg = T[6], h = T[8], i2 = T[9], j = T[10];
    const double det = a * (f * j - gg * i2) - b * (e * j - gg * h) + cc * (e * i2 - f * h);
    if (!(std::fabs(det) > 0)) return "T_mesh_to_sdf is singular";
    const double inv[9] = {(f * j - gg * i2) / det, (cc * i2 - b * j) / det, (b * gg - cc * f) / det,
                           (gg * h - e * j) / det,  (a * j - cc * h) / det,  (cc * e - a * gg) / det,
                           (e * i2 - f * h) / det,  (b * h - a * i2) / det,  (a * f - b * e) / det};
    for (int k = 0; k < 9; ++k) d.Rinv[k] = (float)inv[k];
    d.cell_size = (float)g.cell_size;
    d.sdf_max = (float)g.sdf_max;
    d.floor_h = (float)c.floor_height;
  }
  return nullptr;
}

}  // namespace gbmpm

namespace {

bool scene_range_ok(mpm_ctx* ctx, int64_t s0, int64_t s1) { return s0 >= 0 && s1 <= ctx->n_scenes && s0 < s1; }

}  // namespace

int mpm_ctx_destroy(mpm_ctx* ctx);
// Allocates every device buffer of a context whose host tables are filled, uploads them
// and initialises the particle slots; on failure frees the context.
static int ctx_alloc_init(mpm_ctx* ctx, int32_t device, const std::vector<int32_t>& block_scene_h, mpm_ctx** out) {
  int r = MPM_OK;
  do {
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) {
      r = fail(nullptr, MPM_ERR_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
      break;
    }
    cudaDeviceProp prop;
    e = cudaGetDeviceProperties(&prop, device);
    if (e != cudaSuccess) {
      r = fail(nullptr, MPM_ERR_CUDA, std::string("cudaGetDeviceProperties: ") + cudaGetErrorString(e));
      break;
    }
    ctx->n_sm = prop.multiProcessorCount;
    ctx->max_items = ctx->cap / 32 + ctx->K + 4;
    // a pool's live ranges are rounded up to whole tiles per slot: one extra tile per slot at most
    ctx->n_tiles = (int)((ctx->K + 2 + SCAN_TILE - 1) / SCAN_TILE) + (ctx->pool ? (int)ctx->n_scenes + 1 : 0);
    if ((r = dalloc(ctx, &ctx->d_scenes, ctx->n_scenes))) break;
    if ((r = dalloc(ctx, &ctx->d_mats, ctx->n_mats > 0 ? ctx->n_mats : 1))) break;
    if ((r = dalloc(ctx, &ctx->d_block_scene, ctx->K))) break;
    if ((r = dalloc(ctx, &ctx->d_pbegin, ctx->n_scenes + 1))) break;
    if ((r = dalloc(ctx, &ctx->d_first_mat, ctx->n_scenes))) break;
    for (int b = 0; b < 2 && !r; ++b) {
      if ((r = dalloc(ctx, &ctx->d_pbuf[b], (size_t)ctx->nf * ctx->cap))) break;
      if ((r = dalloc(ctx, &ctx->d_grid[b], (size_t)ctx->K * BLK_NODES))) break;
      if ((r = dalloc(ctx, &ctx->d_flags[b], ctx->K))) break;
      if ((r = dalloc(ctx, &ctx->d_list[b], ctx->K))) break;
    }
    if (r) break;
    if ((r = dalloc(ctx, &ctx->d_nlist, 2))) break;
    if ((r = dalloc(ctx, &ctx->d_key, ctx->cap))) break;
    if ((r = dalloc(ctx, &ctx->d_rank, ctx->cap))) break;
    if ((r = dalloc(ctx, &ctx->d_perm, ctx->cap))) break;
    if ((r = dalloc(ctx, &ctx->d_cell8, ctx->cap))) break;
    if ((r = dalloc(ctx, &ctx->d_slot_cell, ctx->cap))) break;
    if ((r = dalloc(ctx, &ctx->d_count, ctx->K + 2))) break;
    if ((r = dalloc(ctx, &ctx->d_offset, ctx->K + 2))) break;
    if ((r = dalloc(ctx, &ctx->d_items, ctx->max_items))) break;
    if ((r = dalloc(ctx, &ctx->d_nitems, 1))) break;
    if ((r = dalloc(ctx, &ctx->d_partials, ctx->n_tiles))) break;
    if ((r = dalloc(ctx, &ctx->d_scan_state, ctx->n_tiles))) break;
    if ((r = dalloc(ctx, &ctx->d_scan_sync, 2))) break;
    if ((r = dalloc(ctx, &ctx->d_scan_tiles, ctx->n_tiles))) break;
    if ((r = dalloc(ctx, &ctx->d_n_scan_tiles, 1))) break;
    if ((r = dalloc(ctx, &ctx->d_status, 1))) break;
    if ((r = dalloc(ctx, &ctx->d_fp64, 1))) break;
    if ((r = dalloc(ctx, &ctx->d_tmp64, 1))) break;
    if ((r = dalloc(ctx, &ctx->d_steps, ctx->n_scenes))) break;
    if ((r = dalloc(ctx, &ctx->d_n, 1))) break;
  } while (0);
  if (r) {
    if (r != MPM_OK && ctx->err.size()) fail(nullptr, r, ctx->err);
    mpm_ctx_destroy(ctx);
    return r;
  }
#define CKC(call)                                                                                   \
  do {                                                                                              \
    cudaError_t e_ = (call);                                                                        \
    if (e_ != cudaSuccess) {                                                                        \
      fail(nullptr, MPM_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));              \
      mpm_ctx_destroy(ctx);                                                                         \
      return MPM_ERR_CUDA;                                                                          \
    }                                                                                               \
  } while (0)
  CKC(cudaStreamCreateWithFlags(&ctx->cs, cudaStreamNonBlocking));
  CKC(cudaEventCreateWithFlags(&ctx->ev_in, cudaEventDisableTiming));
  CKC(cudaEventCreateWithFlags(&ctx->ev_out, cudaEventDisableTiming));
  CKC(cudaMemcpyAsync(ctx->d_scenes, ctx->scenes_h.data(), sizeof(SceneDev) * ctx->n_scenes, cudaMemcpyHostToDevice, ctx->cs));
  if (ctx->n_mats > 0)
    CKC(cudaMemcpyAsync(ctx->d_mats, ctx->mats_h.data(), sizeof(MaterialDev) * ctx->n_mats, cudaMemcpyHostToDevice,
                        ctx->cs));
  if (ctx->K > 0)
    CKC(cudaMemcpyAsync(ctx->d_block_scene, block_scene_h.data(), sizeof(int32_t) * ctx->K, cudaMemcpyHostToDevice, ctx->cs));
  CKC(cudaMemcpyAsync(ctx->d_pbegin, ctx->pbegin_h.data(), sizeof(int64_t) * (ctx->n_scenes + 1), cudaMemcpyHostToDevice,
                      ctx->cs));
  CKC(cudaMemcpyAsync(ctx->d_first_mat, ctx->first_mat_h.data(), sizeof(int32_t) * ctx->n_scenes, cudaMemcpyHostToDevice,
                      ctx->cs));
  for (int b = 0; b < 2; ++b) {
    CKC(cudaMemsetAsync(ctx->d_grid[b], 0, sizeof(float4) * (size_t)ctx->K * BLK_NODES, ctx->cs));
    CKC(cudaMemsetAsync(ctx->d_flags[b], 0, sizeof(int32_t) * (size_t)(ctx->K > 0 ? ctx->K : 1), ctx->cs));
    CKC(cudaMemsetAsync(ctx->d_pbuf[b], 0, sizeof(float) * (size_t)ctx->nf * ctx->cap, ctx->cs));
  }
  CKC(cudaMemsetAsync(ctx->d_nlist, 0, sizeof(int32_t) * 2, ctx->cs));
  CKC(cudaMemsetAsync(ctx->d_count, 0, sizeof(int32_t) * (ctx->K + 2), ctx->cs));
  CKC(cudaMemsetAsync(ctx->d_nitems, 0, sizeof(int32_t), ctx->cs));
  CKC(cudaMemsetAsync(ctx->d_scan_state, 0, sizeof(unsigned long long) * ctx->n_tiles, ctx->cs));
  CKC(cudaMemsetAsync(ctx->d_scan_sync, 0, sizeof(int32_t) * 2, ctx->cs));
  CKC(cudaMemsetAsync(ctx->d_status, 0, sizeof(uint32_t), ctx->cs));
  CKC(cudaMemsetAsync(ctx->d_fp64, 0, sizeof(unsigned long long), ctx->cs));
  CKC(cudaMemsetAsync(ctx->d_steps, 0xff, sizeof(int32_t) * ctx->n_scenes, ctx->cs));  // -1: unlimited
  CKC(cudaMemcpyAsync(ctx->d_n, &ctx->n, sizeof(int64_t), cudaMemcpyHostToDevice, ctx->cs));
  if (upload_scan_tiles(ctx)) {
    fail(nullptr, MPM_ERR_CUDA, ctx->err);
    mpm_ctx_destroy(ctx);
    return MPM_ERR_CUDA;
  }
  if (compute_launch_shapes(ctx)) {
    fail(nullptr, MPM_ERR_CUDA, ctx->err);
    mpm_ctx_destroy(ctx);
    return MPM_ERR_CUDA;
  }
  if (ctx->n > 0 && ctx->n_mats > 0) {
    KParams Pp = make_params(ctx, 0, 0, 0);
    k_init_particles<<<ctx->io_blocks, 256, 0, ctx->cs>>>(Pp, ctx->d_pbegin, ctx->d_first_mat, ctx->n_scenes);
    CKC(cudaGetLastError());
  }
  CKC(cudaStreamSynchronize(ctx->cs));
#undef CKC
  *out = ctx;
  return MPM_OK;
}

// =====================================================================================
extern "C" {

const char* mpm_last_error(const mpm_ctx* ctx) {
  if (ctx) return ctx->err.c_str();
  std::lock_guard<std::mutex> lk(g_err_mu);
  return g_create_err.c_str();
}

int mpm_ctx_create(const mpm_scene_config* scenes, int64_t n_scenes, const mpm_material* materials,
                   int32_t n_materials, int32_t device, mpm_ctx** out) {
  if (!out) return fail(nullptr, MPM_ERR_BAD_ARG, "out is NULL");
  *out = nullptr;
  if (!scenes || n_scenes <= 0) return fail(nullptr, MPM_ERR_BAD_ARG, "need at least one scene");
  if (n_materials < 0 || (n_materials > 0 && !materials)) return fail(nullptr, MPM_ERR_BAD_ARG, "bad material table");
  if ((int64_t)n_materials > (int64_t)INFO_MAT_MASK) return fail(nullptr, MPM_ERR_BAD_ARG, "too many materials");

  mpm_ctx* ctx = new mpm_ctx();
  ctx->device = device;
  ctx->n_scenes = n_scenes;
  ctx->n_mats = n_materials;

  // materials: grouped by scene in ascending order
  std::vector<int32_t> mat_begin(n_scenes, -1), mat_count(n_scenes, 0);
  bool muscle = false;
  int32_t prev_scene = -1;
  for (int32_t i = 0; i < n_materials; ++i) {
    const mpm_material& m = materials[i];
    if (m.scene < 0 || m.scene >= n_scenes || m.scene < prev_scene) {
      delete ctx;
      return fail(nullptr, MPM_ERR_BAD_ARG, "materials must be grouped by scene in ascending scene order");
    }
    if (m.type < MPM_MAT_ELASTIC || m.type > MPM_MAT_MUSCLE) {
      delete ctx;
      return fail(nullptr, MPM_ERR_BAD_ARG, "unknown material type");
    }
    prev_scene = m.scene;
    if (mat_begin[m.scene] < 0) mat_begin[m.scene] = i;
    mat_count[m.scene]++;
    muscle = muscle || m.type == MPM_MAT_MUSCLE;
  }
  ctx->nf = muscle ? NF_MUSCLE : NF_BASE;
  ctx->mat_count_h = mat_count;

  // scenes: derived constants exactly as MPMSolver.__init__ (mpm_solver.py:32-80)
  int64_t K = 0, P = 0;
  ctx->pbegin_h.resize(n_scenes + 1);
  ctx->first_mat_h.resize(n_scenes);
  std::vector<int32_t> block_scene_h;
  for (int64_t s = 0; s < n_scenes; ++s) {
    const mpm_scene_config& c = scenes[s];
    if (!(c.grid_density > 0) || !(c.particle_size > 0) || !(c.substep_dt > 0) || c.n_particles < 0) {
      delete ctx;
      return fail(nullptr, MPM_ERR_BAD_ARG, "scene " + std::to_string(s) + ": invalid grid_density/particle_size/dt");
    }
    SceneDev S;
    std::string derr;
    if (int e = derive_scene(c, S, derr)) {
      delete ctx;
      return fail(nullptr, e, derr);
    }
    S.mat_begin = mat_begin[s] < 0 ? 0 : mat_begin[s];
    S.block_base = K;
    S.p_begin = P;
    S.n_particles = c.n_particles;
    if (c.n_particles > 0 && mat_count[s] == 0) {
      delete ctx;
      return fail(nullptr, MPM_ERR_BAD_ARG, "scene " + std::to_string(s) + " has particles but no material");
    }
    const int64_t nb = (int64_t)S.bres[0] * S.bres[1] * S.bres[2];
    block_scene_h.insert(block_scene_h.end(), nb, (int32_t)s);
    K += nb;
    ctx->pbegin_h[s] = P;
    ctx->first_mat_h[s] = S.mat_begin;
    P += c.n_particles;
    ctx->scenes_h.push_back(S);
    if (s == 0) ctx->eps_norm = (float)c.mass_eps;
  }
  ctx->pbegin_h[n_scenes] = P;
  if (K + 2 >= (int64_t)INT32_MAX / 2 || P >= (int64_t)INT32_MAX / 2) {
    delete ctx;
    return fail(nullptr, MPM_ERR_BAD_ARG, "too many grid blocks or particles for one context");
  }
  ctx->K = K;
  ctx->n = P;
  ctx->n_phys = P;
  ctx->cap = ((P + 63) / 64) * 64;
  if (P < 65536) {  // small scenes are latency-bound: items of 64 particles spread them over more SMs
    ctx->p2g_threads = 64;
    ctx->ppt = 1;
  }
  if (ctx->cap == 0) ctx->cap = 64;

  for (int32_t i = 0; i < n_materials; ++i) {
    const mpm_material& m = materials[i];
    const mpm_scene_config& c = scenes[m.scene];
    MaterialDev M = derive_material(m, c);
    ctx->mats_h.push_back(M);
  }

  return ctx_alloc_init(ctx, device, block_scene_h, out);
}

int mpm_ctx_destroy(mpm_ctx* ctx) {
  if (!ctx) return MPM_OK;
  cudaSetDevice(ctx->device);
  if (ctx->cs) cudaStreamSynchronize(ctx->cs);
  drop_graph(ctx);
  for (auto& tp : ctx->pending) {
    cudaEventDestroy(tp.a);
    cudaEventDestroy(tp.b);
  }
  for (auto e : ctx->ev_pool) cudaEventDestroy(e);
  for (void* p : ctx->allocs) cudaFree(p);
  if (ctx->d_pin) cudaFree(ctx->d_pin);
  if (ctx->d_cons) cudaFree(ctx->d_cons);
  if (ctx->d_colliders) cudaFree(ctx->d_colliders);
  for (auto& g : ctx->sdf_grids) {
    if (g.val) cudaFree(g.val);
    if (g.grad) cudaFree(g.grad);
  }
  if (ctx->d_ffs) cudaFree(ctx->d_ffs);
  if (ctx->d_ff_step) cudaFree(ctx->d_ff_step);
  if (ctx->d_collider_acc) cudaFree(ctx->d_collider_acc);
  if (ctx->d_cpic_mask) cudaFree(ctx->d_cpic_mask);
  for (int k = 0; k < 2; ++k) {
    if (ctx->ext[k].head) cudaFree(ctx->ext[k].head);
    if (ctx->ext[k].next) cudaFree(ctx->ext[k].next);
    if (ctx->ext[k].node) cudaFree(ctx->ext[k].node);
  }
  if (ctx->d_links) cudaFree(ctx->d_links);
  if (ctx->ev_in) cudaEventDestroy(ctx->ev_in);
  if (ctx->ev_out) cudaEventDestroy(ctx->ev_out);
  if (ctx->cs) cudaStreamDestroy(ctx->cs);
  delete ctx;
  return MPM_OK;
}

int mpm_add_particles(mpm_ctx* ctx, int64_t scene_begin, int64_t scene_end, int64_t particle_start, int64_t n,
                      int32_t material, int32_t active, const float* pos, void* stream) {
  if (!ctx) return MPM_ERR_BAD_ARG;
  if (!scene_range_ok(ctx, scene_begin, scene_end)) return fail(ctx, MPM_ERR_BAD_ARG, "bad scene range");
  if (ctx->phase != 0) return fail(ctx, MPM_ERR_STATE, "add_particles inside a substep");
  if (n <= 0) return MPM_OK;
  if (!pos) return fail(ctx, MPM_ERR_BAD_ARG, "pos is NULL");
  for (int64_t s = scene_begin; s < scene_end; ++s) {
    const SceneDev& S = ctx->scenes_h[s];
    if (material < 0 || material >= ctx->mat_count_h[s]) return fail(ctx, MPM_ERR_BAD_ARG, "material index out of range for scene");
    if (particle_start < 0 || particle_start + n > S.n_particles)
      return fail(ctx, MPM_ERR_BAD_ARG, "particle range exceeds the scene's capacity");
  }
  int r = enter(ctx, stream);
  if (r) return r;
  KParams P = make_params(ctx, ctx->cur, ctx->cur, ctx->cur);
  k_add_particles<<<ctx->io_blocks, 256, 0, ctx->cs>>>(P, scene_begin, scene_end, particle_start, n, material, active,
                                                       pos);
  CKL();
  ctx->sorted = false;
  return leave(ctx, stream);
}

int mpm_get_state(mpm_ctx* ctx, int64_t scene_begin, int64_t scene_end, float* pos, float* vel, float* C, float* F,
                  float* Jp, uint8_t* active, void* stream) {
  NvtxRange nvtx_range("mpm_get_state");
  if (!ctx) return MPM_ERR_BAD_ARG;
  if (!scene_range_ok(ctx, scene_begin, scene_end)) return fail(ctx, MPM_ERR_BAD_ARG, "bad scene range");
  if (ctx->phase != 0) return fail(ctx, MPM_ERR_STATE, "get_state inside a substep");
  int r = enter(ctx, stream);
  if (r) return r;
  KParams P = make_params(ctx, ctx->cur, ctx->cur, ctx->cur);
  if (!ctx->pool && ctx->n_phys == ctx->n) {  // every row holds one particle: gather in row order
    const int64_t rows = ctx->pbegin_h[scene_end] - ctx->pbegin_h[scene_begin];
    uint32_t* row_info = reinterpret_cast<uint32_t*>(ctx->d_rank);
    k_row_slots<<<ctx->io_blocks, 256, 0, ctx->cs>>>(P, scene_begin, scene_end, ctx->d_key, row_info);
    k_get_state_rows<<<ctx->io_blocks, 256, 0, ctx->cs>>>(P, rows, ctx->d_key, row_info, pos, vel, C, F, Jp, active);
  } else {
    k_get_state<<<ctx->io_blocks, 256, 0, ctx->cs>>>(P, scene_begin, scene_end, pos, vel, C, F, Jp, active);
  }
  CKL();
  return leave(ctx, stream);
}

int mpm_set_state(mpm_ctx* ctx, int64_t scene_begin, int64_t scene_end, const float* pos, const float* vel,
                  const float* C, const float* F, const float* Jp, const uint8_t* active, void* stream) {
  NvtxRange nvtx_range("mpm_set_state");
  if (!ctx) return MPM_ERR_BAD_ARG;
  if (!scene_range_ok(ctx, scene_begin, scene_end)) return fail(ctx, MPM_ERR_BAD_ARG, "bad scene range");
  if (ctx->phase != 0) return fail(ctx, MPM_ERR_STATE, "set_state inside a substep");
  int r = enter(ctx, stream);
  if (r) return r;
  KParams P = make_params(ctx, ctx->cur, ctx->cur, ctx->cur);
  const bool whole = !ctx->pool && ctx->n_phys == ctx->n && scene_begin == 0 && scene_end == ctx->n_scenes &&
                     ctx->nf == NF_BASE && pos && vel && C && F && Jp;
  if (whole) {  // a full state of every scene: rewrite it in row order
    uint32_t* row_info = reinterpret_cast<uint32_t*>(ctx->d_rank);
    k_row_slots<<<ctx->io_blocks, 256, 0, ctx->cs>>>(P, 0, ctx->n_scenes, ctx->d_key, row_info);
    k_set_state_rows<<<ctx->io_blocks, 256, 0, ctx->cs>>>(P, ctx->n, row_info, pos, vel, C, F, Jp, active);
  } else {
    k_set_state<<<ctx->io_blocks, 256, 0, ctx->cs>>>(P, scene_begin, scene_end, pos, vel, C, F, Jp, active);
  }
  CKL();
  ctx->sorted = false;
  return leave(ctx, stream);
}

static int particles_field(mpm_ctx* ctx, int32_t field, int write, int64_t s0, int64_t s1, int64_t start, int64_t n,
                           float* data, void* stream) {
  if (!ctx) return MPM_ERR_BAD_ARG;
  if (!scene_range_ok(ctx, s0, s1)) return fail(ctx, MPM_ERR_BAD_ARG, "bad scene range");
  if (field < 0 || field > MPM_FIELD_POS_RESET) return fail(ctx, MPM_ERR_BAD_ARG, "unknown field");
  if (field == MPM_FIELD_POS_RESET && !write) return fail(ctx, MPM_ERR_BAD_ARG, "POS_RESET is write-only");
  if ((field == MPM_FIELD_ACTU || field == MPM_FIELD_MUSCLE_DIR) && ctx->nf == NF_BASE)
    return fail(ctx, MPM_ERR_BAD_ARG, "no muscle material in this context");
  if (ctx->phase != 0) return fail(ctx, MPM_ERR_STATE, "particle access inside a substep");
  if (n <= 0) return MPM_OK;
  if (!data) return fail(ctx, MPM_ERR_BAD_ARG, "data is NULL");
  int r = enter(ctx, stream);
  if (r) return r;
  if (write && field == MPM_FIELD_FREE && !ctx->d_pin) {
    const size_t words = ((size_t)ctx->K * BLK_NODES + 31) / 32;
    cudaError_t e = cudaMalloc((void**)&ctx->d_pin, words * sizeof(uint32_t));
    if (e != cudaSuccess) return fail(ctx, MPM_ERR_OOM, "pin bitmap allocation failed");
    CK(cudaMemsetAsync(ctx->d_pin, 0, words * sizeof(uint32_t), ctx->cs));
    drop_graph(ctx);
  }
  KParams P = make_params(ctx, ctx->cur, ctx->cur, ctx->cur);
  k_particles_field<<<ctx->io_blocks, 256, 0, ctx->cs>>>(P, field, write, s0, s1, start, n, data);
  CKL();
  if (write && (field == MPM_FIELD_POS || field == MPM_FIELD_POS_RESET || field == MPM_FIELD_ACTIVE))
    ctx->sorted = false;
  return leave(ctx, stream);
}

int mpm_set_particles(mpm_ctx* ctx, int32_t field, int64_t scene_begin, int64_t scene_end, int64_t particle_start,
                      int64_t n, const float* data, void* stream) {
  return particles_field(ctx, field, 1, scene_begin, scene_end, particle_start, n, const_cast<float*>(data), stream);
}

int mpm_get_particles(mpm_ctx* ctx, int32_t field, int64_t scene_begin, int64_t scene_end, int64_t particle_start,
                      int64_t n, float* data, void* stream) {
  return particles_field(ctx, field, 0, scene_begin, scene_end, particle_start, n, data, stream);
}

int mpm_set_gravity(mpm_ctx* ctx, int64_t scene_begin, int64_t scene_end, const double* gravity_host) {
  if (!ctx) return MPM_ERR_BAD_ARG;
  if (!scene_range_ok(ctx, scene_begin, scene_end) || !gravity_host) return fail(ctx, MPM_ERR_BAD_ARG, "bad args");
  for (int64_t s = scene_begin; s < scene_end; ++s)
    for (int d = 0; d < 3; ++d) ctx->scenes_h[s].grav[d] = (float)gravity_host[(s - scene_begin) * 3 + d];
  CK(cudaSetDevice(ctx->device));
  CK(cudaMemcpyAsync(ctx->d_scenes + scene_begin, ctx->scenes_h.data() + scene_begin,
                     sizeof(SceneDev) * (scene_end - scene_begin), cudaMemcpyHostToDevice, ctx->cs));
  CK(cudaStreamSynchronize(ctx->cs));
  return MPM_OK;
}

int mpm_substeps(mpm_ctx* ctx, int32_t n_substeps, void* stream) {
  NvtxRange nvtx_range("mpm_substeps");
  if (!ctx) return MPM_ERR_BAD_ARG;
  if (n_substeps < 0) return fail(ctx, MPM_ERR_BAD_ARG, "negative substep count");
  if (ctx->phase != 0) return fail(ctx, MPM_ERR_STATE, "mpm_substeps inside a split substep");
  if (n_substeps == 0) return MPM_OK;
  int r = enter(ctx, stream);
  if (r) return r;
  if (!ctx->sorted && (r = launch_rekey(ctx, ctx->cs))) return r;
  int left = n_substeps;
  const bool graph = ctx->use_graph && !ctx->profiling && left >= 2;
  if (graph) {
    if (ctx->cur == 1) {
      if ((r = launch_substep(ctx, 1, ctx->cs))) return r;
      ctx->cur = 0;
      ctx->n_phys = ctx->n;
      --left;
    }
    if (left >= 2) {
      if ((r = ensure_graph(ctx))) return r;
      for (int i = 0; i + 1 < left; i += 2) CK(cudaGraphLaunch(ctx->gexec, ctx->cs));
      left &= 1;
    }
  }
  while (left-- > 0) {
    if ((r = launch_substep(ctx, ctx->cur, ctx->cs))) return r;
    ctx->cur ^= 1;
    ctx->n_phys = ctx->n;
  }
  ctx->n_phys = ctx->n;
  return leave(ctx, stream);
}

int mpm_substep_pre(mpm_ctx* ctx, void* stream) {
  NvtxRange nvtx_range("mpm_substep_pre");
  if (!ctx) return MPM_ERR_BAD_ARG;
  if (ctx->phase != 0) return fail(ctx, MPM_ERR_STATE, "substep_pre called twice");
  int r = enter(ctx, stream);
  if (r) return r;
  if (!ctx->sorted && (r = launch_rekey(ctx, ctx->cs))) return r;
  if ((r = launch_pre(ctx, ctx->cur, ctx->cs))) return r;
  ctx->phase = 1;
  return leave(ctx, stream);
}

int mpm_substep_grid_op(mpm_ctx* ctx, void* stream) {
  NvtxRange nvtx_range("mpm_substep_grid_op");
  if (!ctx) return MPM_ERR_BAD_ARG;
  if (ctx->phase != 1) return fail(ctx, MPM_ERR_STATE, "grid_op must follow substep_pre");
  int r = enter(ctx, stream);
  if (r) return r;
  if ((r = launch_grid(ctx, ctx->cur, ctx->cs))) return r;
  ctx->phase = 2;
  return leave(ctx, stream);
}

int mpm_substep_grid_stage(mpm_ctx* ctx, int32_t stage, int32_t ff_begin, int32_t ff_end, void* stream) {
  NvtxRange nvtx_range("mpm_substep_grid_stage");
  if (!ctx) return MPM_ERR_BAD_ARG;
  if (stage < 1 || stage > 3) return fail(ctx, MPM_ERR_BAD_ARG, "grid stage must be 1, 2 or 3");
  if (ff_begin < 0 || ff_begin > ff_end || ff_end > ctx->n_ffs)
    return fail(ctx, MPM_ERR_BAD_ARG, "force-field range outside the fields set");
  if (stage == 1 ? ctx->phase != 1 : ctx->phase != 3)
    return fail(ctx, MPM_ERR_STATE, stage == 1 ? "grid stage 1 must follow substep_pre"
                                               : "grid stages 2 and 3 must follow stage 1");
  int r = enter(ctx, stream);
  if (r) return r;
  if ((r = launch_grid(ctx, ctx->cur, ctx->cs, stage, ff_begin, ff_end))) return r;
  ctx->phase = stage == 3 ? 2 : 3;
  return leave(ctx, stream);
}

int mpm_grid_nodes(mpm_ctx* ctx, float** nodes, int64_t* n_nodes) {
  if (!ctx || !nodes || !n_nodes) return MPM_ERR_BAD_ARG;
  if (ctx->phase == 0) return fail(ctx, MPM_ERR_STATE, "the grid exists between substep_pre and substep_post");
  *nodes = reinterpret_cast<float*>(ctx->d_grid[ctx->cur]);
  *n_nodes = ctx->K * BLK_NODES;
  return MPM_OK;
}

int mpm_grid_node_positions(mpm_ctx* ctx, float* pos, int32_t* scene, void* stream) {
  NvtxRange nvtx_range("mpm_grid_node_positions");
  if (!ctx || !pos) return MPM_ERR_BAD_ARG;
  int r = enter(ctx, stream);
  if (r) return r;
  KParams P = make_params(ctx, ctx->cur, ctx->cur, ctx->cur);
  k_node_positions<<<ctx->n_sm * 8, 256, 0, ctx->cs>>>(P, pos, scene);
  CKL();
  return leave(ctx, stream);
}

int mpm_substep_post(mpm_ctx* ctx, void* stream) {
  NvtxRange nvtx_range("mpm_substep_post");
  if (!ctx) return MPM_ERR_BAD_ARG;
  if (ctx->phase != 2) return fail(ctx, MPM_ERR_STATE, "substep_post must follow grid_op");
  int r = enter(ctx, stream);
  if (r) return r;
  if ((r = launch_post(ctx, ctx->cur, ctx->cs))) return r;
  ctx->cur ^= 1;
  ctx->n_phys = ctx->n;
  ctx->phase = 0;
  return leave(ctx, stream);
}

int mpm_get_grid(mpm_ctx* ctx, int64_t scene, float* out, void* stream) {
  NvtxRange nvtx_range("mpm_get_grid");
  if (!ctx) return MPM_ERR_BAD_ARG;
  if (scene < 0 || scene >= ctx->n_scenes || !out) return fail(ctx, MPM_ERR_BAD_ARG, "bad args");
  const int g = ctx->phase == 0 ? (ctx->cur ^ 1) : ctx->cur;
  int r = enter(ctx, stream);
  if (r) return r;
  KParams P = make_params(ctx, ctx->cur, ctx->cur, g);
  P.fuse_grid = (ctx->phase == 0 && ctx->grid_momentum[g]) ? 1 : 0;
  k_get_grid<<<ctx->n_sm * 8, 256, 0, ctx->cs>>>(P, scene, out);
  CKL();
  return leave(ctx, stream);
}

constexpr int32_t MAX_COLLIDERS = 256;
constexpr int32_t MAX_FORCE_FIELDS = 64;

int mpm_set_force_fields(mpm_ctx* ctx, int32_t n, const mpm_force_field* fields) {
  if (!ctx) return MPM_ERR_BAD_ARG;
  if (n < 0 || n > MAX_FORCE_FIELDS || (n > 0 && !fields)) return fail(ctx, MPM_ERR_BAD_ARG, "bad force-field arguments");
  if (ctx->phase != 0) return fail(ctx, MPM_ERR_STATE, "force fields inside a substep");
  std::vector<ForceFieldDev> h((size_t)n);
  for (int32_t i = 0; i < n; ++i)
    if (!force_field_dev(fields[i], h[(size_t)i])) return fail(ctx, MPM_ERR_BAD_ARG, "unknown force field");
  CK(cudaSetDevice(ctx->device));
  if (!ctx->d_ffs && n > 0) {
    cudaError_t e = cudaMalloc((void**)&ctx->d_ffs, sizeof(ForceFieldDev) * MAX_FORCE_FIELDS);
    if (e == cudaSuccess) e = cudaMalloc((void**)&ctx->d_ff_step, sizeof(unsigned long long));
    if (e != cudaSuccess) {
      cudaGetLastError();
      return fail(ctx, MPM_ERR_OOM, "force-field table allocation failed");
    }
    drop_graph(ctx);  // captured substeps now advance the noise counter
  }
  if (ctx->d_ff_step) CK(cudaMemsetAsync(ctx->d_ff_step, 0, sizeof(unsigned long long), ctx->cs));
  if (n > 0) {
    CK(cudaMemcpyAsync(ctx->d_ffs, h.data(), sizeof(ForceFieldDev) * n, cudaMemcpyHostToDevice, ctx->cs));
    CK(cudaStreamSynchronize(ctx->cs));
  }
  if (n != ctx->n_ffs) drop_graph(ctx);  // the count is a captured kernel argument
  ctx->n_ffs = n;
  return MPM_OK;
}

int mpm_set_colliders(mpm_ctx* ctx, int32_t n, const mpm_collider* colliders) {
  NvtxRange nvtx_range("mpm_set_colliders");
  if (!ctx) return MPM_ERR_BAD_ARG;
  if (n < 0 || n > MAX_COLLIDERS || (n > 0 && !colliders)) return fail(ctx, MPM_ERR_BAD_ARG, "bad collider arguments");
  if (ctx->phase != 0) return fail(ctx, MPM_ERR_STATE, "colliders inside a substep");
  std::vector<ColliderDev> h((size_t)n);
  for (int32_t i = 0; i < n; ++i) {
    const mpm_collider& c = colliders[i];
    if (c.scene < -1 || c.scene >= ctx->n_scenes) return fail(ctx, MPM_ERR_BAD_ARG, "collider scene out of range");
    if (ctx->cpic_slots > 0 && i >= ctx->cpic_slots)
      return fail(ctx, MPM_ERR_BAD_ARG, "more colliders than CPIC slots (mpm_enable_cpic)");
    if (const char* e = collider_dev(ctx, c, h[(size_t)i])) return fail(ctx, MPM_ERR_BAD_ARG, e);
  }
  int32_t n_tools = 0;
  for (int32_t i = 0; i < n; ++i) n_tools += colliders[i].type == MPM_COLLIDER_TOOL ? 1 : 0;
  CK(cudaSetDevice(ctx->device));
  if (!ctx->d_colliders && n > 0) {
    cudaError_t e = cudaMalloc((void**)&ctx->d_colliders, sizeof(ColliderDev) * MAX_COLLIDERS);
    if (e == cudaSuccess) e = cudaMalloc((void**)&ctx->d_collider_acc, sizeof(double) * 6 * MAX_COLLIDERS);
    if (e != cudaSuccess) return fail(ctx, MPM_ERR_OOM, "collider table allocation failed");
  }
  if (n > 0) {
    CK(cudaMemcpyAsync(ctx->d_colliders, h.data(), sizeof(ColliderDev) * n, cudaMemcpyHostToDevice, ctx->cs));
    CK(cudaMemsetAsync(ctx->d_collider_acc, 0, sizeof(double) * 6 * MAX_COLLIDERS, ctx->cs));
    CK(cudaStreamSynchronize(ctx->cs));
  }
  if (n != ctx->n_colliders || (n_tools > 0) != (ctx->n_tools > 0)) drop_graph(ctx);  // captured kernel arguments
  ctx->n_colliders = n;
  ctx->n_tools = n_tools;
  return MPM_OK;
}

int mpm_add_sdf_grid(mpm_ctx* ctx, const int32_t* res, const float* values, const float* grads,
                     const double* T_mesh_to_sdf, double cell_size, double sdf_max, int32_t* id_out) {
  if (!ctx) return MPM_ERR_BAD_ARG;
  if (!res || !values || !T_mesh_to_sdf || !id_out) return fail(ctx, MPM_ERR_BAD_ARG, "null SDF grid argument");
  if (res[0] < 2 || res[1] < 2 || res[2] < 2 || (int64_t)res[0] * res[1] * res[2] > (int64_t)1 << 30)
    return fail(ctx, MPM_ERR_BAD_ARG, "SDF grid resolution must be >= 2 per axis");
  if (!(cell_size > 0)) return fail(ctx, MPM_ERR_BAD_ARG, "SDF cell_size must be > 0");
  if (ctx->phase != 0) return fail(ctx, MPM_ERR_STATE, "SDF grid inside a substep");
  const size_t nv = (size_t)res[0] * res[1] * res[2];
  mpm_ctx::SdfGrid g;
  for (int k = 0; k < 3; ++k) g.res[k] = res[k];
  for (int k = 0; k < 16; ++k) g.T[k] = T_mesh_to_sdf[k];
  g.cell_size = cell_size;
  g.sdf_max = sdf_max;
  CK(cudaSetDevice(ctx->device));
  cudaError_t e = cudaMalloc((void**)&g.val, sizeof(float) * nv);
  if (e == cudaSuccess && grads) e = cudaMalloc((void**)&g.grad, sizeof(float) * 3 * nv);
  if (e != cudaSuccess) {
    if (g.val) cudaFree(g.val);
    cudaGetLastError();
    return fail(ctx, MPM_ERR_OOM, "SDF grid allocation failed");
  }
  e = cudaMemcpy(g.val, values, sizeof(float) * nv, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && grads) e = cudaMemcpy(g.grad, grads, sizeof(float) * 3 * nv, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(g.val);
    if (g.grad) cudaFree(g.grad);
    return fail(ctx, MPM_ERR_CUDA, std::string("SDF grid upload: ") + cudaGetErrorString(e));
  }
  ctx->sdf_grids.push_back(g);
  *id_out = (int32_t)ctx->sdf_grids.size() - 1;
  return MPM_OK;
}

int mpm_get_collider_poses(mpm_ctx* ctx, double* out_host, void* stream) {
  if (!ctx || !out_host) return MPM_ERR_BAD_ARG;
  if (ctx->n_colliders == 0) return MPM_OK;
  int r = enter(ctx, stream);
  if (r) return r;
  std::vector<ColliderDev> h((size_t)ctx->n_colliders);
  CK(cudaMemcpyAsync(h.data(), ctx->d_colliders, sizeof(ColliderDev) * h.size(), cudaMemcpyDeviceToHost, ctx->cs));
  CK(cudaStreamSynchronize(ctx->cs));
  for (size_t i = 0; i < h.size(); ++i) {
    for (int k = 0; k < 3; ++k) out_host[i * 7 + k] = h[i].pos[k];
    for (int k = 0; k < 4; ++k) out_host[i * 7 + 3 + k] = h[i].quat[k];
  }
  return leave(ctx, stream);
}

int mpm_enable_cpic(mpm_ctx* ctx, int32_t n_slots, void* stream) {
  if (!ctx) return MPM_ERR_BAD_ARG;
  if (n_slots < 0 || n_slots > MAX_COLLIDERS) return fail(ctx, MPM_ERR_BAD_ARG, "bad CPIC slot count");
  if (ctx->pool) return fail(ctx, MPM_ERR_BAD_ARG, "CPIC is not available in pool mode");
  if (ctx->phase != 0) return fail(ctx, MPM_ERR_STATE, "CPIC set-up inside a substep");
  if (n_slots > 0 && ctx->n_colliders > n_slots)
    return fail(ctx, MPM_ERR_BAD_ARG, "fewer CPIC slots than colliders");
  int r = enter(ctx, stream);
  if (r) return r;
  const size_t cap = (size_t)ctx->cap;
  const int nf_new = n_slots > 0 ? NF_MUSCLE + 3 * n_slots : ctx->nf;
  if (nf_new > ctx->nf) {  // grow both particle buffers; the current one keeps its planes
    float* nb[2] = {nullptr, nullptr};
    for (int b = 0; b < 2; ++b) {
      cudaError_t e = cudaMalloc((void**)&nb[b], sizeof(float) * (size_t)nf_new * cap);
      if (e != cudaSuccess) {
        cudaGetLastError();
        if (nb[0]) cudaFree(nb[0]);
        return fail(ctx, MPM_ERR_OOM, "CPIC particle planes: " + std::string(cudaGetErrorString(e)));
      }
    }
    float* cur = nb[ctx->cur];
    CK(cudaMemcpyAsync(cur, ctx->d_pbuf[ctx->cur], sizeof(float) * (size_t)ctx->nf * cap, cudaMemcpyDeviceToDevice,
                       ctx->cs));
    if (ctx->nf == NF_BASE) {  // muscle planes at their defaults: actu 0, direction (0, 0, 1)
      k_fill_plane<<<ctx->io_blocks, 256, 0, ctx->cs>>>(cur + (size_t)PF_ACTU * cap, (int64_t)(3 * cap), 0.f);
      k_fill_plane<<<ctx->io_blocks, 256, 0, ctx->cs>>>(cur + (size_t)(PF_MDIR + 2) * cap, (int64_t)cap, 1.f);
      CKL();
    }
    CK(cudaStreamSynchronize(ctx->cs));
    for (int b = 0; b < 2; ++b) {
      for (void*& a : ctx->allocs)
        if (a == (void*)ctx->d_pbuf[b]) a = (void*)nb[b];
      cudaFree(ctx->d_pbuf[b]);
      ctx->d_pbuf[b] = nb[b];
    }
    ctx->nf = nf_new;
  }
  if (n_slots > 0) {  // the normals start at zero (LegacyCoupler.reset, legacy_coupler.py:114)
    CK(cudaMemsetAsync(ctx->d_pbuf[ctx->cur] + (size_t)PF_CPIC * cap, 0, sizeof(float) * 3 * (size_t)n_slots * cap,
                       ctx->cs));
    if (!ctx->d_cpic_mask) {
      cudaError_t e = cudaMalloc((void**)&ctx->d_cpic_mask, sizeof(uint32_t) * cap);
      if (e != cudaSuccess) {
        cudaGetLastError();
        ctx->d_cpic_mask = nullptr;
        return fail(ctx, MPM_ERR_OOM, "CPIC mask allocation failed");
      }
    }
  }
  ctx->cpic_slots = n_slots;
  drop_graph(ctx);  // kernel choice and plane count are captured
  if ((r = compute_launch_shapes(ctx))) return r;
  return leave(ctx, stream);
}

int mpm_set_coupled_particles(mpm_ctx* ctx, int32_t kind, int64_t n, const float* pos, float* vel, const float* mass,
                              const uint8_t* free_, void* stream) {
  if (!ctx) return MPM_ERR_BAD_ARG;
  if (kind != MPM_COUPLED_SPH && kind != MPM_COUPLED_PBD) return fail(ctx, MPM_ERR_BAD_ARG, "unknown coupled set");
  if (n < 0 || (n > 0 && (!pos || !vel || !mass))) return fail(ctx, MPM_ERR_BAD_ARG, "bad coupled particle arrays");
  if (n > 0 && n * ctx->n_scenes >= (int64_t)INT32_MAX) return fail(ctx, MPM_ERR_BAD_ARG, "too many coupled particles");
  if (ctx->pool) return fail(ctx, MPM_ERR_BAD_ARG, "particle coupling is not available in pool mode");
  if (ctx->phase != 0) return fail(ctx, MPM_ERR_STATE, "coupling set-up inside a substep");
  int r = enter(ctx, stream);
  if (r) return r;
  ExtSetDev& E = ctx->ext[kind];
  const int64_t total = n * ctx->n_scenes;
  if (n > 0 && !E.head) {
    const size_t nodes = (size_t)ctx->K * BLK_NODES;
    cudaError_t e = cudaMalloc((void**)&E.head, sizeof(int32_t) * nodes);
    if (e != cudaSuccess) {
      cudaGetLastError();
      E.head = nullptr;
      return fail(ctx, MPM_ERR_OOM, "coupling bins: " + std::string(cudaGetErrorString(e)));
    }
    CK(cudaMemsetAsync(E.head, 0xff, sizeof(int32_t) * nodes, ctx->cs));  // every list empty (-1)
  }
  if (total > ctx->ext_cap[kind]) {
    if (E.next) cudaFree(E.next);
    if (E.node) cudaFree(E.node);
    E.next = nullptr;
    E.node = nullptr;
    ctx->ext_cap[kind] = 0;
    cudaError_t e = cudaMalloc((void**)&E.next, sizeof(int32_t) * (size_t)total);
    if (e == cudaSuccess) e = cudaMalloc((void**)&E.node, sizeof(int64_t) * (size_t)total);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return fail(ctx, MPM_ERR_OOM, "coupling lists: " + std::string(cudaGetErrorString(e)));
    }
    ctx->ext_cap[kind] = total;
  }
  const uint8_t* fr = kind == MPM_COUPLED_PBD ? free_ : nullptr;
  const bool changed = E.n != n || E.pos != pos || E.vel != vel || E.mass != mass || E.free_ != fr;
  E.pos = pos;
  E.vel = vel;
  E.mass = mass;
  E.free_ = fr;
  E.n = n;
  if (changed) drop_graph(ctx);  // the arrays are captured kernel arguments
  return leave(ctx, stream);
}

int mpm_get_collider_forces(mpm_ctx* ctx, double* out_host, int32_t reset, void* stream) {
  if (!ctx || !out_host) return MPM_ERR_BAD_ARG;
  if (ctx->n_colliders == 0) return MPM_OK;
  int r = enter(ctx, stream);
  if (r) return r;
  CK(cudaMemcpyAsync(out_host, ctx->d_collider_acc, sizeof(double) * 6 * ctx->n_colliders, cudaMemcpyDeviceToHost,
                     ctx->cs));
  if (reset) CK(cudaMemsetAsync(ctx->d_collider_acc, 0, sizeof(double) * 6 * MAX_COLLIDERS, ctx->cs));
  CK(cudaStreamSynchronize(ctx->cs));
  return leave(ctx, stream);
}

static int ensure_constraints(mpm_ctx* ctx) {
  if (ctx->d_cons) return MPM_OK;
  if (ctx->pool) return fail(ctx, MPM_ERR_BAD_ARG, "particle constraints are not available in pool mode");
  cudaError_t e = cudaMalloc((void**)&ctx->d_cons, sizeof(ConstraintDev) * (size_t)ctx->cap);
  if (e != cudaSuccess) {
    ctx->d_cons = nullptr;
    return fail(ctx, MPM_ERR_OOM, "constraint table allocation failed");
  }
  CK(cudaMemsetAsync(ctx->d_cons, 0, sizeof(ConstraintDev) * (size_t)ctx->cap, ctx->cs));
  drop_graph(ctx);  // substeps now launch the constraint kernel
  return MPM_OK;
}

int mpm_set_particle_constraints(mpm_ctx* ctx, int64_t scene_begin, int64_t scene_end, int64_t particle_start,
                                 int64_t n, const uint8_t* mask, double stiffness, int32_t link_idx,
                                 const float* link_pos, const float* link_quat, void* stream) {
  if (!ctx) return MPM_ERR_BAD_ARG;
  if (!scene_range_ok(ctx, scene_begin, scene_end)) return fail(ctx, MPM_ERR_BAD_ARG, "bad scene range");
  if (ctx->phase != 0) return fail(ctx, MPM_ERR_STATE, "constraints inside a substep");
  if (n <= 0) return MPM_OK;
  if (!mask || !link_pos || !link_quat || particle_start < 0) return fail(ctx, MPM_ERR_BAD_ARG, "bad arguments");
  int r = enter(ctx, stream);
  if (r) return r;
  if ((r = ensure_constraints(ctx))) return r;
  KParams P = make_params(ctx, ctx->cur, ctx->cur, ctx->cur);
  k_set_constraints<<<ctx->io_blocks, 256, 0, ctx->cs>>>(P, scene_begin, scene_end, particle_start, n, mask,
                                                          (float)stiffness, link_idx, link_pos, link_quat,
                                                          ctx->d_cons);
  CKL();
  return leave(ctx, stream);
}

int mpm_remove_particle_constraints(mpm_ctx* ctx, int64_t scene_begin, int64_t scene_end, int64_t particle_start,
                                    int64_t n, const uint8_t* mask, void* stream) {
  if (!ctx) return MPM_ERR_BAD_ARG;
  if (!scene_range_ok(ctx, scene_begin, scene_end)) return fail(ctx, MPM_ERR_BAD_ARG, "bad scene range");
  if (ctx->phase != 0) return fail(ctx, MPM_ERR_STATE, "constraints inside a substep");
  if (!ctx->d_cons || n <= 0) return MPM_OK;
  if (!mask || particle_start < 0) return fail(ctx, MPM_ERR_BAD_ARG, "bad arguments");
  int r = enter(ctx, stream);
  if (r) return r;
  KParams P = make_params(ctx, ctx->cur, ctx->cur, ctx->cur);
  k_remove_constraints<<<ctx->io_blocks, 256, 0, ctx->cs>>>(P, scene_begin, scene_end, particle_start, n, mask,
                                                             ctx->d_cons);
  CKL();
  return leave(ctx, stream);
}

int mpm_set_link_poses(mpm_ctx* ctx, int32_t n_links, const float* poses_host) {
  if (!ctx) return MPM_ERR_BAD_ARG;
  if (n_links < 0 || (n_links > 0 && !poses_host)) return fail(ctx, MPM_ERR_BAD_ARG, "bad arguments");
  CK(cudaSetDevice(ctx->device));
  const size_t count = (size_t)ctx->n_scenes * n_links * 7;
  if (n_links != ctx->n_links) {
    if (ctx->d_links) CK(cudaFree(ctx->d_links));
    ctx->d_links = nullptr;
    if (count > 0) {
      cudaError_t e = cudaMalloc((void**)&ctx->d_links, count * sizeof(float));
      if (e != cudaSuccess) {
        ctx->d_links = nullptr;
        ctx->n_links = 0;
        drop_graph(ctx);
        return fail(ctx, MPM_ERR_OOM, "link table allocation failed");
      }
    }
    ctx->n_links = n_links;
    drop_graph(ctx);  // the captured constraint launch holds the table pointer
  }
  if (count > 0) {
    CK(cudaMemcpyAsync(ctx->d_links, poses_host, count * sizeof(float), cudaMemcpyHostToDevice, ctx->cs));
    CK(cudaStreamSynchronize(ctx->cs));
  }
  return MPM_OK;
}

int mpm_test_wait_timeout(mpm_ctx* ctx, void* stream) {
  if (!ctx) return MPM_ERR_BAD_ARG;
  if (ctx->phase != 0) return fail(ctx, MPM_ERR_STATE, "wait test inside a substep");
  if (ctx->K + 2 <= SCAN_SINGLE_MAX) return fail(ctx, MPM_ERR_BAD_ARG, "context too small for the one-pass scan");
  int r = enter(ctx, stream);
  if (r) return r;
  KParams P = make_params(ctx, ctx->cur, ctx->cur, ctx->cur);
  P.scan_hold_tile0 = 1;
  P.scan_spin_limit = 1u << 12;
  k_scan_onepass<<<ctx->n_tiles, SCAN_THREADS, 0, ctx->cs>>>(P);
  CKL();
  ctx->sorted = false;  // offsets and work items are rebuilt before the next substep
  return leave(ctx, stream);
}

int mpm_sample_regular(int32_t shape, const double* pos, const double* size, double p_size, float* out,
                       int64_t capacity, int64_t* n_out, void* stream) {
  if (!pos || !size || !n_out || !(p_size > 0) || shape < 0 || shape > 2) return MPM_ERR_BAD_ARG;
  LatticeDev L;
  std::memset(&L, 0, sizeof(L));
  L.shape = shape;
  double ext[3];
  if (shape == 0) ext[0] = size[0], ext[1] = size[1], ext[2] = size[2];
  else if (shape == 1) ext[0] = ext[1] = ext[2] = 2 * size[0];
  else ext[0] = ext[1] = 2 * size[0], ext[2] = size[1];
  int64_t total_rows = 1;
  for (int d = 0; d < 3; ++d) {
    const double n = std::nearbyint(ext[d] / p_size);  // Python round(): half to even
    L.n[d] = n < 1 ? 1 : (int64_t)n;
    const double lower = pos[d] - ext[d] / 2, upper = pos[d] + ext[d] / 2;
    L.lo[d] = lower + 0.5 * p_size;
    L.hi[d] = upper - 0.5 * p_size;
    L.step[d] = L.n[d] > 1 ? (L.hi[d] - L.lo[d]) / (double)(L.n[d] - 1) : 0.0;
    L.center[d] = pos[d];
  }
  L.radius = shape == 0 ? 0.0 : size[0];
  total_rows = L.n[0] * L.n[1];
  if (L.n[0] * L.n[1] * L.n[2] > ((int64_t)1 << 40)) return MPM_ERR_BAD_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  int64_t* d_rows = nullptr;
  if (cudaMalloc((void**)&d_rows, sizeof(int64_t) * (size_t)total_rows) != cudaSuccess) {
    cudaGetLastError();
    return MPM_ERR_OOM;
  }
  const int blocks = (int)std::min<int64_t>((total_rows + 255) / 256, 4096);
  k_lattice_rows<<<blocks, 256, 0, s>>>(L, d_rows);
  std::vector<int64_t> rows((size_t)total_rows);
  cudaError_t e = cudaMemcpyAsync(rows.data(), d_rows, sizeof(int64_t) * (size_t)total_rows, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  int64_t total = 0;
  for (auto& c : rows) {  // exclusive scan
    const int64_t v = c;
    c = total;
    total += v;
  }
  *n_out = total;
  if (e == cudaSuccess && out && capacity >= total && total > 0) {
    e = cudaMemcpyAsync(d_rows, rows.data(), sizeof(int64_t) * (size_t)total_rows, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) k_lattice_fill<<<blocks, 256, 0, s>>>(L, d_rows, out);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  }
  cudaFree(d_rows);
  if (e != cudaSuccess) return MPM_ERR_CUDA;
  return (out && capacity < total) ? MPM_ERR_BAD_ARG : MPM_OK;
}

int mpm_render_fields(mpm_ctx* ctx, int64_t scene_begin, int64_t scene_end, float* pos_out, float* vel_out,
                      uint8_t* active_out, int64_t n_vverts, int32_t n_supports, const int32_t* support_idx,
                      const float* support_w, float* vvert_pos_out, uint8_t* vvert_active_out, void* stream) {
  NvtxRange nvtx_range("mpm_render_fields");
  if (!ctx) return MPM_ERR_BAD_ARG;
  if (!scene_range_ok(ctx, scene_begin, scene_end)) return fail(ctx, MPM_ERR_BAD_ARG, "bad scene range");
  if (ctx->phase != 0) return fail(ctx, MPM_ERR_STATE, "render fields inside a substep");
  if (!pos_out || !active_out) return fail(ctx, MPM_ERR_BAD_ARG, "pos_out and active_out are required");
  if (n_vverts < 0 || (n_vverts > 0 && (n_supports <= 0 || !support_idx || !support_w || !vvert_pos_out)))
    return fail(ctx, MPM_ERR_BAD_ARG, "bad visual-vertex arguments");
  int r = enter(ctx, stream);
  if (r) return r;
  KParams P = make_params(ctx, ctx->cur, ctx->cur, ctx->cur);
  k_get_state<<<ctx->io_blocks, 256, 0, ctx->cs>>>(P, scene_begin, scene_end, pos_out, vel_out, nullptr, nullptr,
                                                    nullptr, active_out);
  CKL();
  const SceneDev& last = ctx->scenes_h[scene_end - 1];
  const int64_t rows = last.p_begin + last.n_particles - ctx->scenes_h[scene_begin].p_begin;
  if (n_vverts > 0) {
    k_render_vverts<<<ctx->io_blocks, 256, 0, ctx->cs>>>(P, scene_begin, scene_end, pos_out, active_out, n_vverts,
                                                        n_supports, support_idx, support_w, vvert_pos_out,
                                                        vvert_active_out);
    CKL();
  }
  if (rows > 0) {
    k_render_nowhere<<<ctx->io_blocks, 256, 0, ctx->cs>>>(rows, active_out, pos_out);
    CKL();
  }
  return leave(ctx, stream);
}

int mpm_count_touched_nodes(mpm_ctx* ctx, int64_t* out_host, void* stream) {
  if (!ctx || !out_host) return MPM_ERR_BAD_ARG;
  const int g = ctx->phase == 0 ? (ctx->cur ^ 1) : ctx->cur;
  int r = enter(ctx, stream);
  if (r) return r;
  KParams P = make_params(ctx, ctx->cur, ctx->cur, g);
  CK(cudaMemsetAsync(ctx->d_tmp64, 0, sizeof(unsigned long long), ctx->cs));
  k_count_touched<<<ctx->n_sm * 8, 256, 0, ctx->cs>>>(P, ctx->d_tmp64);
  CKL();
  unsigned long long v = 0;
  CK(cudaMemcpyAsync(&v, ctx->d_tmp64, sizeof(v), cudaMemcpyDeviceToHost, ctx->cs));
  CK(cudaStreamSynchronize(ctx->cs));
  *out_host = (int64_t)v;
  return leave(ctx, stream);
}

int mpm_status_word(mpm_ctx* ctx, uint32_t* status_host, int64_t* fp64_svd_host, int32_t clear, void* stream) {
  if (!ctx) return MPM_ERR_BAD_ARG;
  int r = enter(ctx, stream);
  if (r) return r;
  uint32_t st = 0;
  unsigned long long f64 = 0;
  CK(cudaMemcpyAsync(&st, ctx->d_status, sizeof(st), cudaMemcpyDeviceToHost, ctx->cs));
  CK(cudaMemcpyAsync(&f64, ctx->d_fp64, sizeof(f64), cudaMemcpyDeviceToHost, ctx->cs));
  if (clear) {
    CK(cudaMemsetAsync(ctx->d_status, 0, sizeof(uint32_t), ctx->cs));
    CK(cudaMemsetAsync(ctx->d_fp64, 0, sizeof(unsigned long long), ctx->cs));
  }
  CK(cudaStreamSynchronize(ctx->cs));
  if (status_host) *status_host = st;
  if (fp64_svd_host) *fp64_svd_host = (int64_t)f64;
  return leave(ctx, stream);
}

int mpm_set_tuning(mpm_ctx* ctx, int32_t p2g_threads, int32_t particles_per_thread, int32_t use_graph,
                   int32_t g2p_threads) {
  if (!ctx) return MPM_ERR_BAD_ARG;
  if (p2g_threads < 64 || p2g_threads > P2G_MAX_THREADS || p2g_threads % 32 || particles_per_thread < 1 ||
      p2g_threads * particles_per_thread > P2G_MAX_CHUNK)
    return fail(ctx, MPM_ERR_BAD_ARG, "tuning out of range (threads 64..256 step 32, threads*ppt <= 1024)");
  if (ctx->phase != 0) return fail(ctx, MPM_ERR_STATE, "tuning inside a substep");
  if (g2p_threads != 0 && (g2p_threads < 64 || g2p_threads > 256 || g2p_threads % 32))
    return fail(ctx, MPM_ERR_BAD_ARG, "g2p threads out of range (64..256 step 32)");
  const int g2p_t = g2p_threads ? g2p_threads : ctx->g2p_threads;
  const bool changed = p2g_threads != ctx->p2g_threads || particles_per_thread != ctx->ppt || g2p_t != ctx->g2p_threads;
  ctx->g2p_threads = g2p_t;
  ctx->p2g_threads = p2g_threads;
  ctx->ppt = particles_per_thread;
  ctx->use_graph = use_graph != 0;
  if (changed) {
    drop_graph(ctx);
    ctx->sorted = false;  // work items depend on the chunk size
    CK(cudaSetDevice(ctx->device));
    return compute_launch_shapes(ctx);
  }
  return MPM_OK;
}

int mpm_get_info(const mpm_ctx* ctx, int64_t* n_particles, int64_t* n_blocks, int64_t* n_scenes) {
  if (!ctx) return MPM_ERR_BAD_ARG;
  if (n_particles) *n_particles = ctx->n;
  if (n_blocks) *n_blocks = ctx->K;
  if (n_scenes) *n_scenes = ctx->n_scenes;
  return MPM_OK;
}

int mpm_scene_grid_res(const mpm_ctx* ctx, int64_t scene, int32_t* res3_host) {
  if (!ctx || scene < 0 || scene >= ctx->n_scenes || !res3_host) return MPM_ERR_BAD_ARG;
  for (int d = 0; d < 3; ++d) res3_host[d] = ctx->scenes_h[scene].res[d];
  return MPM_OK;
}

int mpm_set_profiling(mpm_ctx* ctx, int32_t enable) {
  if (!ctx) return MPM_ERR_BAD_ARG;
  ctx->profiling = enable != 0;
  return MPM_OK;
}

int mpm_kernel_times(mpm_ctx* ctx, double* ms_host, int64_t* counts_host, int32_t reset) {
  if (!ctx) return MPM_ERR_BAD_ARG;
  CK(cudaSetDevice(ctx->device));
  CK(cudaStreamSynchronize(ctx->cs));
  for (auto& tp : ctx->pending) {
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, tp.a, tp.b));
    ctx->ktime_ms[tp.kind] += ms;
    ctx->kcount[tp.kind] += 1;
    ctx->ev_pool.push_back(tp.a);
    ctx->ev_pool.push_back(tp.b);
  }
  ctx->pending.clear();
  for (int k = 0; k < KT_N; ++k) {
    if (ms_host) ms_host[k] = ctx->ktime_ms[k];
    if (counts_host) counts_host[k] = ctx->kcount[k];
    if (reset) {
      ctx->ktime_ms[k] = 0;
      ctx->kcount[k] = 0;
    }
  }
  return MPM_OK;
}

// ------------------------------------------------------------------ pool mode (serving)
int mpm_ctx_create_pool(const mpm_pool_config* cfg, int32_t device, mpm_ctx** out) {
  if (!out || !cfg) return fail(nullptr, MPM_ERR_BAD_ARG, "null argument");
  *out = nullptr;
  if (cfg->max_scenes <= 0 || cfg->particle_capacity <= 0 || cfg->max_grid_res < 4 || cfg->max_materials_per_scene <= 0)
    return fail(nullptr, MPM_ERR_BAD_ARG, "invalid pool configuration");
  const int64_t bres = (cfg->max_grid_res + BLK - 1) / BLK;
  const int64_t max_blocks = bres * bres * bres;
  const int64_t K = cfg->max_scenes * max_blocks;
  const int64_t n_mats = cfg->max_scenes * (int64_t)cfg->max_materials_per_scene;
  if (K + 2 >= (int64_t)INT32_MAX / 2 || cfg->particle_capacity >= (int64_t)INT32_MAX / 2 ||
      n_mats > (int64_t)INFO_MAT_MASK)
    return fail(nullptr, MPM_ERR_BAD_ARG, "pool too large for one context");
  mpm_ctx* ctx = new mpm_ctx();
  ctx->device = device;
  ctx->pool = true;
  ctx->n_scenes = cfg->max_scenes;
  ctx->n_mats = n_mats;
  ctx->max_blocks = max_blocks;
  ctx->max_mats = cfg->max_materials_per_scene;
  ctx->nf = cfg->with_muscle ? NF_MUSCLE : NF_BASE;
  ctx->K = K;
  ctx->cap = ((cfg->particle_capacity + 63) / 64) * 64;
  ctx->n = ctx->n_phys = 0;
  ctx->slot_n.assign(cfg->max_scenes, 0);
  ctx->slot_live.assign(cfg->max_scenes, 0);
  ctx->mat_count_h.assign(cfg->max_scenes, 0);
  ctx->pbegin_h.assign(cfg->max_scenes + 1, 0);
  ctx->first_mat_h.resize(cfg->max_scenes);
  std::vector<int32_t> block_scene_h((size_t)K);
  mpm_scene_config c0;
  std::memset(&c0, 0, sizeof(c0));
  c0.substep_dt = 1e-4;
  c0.grid_density = (double)(cfg->max_grid_res - 1);
  c0.upper_bound[0] = c0.upper_bound[1] = c0.upper_bound[2] = 1.0;
  c0.particle_size = 1.0 / c0.grid_density;
  c0.mass_eps = 1.1920929e-7;
  for (int64_t s = 0; s < cfg->max_scenes; ++s) {
    SceneDev S;
    std::string err;
    derive_scene(c0, S, err);
    S.block_base = s * max_blocks;
    S.mat_begin = (int32_t)(s * cfg->max_materials_per_scene);
    ctx->scenes_h.push_back(S);
    ctx->first_mat_h[s] = S.mat_begin;
    for (int64_t b = 0; b < max_blocks; ++b) block_scene_h[(size_t)(s * max_blocks + b)] = (int32_t)s;
    for (int32_t j = 0; j < cfg->max_materials_per_scene; ++j) {
      mpm_material m;
      std::memset(&m, 0, sizeof(m));
      m.scene = (int32_t)s;
      m.rho = 1000.0;
      m.default_Jp = 1.0;
      ctx->mats_h.push_back(derive_material(m, c0));
    }
  }
  return ctx_alloc_init(ctx, device, block_scene_h, out);
}

int mpm_scene_admit(mpm_ctx* ctx, int64_t slot, const mpm_scene_config* scene, const mpm_material* materials,
                    int32_t n_materials, int64_t n, const float* pos, const int32_t* mat_local, int32_t n_substeps,
                    void* stream) {
  NvtxRange nvtx_range("mpm_scene_admit");
  if (!ctx || !scene || !materials || !pos) return MPM_ERR_BAD_ARG;
  if (!ctx->pool) return fail(ctx, MPM_ERR_STATE, "not a pool context");
  if (ctx->phase != 0) return fail(ctx, MPM_ERR_STATE, "admit inside a substep");
  if (slot < 0 || slot >= ctx->n_scenes || ctx->slot_live[slot]) return fail(ctx, MPM_ERR_BAD_ARG, "slot busy or out of range");
  if (n_materials <= 0 || n_materials > ctx->max_mats) return fail(ctx, MPM_ERR_BAD_ARG, "bad material count");
  if (n <= 0 || ctx->n_phys + n > ctx->cap) return fail(ctx, MPM_ERR_OOM, "particle pool full");
  SceneDev S;
  std::string err;
  if (int e = derive_scene(*scene, S, err)) return fail(ctx, e, err);
  if ((int64_t)S.bres[0] * S.bres[1] * S.bres[2] > ctx->max_blocks)
    return fail(ctx, MPM_ERR_BAD_ARG, "scene grid larger than the pool's per-slot grid");
  for (int32_t j = 0; j < n_materials; ++j) {
    if (materials[j].type < MPM_MAT_ELASTIC || materials[j].type > MPM_MAT_MUSCLE)
      return fail(ctx, MPM_ERR_BAD_ARG, "unknown material type");
    if (materials[j].type == MPM_MAT_MUSCLE && ctx->nf == NF_BASE)
      return fail(ctx, MPM_ERR_BAD_ARG, "pool created without muscle fields");
  }
  S.block_base = slot * ctx->max_blocks;
  S.mat_begin = (int32_t)(slot * ctx->max_mats);
  S.p_begin = 0;
  S.n_particles = n;
  int r = enter(ctx, stream);
  if (r) return r;
  ctx->scenes_h[slot] = S;
  for (int32_t j = 0; j < n_materials; ++j) {
    mpm_material m = materials[j];
    m.scene = (int32_t)slot;
    ctx->mats_h[S.mat_begin + j] = derive_material(m, *scene);
  }
  CK(cudaMemcpyAsync(ctx->d_scenes + slot, &ctx->scenes_h[slot], sizeof(SceneDev), cudaMemcpyHostToDevice, ctx->cs));
  CK(cudaMemcpyAsync(ctx->d_mats + S.mat_begin, &ctx->mats_h[S.mat_begin], sizeof(MaterialDev) * n_materials,
                     cudaMemcpyHostToDevice, ctx->cs));
  int32_t steps = n_substeps < 0 ? -1 : n_substeps;
  CK(cudaMemcpyAsync(ctx->d_steps + slot, &steps, sizeof(int32_t), cudaMemcpyHostToDevice, ctx->cs));
  KParams P = make_params(ctx, ctx->cur, ctx->cur, ctx->cur);
  const int64_t nb = (n + 255) / 256;
  k_admit<<<(unsigned)(nb < 65535 ? nb : 65535), 256, 0, ctx->cs>>>(P, (int32_t)slot, ctx->n_phys, n, pos, mat_local);
  CKL();
  CK(cudaStreamSynchronize(ctx->cs));  // the host records above must outlive the copies
  ctx->n_phys += n;
  ctx->n += n;
  ctx->slot_n[slot] = n;
  ctx->slot_live[slot] = 1;
  ctx->mat_count_h[slot] = n_materials;
  ctx->sorted = false;
  CK(cudaMemcpyAsync(ctx->d_n, &ctx->n, sizeof(int64_t), cudaMemcpyHostToDevice, ctx->cs));
  CK(cudaStreamSynchronize(ctx->cs));
  if ((r = upload_scan_tiles(ctx))) return r;
  if ((r = compute_launch_shapes(ctx))) return r;
  return leave(ctx, stream);
}

int mpm_scene_retire(mpm_ctx* ctx, int64_t slot, void* stream) {
  NvtxRange nvtx_range("mpm_scene_retire");
  if (!ctx) return MPM_ERR_BAD_ARG;
  if (!ctx->pool) return fail(ctx, MPM_ERR_STATE, "not a pool context");
  if (ctx->phase != 0) return fail(ctx, MPM_ERR_STATE, "retire inside a substep");
  if (slot < 0 || slot >= ctx->n_scenes || !ctx->slot_live[slot]) return fail(ctx, MPM_ERR_BAD_ARG, "slot not live");
  int r = enter(ctx, stream);
  if (r) return r;
  KParams P = make_params(ctx, ctx->cur, ctx->cur, ctx->cur);
  k_retire<<<ctx->io_blocks, 256, 0, ctx->cs>>>(P, (int32_t)slot);
  CKL();
  int32_t frozen = 0;
  CK(cudaMemcpyAsync(ctx->d_steps + slot, &frozen, sizeof(int32_t), cudaMemcpyHostToDevice, ctx->cs));
  // dead particles sort after every live one; the next P2G drops them (the slot's blocks are still
  // in the scan while its particles are re-keyed)
  if ((r = launch_rekey(ctx, ctx->cs))) return r;
  CK(cudaStreamSynchronize(ctx->cs));
  ctx->n -= ctx->slot_n[slot];
  ctx->slot_n[slot] = 0;
  ctx->slot_live[slot] = 0;
  if ((r = upload_scan_tiles(ctx))) return r;
  CK(cudaMemcpyAsync(ctx->d_n, &ctx->n, sizeof(int64_t), cudaMemcpyHostToDevice, ctx->cs));
  CK(cudaStreamSynchronize(ctx->cs));
  if ((r = compute_launch_shapes(ctx))) return r;
  return leave(ctx, stream);
}

int mpm_scene_steps_left(mpm_ctx* ctx, int32_t* out_host, void* stream) {
  if (!ctx || !out_host) return MPM_ERR_BAD_ARG;
  int r = enter(ctx, stream);
  if (r) return r;
  CK(cudaMemcpyAsync(out_host, ctx->d_steps, sizeof(int32_t) * ctx->n_scenes, cudaMemcpyDeviceToHost, ctx->cs));
  CK(cudaStreamSynchronize(ctx->cs));
  return leave(ctx, stream);
}

int mpm_version(void) { return 1; }

}  // extern "C"
