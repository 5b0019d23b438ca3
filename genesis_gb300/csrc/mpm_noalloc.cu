// mpm_noalloc.cu - mpm_substeps_noalloc: MPM substeps of one small scene that allocate no
// device memory.
//
// Who needs it: callers that may not allocate device memory at all - plug-ins whose host
// application owns every device allocation through its own budgeted pool, and real-time
// control loops that forbid allocator calls after start-up (cudaMalloc and cudaFree may
// synchronise the device and take unbounded time).  They pass their own particle arrays
// (updated in place) and get the substeps without a context: the grid, which the other
// entry points keep in a context's cudaMalloc'd pool, lives here in a fixed file-scope
// device array that the library reserves when it is loaded.
//
// Limits and sharing:
//  * the grid may have at most NOALLOC_MAX_NODES = 524288 nodes (e.g. 80^3; the unit cube at
//    grid_density 64 has 65^3 = 274625); 8 MiB of device memory on every GPU that loads the
//    library, held until the process exits;  at most 16 materials, no muscle material;
//  * every call uses the same array, so calls that overlap on the GPU (different streams,
//    or different host threads without ordering) race on it; the grid is cleared at the
//    start of every substep and the status word at the start of every call;
//  * particles are not re-sorted (a plain scatter with global vector atomics), so this path
//    is meant for small scenes; the context entry points are the fast path.
// The first call on a device looks up the array's device address (cudaGetSymbolAddress)
// with that device current; make that first call before any stream capture.  The address is
// kept per device ordinal, for the device's primary context (the one the CUDA runtime and
// PyTorch use); callers that drive the device through contexts of their own made with
// cuCtxCreate are not supported.  Every call ends by synchronising its stream to read the
// status word.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "gbmpm.h"
#include "mpm_kernels.cuh"

namespace gbmpm {
namespace {

constexpr int64_t NOALLOC_MAX_NODES = 524288;
constexpr int NOALLOC_MAX_MATERIALS = 16;
constexpr int NOALLOC_MAX_DEVICES = 64;

// The scratch: grid nodes (momentum xyz, mass) then (velocity xyz, mass), plus one status word.
static __device__ __align__(256) float4 g_noalloc_grid[NOALLOC_MAX_NODES];
static __device__ __align__(256) uint32_t g_noalloc_status[64];

struct NoallocParams {
  float4* grid;        // device address of g_noalloc_grid
  uint32_t* status;    // device address of g_noalloc_status
  SceneDev S;
  MaterialDev mats[NOALLOC_MAX_MATERIALS];
  int32_t n_mats;
  int64_t n;
  float* pos;
  float* vel;
  float* C;
  float* F;
  float* Jp;
  const int32_t* mat;
  const uint8_t* active;
  float eps;
};

__device__ __forceinline__ int64_t dense_index(const SceneDev& S, int gx, int gy, int gz) {
  return ((int64_t)gx * S.res[1] + gy) * S.res[2] + gz;
}

__global__ void k_na_clear(NoallocParams Q, int64_t nodes, int clear_status) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nodes; i += (int64_t)gridDim.x * blockDim.x)
    Q.grid[i] = make_float4(0.f, 0.f, 0.f, 0.f);
  if (clear_status && blockIdx.x == 0 && threadIdx.x == 0) Q.status[0] = 0u;
}

// compute_F_tmp + svd + material + stress + APIC scatter (mpm_solver.py:293-421), unsorted.
__global__ void __launch_bounds__(256) k_na_p2g(NoallocParams Q) {
  const SceneDev& S = Q.S;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < Q.n; i += (int64_t)gridDim.x * blockDim.x) {
    if (Q.active && !Q.active[i]) continue;
    const int m = Q.mat ? Q.mat[i] : 0;
    if (m < 0 || m >= Q.n_mats) {
      atomicOr(Q.status, 2u);
      continue;
    }
    const MaterialDev& M = Q.mats[m];
    float x[3], v[3], C[9], F[9];
    for (int d = 0; d < 3; ++d) {
      x[d] = Q.pos[i * 3 + d];
      v[d] = Q.vel[i * 3 + d];
    }
    for (int k = 0; k < 9; ++k) {
      C[k] = Q.C[i * 9 + k];
      F[k] = Q.F[i * 9 + k];
    }
    int b[3];
    if (!stencil_origin(S, x, b)) {
      atomicOr(Q.status, (isfinite(x[0]) && isfinite(x[1]) && isfinite(x[2])) ? 2u : 1u);
      continue;
    }
    float A[9], Ft[9];
    for (int k = 0; k < 9; ++k) A[k] = ((k % 4 == 0) ? 1.f : 0.f) + S.dt * C[k];
    mat_mul(A, F, Ft);
    float U[9], sig[3], V[9];
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
    const float mdir[3] = {0.f, 0.f, 1.f};
    float Fn[9], Pk[9], Jpn;
    material_update<float>(M, Ft, U, sig, V, Q.Jp[i], 0.f, mdir, Q.eps, Fn, Jpn, Pk);
    for (int k = 0; k < 9; ++k) Q.F[i * 9 + k] = Fn[k];
    Q.Jp[i] = Jpn;
    const float mass = M.mass;
    float aff[9];
    for (int k = 0; k < 9; ++k) aff[k] = S.stress_scale * Pk[k] + mass * C[k];
    float fx[3], w[3][3];
    for (int d = 0; d < 3; ++d) {
      const float t = __fmul_rn(x[d], S.inv_dx);
      fx[d] = t - (float)(b[d] + S.offset[d]);
      bspline_w(fx[d], w[d]);
    }
    for (int ox = 0; ox < 3; ++ox)
      for (int oy = 0; oy < 3; ++oy)
        for (int oz = 0; oz < 3; ++oz) {
          const float wt = w[0][ox] * w[1][oy] * w[2][oz];
          const float dp[3] = {((float)ox - fx[0]) * S.dx, ((float)oy - fx[1]) * S.dx, ((float)oz - fx[2]) * S.dx};
          float4 g;
          g.x = wt * (mass * v[0] + aff[0] * dp[0] + aff[1] * dp[1] + aff[2] * dp[2]);
          g.y = wt * (mass * v[1] + aff[3] * dp[0] + aff[4] * dp[1] + aff[5] * dp[2]);
          g.z = wt * (mass * v[2] + aff[6] * dp[0] + aff[7] * dp[1] + aff[8] * dp[2]);
          g.w = wt * mass;
          atomicAdd(&Q.grid[dense_index(S, b[0] + ox, b[1] + oy, b[2] + oz)], g);
        }
  }
}

// legacy_coupler.py:356-501 without coupling partners.
__global__ void k_na_grid(NoallocParams Q, int64_t nodes) {
  const SceneDev& S = Q.S;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nodes; i += (int64_t)gridDim.x * blockDim.x) {
    const float4 q = Q.grid[i];
    float v[3] = {0.f, 0.f, 0.f};
    if (q.w > S.eps) {
      const int g[3] = {(int)(i / ((int64_t)S.res[1] * S.res[2])), (int)((i / S.res[2]) % S.res[1]), (int)(i % S.res[2])};
      const float inv = 1.f / q.w;
      v[0] = inv * q.x + S.dt * S.grav[0];
      v[1] = inv * q.y + S.dt * S.grav[1];
      v[2] = inv * q.z + S.dt * S.grav[2];
      for (int d = 0; d < 3; ++d) {
        const float p = (float)(g[d] + S.offset[d]) * S.dx;
        if (p >= S.hi[d] && v[d] >= 0.f) v[d] *= -S.restitution;
        else if (p <= S.lo[d] && v[d] <= 0.f) v[d] *= -S.restitution;
      }
    }
    Q.grid[i] = make_float4(v[0], v[1], v[2], q.w);
  }
}

// mpm_solver.py:423-481 with the particle boundary of boundaries.py:22-32.
__global__ void __launch_bounds__(256) k_na_g2p(NoallocParams Q) {
  const SceneDev& S = Q.S;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < Q.n; i += (int64_t)gridDim.x * blockDim.x) {
    if (Q.active && !Q.active[i]) continue;
    float x[3];
    for (int d = 0; d < 3; ++d) x[d] = Q.pos[i * 3 + d];
    int b[3];
    if (!stencil_origin(S, x, b)) continue;  // reported by k_na_p2g
    float fx[3], w[3][3];
    for (int d = 0; d < 3; ++d) {
      const float t = __fmul_rn(x[d], S.inv_dx);
      fx[d] = t - (float)(b[d] + S.offset[d]);
      bspline_w(fx[d], w[d]);
    }
    float v[3] = {0.f, 0.f, 0.f}, Cn[9];
    for (int k = 0; k < 9; ++k) Cn[k] = 0.f;
    for (int ox = 0; ox < 3; ++ox)
      for (int oy = 0; oy < 3; ++oy)
        for (int oz = 0; oz < 3; ++oz) {
          const float4 g = Q.grid[dense_index(S, b[0] + ox, b[1] + oy, b[2] + oz)];
          const float wt = w[0][ox] * w[1][oy] * w[2][oz];
          const float dp[3] = {(float)ox - fx[0], (float)oy - fx[1], (float)oz - fx[2]};
          const float gv[3] = {g.x, g.y, g.z};
          for (int r = 0; r < 3; ++r) {
            v[r] += wt * gv[r];
            const float s = 4.f * S.inv_dx * wt * gv[r];
            for (int c = 0; c < 3; ++c) Cn[r * 3 + c] += s * dp[c];
          }
        }
    bool finite = true;
    for (int d = 0; d < 3; ++d) {
      float xn = x[d] + S.dt * v[d];
      finite = finite && isfinite(xn) && isfinite(v[d]);
      if (xn >= S.hi[d] && v[d] >= 0.f) v[d] *= -S.restitution;
      else if (xn <= S.lo[d] && v[d] <= 0.f) v[d] *= -S.restitution;
      Q.pos[i * 3 + d] = fmaxf(fminf(xn, S.hi[d]), S.lo[d]);
      Q.vel[i * 3 + d] = v[d];
    }
    for (int k = 0; k < 9; ++k) Q.C[i * 9 + k] = Cn[k];
    if (!finite) atomicOr(Q.status, 1u);
  }
}

// Per-device device addresses of the scratch, looked up once with the device current.
std::mutex g_na_mu;
float4* g_na_grid_ptr[NOALLOC_MAX_DEVICES] = {};
uint32_t* g_na_status_ptr[NOALLOC_MAX_DEVICES] = {};
thread_local std::string g_na_err;  // text of the calling thread's last failed call

int na_fail(int code, const std::string& msg) {
  g_na_err = msg;
  return code;
}

}  // namespace
}  // namespace gbmpm

namespace gbmpm {
// Scene and material derivation shared with the context entry points (mpm_capi.cu).
int derive_scene(const mpm_scene_config& c, SceneDev& S, std::string& err);
MaterialDev derive_material(const mpm_material& m, const mpm_scene_config& c);
}  // namespace gbmpm

using namespace gbmpm;

extern "C" {

const char* mpm_noalloc_last_error(void) { return g_na_err.c_str(); }

int mpm_substeps_noalloc(const mpm_scene_config* scene, const mpm_material* materials, int32_t n_materials, int64_t n,
                         float* pos, float* vel, float* C, float* F, float* Jp, const int32_t* mat,
                         const uint8_t* active, int32_t n_substeps, void* stream) {
  if (!scene || !materials || n_materials <= 0) return na_fail(MPM_ERR_BAD_ARG, "scene and materials are required");
  if (n_materials > NOALLOC_MAX_MATERIALS) return na_fail(MPM_ERR_BAD_ARG, "more than 16 materials");
  if (n < 0 || n_substeps < 0) return na_fail(MPM_ERR_BAD_ARG, "negative particle or substep count");
  if (n > 0 && (!pos || !vel || !C || !F || !Jp)) return na_fail(MPM_ERR_BAD_ARG, "particle arrays are required");
  NoallocParams Q;
  std::memset(&Q, 0, sizeof(Q));
  std::string err;
  if (int e = derive_scene(*scene, Q.S, err)) return na_fail(e, err);
  const int64_t nodes = (int64_t)Q.S.res[0] * Q.S.res[1] * Q.S.res[2];
  if (nodes > NOALLOC_MAX_NODES)
    return na_fail(MPM_ERR_BAD_ARG, "grid of " + std::to_string(nodes) +
                                        " nodes exceeds the no-allocation limit of 524288 nodes (e.g. 80^3)");
  for (int32_t j = 0; j < n_materials; ++j) {
    if (materials[j].type < MPM_MAT_ELASTIC || materials[j].type > MPM_MAT_ELASTOPLASTIC)
      return na_fail(MPM_ERR_BAD_ARG, "material type not supported without a context (muscle needs one)");
    Q.mats[j] = derive_material(materials[j], *scene);
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return na_fail(MPM_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) return na_fail(MPM_ERR_BAD_ARG, "device index above 63");
  {
    std::lock_guard<std::mutex> lk(g_na_mu);
    if (!g_na_grid_ptr[dev]) {  // once per device, with that device current
      void* gp = nullptr;
      void* sp = nullptr;
      e = cudaGetSymbolAddress(&gp, g_noalloc_grid);
      if (e != cudaSuccess) return na_fail(MPM_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      e = cudaGetSymbolAddress(&sp, g_noalloc_status);
      if (e != cudaSuccess) return na_fail(MPM_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      g_na_grid_ptr[dev] = (float4*)gp;
      g_na_status_ptr[dev] = (uint32_t*)sp;
    }
    Q.grid = g_na_grid_ptr[dev];
    Q.status = g_na_status_ptr[dev];
  }
  Q.n_mats = n_materials;
  Q.n = n;
  Q.pos = pos;
  Q.vel = vel;
  Q.C = C;
  Q.F = F;
  Q.Jp = Jp;
  Q.mat = mat;
  Q.active = active;
  Q.eps = (float)scene->mass_eps;
  cudaStream_t s = (cudaStream_t)stream;
  const int pb = (int)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096);
  const int gb = (int)((nodes + 255) / 256 < 4096 ? (nodes + 255) / 256 : 4096);
  for (int32_t k = 0; k < n_substeps; ++k) {
    k_na_clear<<<gb, 256, 0, s>>>(Q, nodes, k == 0);
    if (n > 0) k_na_p2g<<<pb, 256, 0, s>>>(Q);
    k_na_grid<<<gb, 256, 0, s>>>(Q, nodes);
    if (n > 0) k_na_g2p<<<pb, 256, 0, s>>>(Q);
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return na_fail(MPM_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
  if (n_substeps == 0) return MPM_OK;
  uint32_t st = 0;
  e = cudaMemcpyAsync(&st, Q.status, sizeof(st), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return na_fail(MPM_ERR_CUDA, std::string("status read: ") + cudaGetErrorString(e));
  if (st & 1u) return na_fail(MPM_ERR_NAN, "NaN detected in MPM states");
  if (st & 2u) return na_fail(MPM_ERR_OOB, "a particle's stencil left the grid (particle skipped)");
  return MPM_OK;
}

}  // extern "C"
