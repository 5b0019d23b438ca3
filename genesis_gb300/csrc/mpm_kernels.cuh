// mpm_kernels.cuh - device data layout and kernel declarations of the MLS-MPM substep.
//
// Layout in HBM (all scenes of a context share one set of buffers):
//  * particles: two buffers (ping-pong), each NF float planes of `cap` entries (SoA):
//      0-2 pos, 3-5 vel, 6-14 C (row-major), 15-23 F, 24 Jp, 25 info (bits), 26 pid (bits),
//      27 actu, 28-30 muscle direction (when a muscle material exists or CPIC is on),
//      31 + 3c .. 33 + 3c the CPIC normal of collider slot c (CPIC only).
//    info = global material index (bits 0-23) | ACTIVE | FREE | DEAD.
//    pid = particle index within its scene (reference particle order for get/set state).
//  * grid: two buffers of float4 nodes grouped in blocks of 4x4x4 nodes (1 KiB each).
//    Global block id = scene.block_base + (bx*bres_y + by)*bres_z + bz; node address =
//    block*64 + (lx*4 + ly)*4 + lz.  Node = (momentum xyz, mass) after P2G and
//    (velocity xyz, mass) after the grid op.
//  * sort: particles are bucketed by the grid block that holds their stencil origin (the
//    cell index at 4^3 granularity).  Buckets [0,K) are grid blocks, K holds inactive
//    particles, K+1 particles of removed scenes.  key/rank come from G2P (warp-aggregated
//    atomics on count[]), with the particle's cell inside its block; an exclusive scan gives
//    bucket offsets and P2G work items; perm[new slot] = old slot drives the gather in the next
//    P2G and slot_cell[new slot] its per-cell counting sort.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "gbmpm.h"
#include "mpm_math.cuh"

namespace gbmpm {

constexpr int BLK = 4;                       // grid block edge (nodes)
constexpr int BLK_NODES = BLK * BLK * BLK;   // 64
constexpr int TILE = BLK + 2;                // P2G shared tile edge: block + stencil reach
constexpr int TILE_NODES = TILE * TILE * TILE;  // 216
constexpr int SCAN_TILE = 512;               // buckets per scan CTA (256 threads x 2)
constexpr int SCAN_THREADS = 256;
constexpr int64_t SCAN_SINGLE_MAX = 4096;     // bucket count up to which one CTA scans
constexpr int SVD_SWEEPS = 4;
constexpr int P2G_MAX_THREADS = 256;         // P2G CTA size limit (warp-private tiles)
constexpr int P2G_MAX_WARPS = P2G_MAX_THREADS / 32;
constexpr int P2G_MAX_CHUNK = 1024;          // particles per P2G work item

// Shared-memory layout of k_p2g (dynamic part): warp tiles, then one scatter record per particle
// at its cell-sorted position, then the item's (cell, rank) words and the old slots of its
// particles.  A record is P2G_REC float4: (q0, q1, q2, mass), (ax0, ax1, ay0, ay1),
// (az0, az1, ax2, ay2), (az2, fx, fy, fz), then the CPIC node mask in .x of the fifth (unused
// without CPIC; the odd stride of 5 float4 puts consecutive records in different bank groups),
// with a_k = dx * affine[:, k]: the pairs (q0, q1), (q2, mass), (ak0, ak1) sit in aligned register
// pairs for the scatter's paired FP32 operations.
constexpr int P2G_REC = 5;
__host__ __device__ __forceinline__ size_t p2g_dyn_smem(int threads, int chunk) {
  return (size_t)(threads / 32) * TILE_NODES * 16 + (size_t)chunk * P2G_REC * 16 + (size_t)chunk * 8;
}
constexpr float SVD_FP64_TOL = 1e-5f;        // accuracy bound of an FP32 SVD (svd_accurate); else FP64

enum : int {
  PF_POS = 0,
  PF_VEL = 3,
  PF_C = 6,
  PF_F = 15,
  PF_JP = 24,
  PF_INFO = 25,
  PF_PID = 26,
  PF_ACTU = 27,
  PF_MDIR = 28,
  NF_BASE = 27,
  NF_MUSCLE = 31,
  PF_CPIC = 31,  // CPIC: 3 planes (the particle-side normal) per collider slot after the muscle planes
};

constexpr uint32_t INFO_MAT_MASK = 0x00FFFFFFu;
constexpr uint32_t INFO_ACTIVE = 1u << 24;
constexpr uint32_t INFO_FREE = 1u << 25;
constexpr uint32_t INFO_DEAD = 1u << 26;

struct SceneDev {
  float dx, inv_dx, dt, stress_scale;  // stress_scale = -dt * p_vol * 4 * inv_dx^2
  float grav[3], eps;
  float lo[3], restitution;
  float hi[3], pad0;
  int32_t res[3], offset[3];  // grid nodes per axis; grid offset (cell index of node 0)
  int32_t bres[3], mat_begin; // blocks per axis; first global material of this scene
  int64_t block_base;         // first global block id of this scene
  int64_t p_begin;            // first output row of this scene (reference [B, N] layout)
  int64_t n_particles;
};

// Kinematic rigid collider of the grid op (mpm_collider in float).
struct ColliderDev {
  int32_t type, scene, pad0, pad1;
  float pos[3], quat[4], size[3], com[3], lin[3], ang[3];
  float friction, softness, restitution, pad2;
  // MPM_COLLIDER_SDF / MPM_COLLIDER_TOOL: voxel SDF grid (device arrays owned by the context)
  const float* val;   // [res0][res1][res2]
  const float* grad;  // [res0][res1][res2][3] (SDF) or null (tool)
  int32_t res[3], pad3;
  float T[12];        // rows 0..2 of T_mesh_to_sdf
  float Rinv[9];      // inverse of T[:3, :3] (tool normals back to the mesh frame)
  float cell_size, sdf_max, floor_h, pad4;
};

// External acceleration field of the grid op (mpm_force_field in float).
struct ForceFieldDev {
  int32_t type, active, pad0, pad1;
  float dir[3], center[3];
  float strength, radius, falloff_pow, flow, linear, quadratic;
  float s_perp, s_radial, falloff_min, falloff_max, damping, frequency;
  unsigned long long seed;  // NOISE
  uint8_t perm[3][256];     // TURBULENCE
};
// The device record of an ABI force field (float copies); false for an unknown type.
bool force_field_dev(const mpm_force_field& f, ForceFieldDev& d);
// The device record of an ABI collider (float copies, SDF grids from ctx); null, or the problem.
const char* collider_dev(const mpm_ctx* ctx, const mpm_collider& c, ColliderDev& d);

// Another solver's particles coupled through the grid op (SPH or PBD), caller-owned device arrays.
struct ExtSetDev {
  const float* pos;      // [n_scenes][n][3]
  float* vel;            // [n_scenes][n][3], updated in place
  const float* mass;     // [n_scenes][n]
  const uint8_t* free_;  // [n_scenes][n] (PBD) or null: every particle takes momentum
  int64_t n;             // particles per scene; 0: set unused
  int32_t* head;         // per grid node: first binned particle, -1 when empty
  int32_t* next;         // per particle: next particle of its node's list
  int64_t* node;         // per particle: node it was binned to, -1 if none
};

struct KParams {
  const SceneDev* scenes;
  const MaterialDev* mats;
  const int32_t* block_scene;  // [K]
  float* src;                  // particle planes read by P2G (old order)
  float* dst;                  // particle planes written by P2G / updated in place by G2P
  int64_t cap;
  int32_t nf;
  int32_t chunk;               // particles per P2G work item
  int64_t n;                   // particles in use (flat kernels outside a substep)
  const int64_t* n_dev;        // particles in use, read on the device by k_perm inside a substep
  int64_t K;                   // grid blocks (real buckets)
  float4* grid;                // grid buffer of this substep
  float4* grid_other;          // the other grid buffer (cleared by the grid op)
  int32_t* flags;              // [K] block touched in `grid`
  int32_t* flags_other;
  int32_t* list;               // active blocks of `grid`
  int32_t* nlist;
  int32_t* list_other;
  int32_t* nlist_other;
  int32_t* key;                // [cap]
  int32_t* rank;               // [cap]
  int32_t* count;              // [K+2]
  int32_t* offset;             // [K+2]
  int32_t* perm;               // [cap]
  uint8_t* cell8;              // [cap] cell of each particle in its block (old order; 64: none)
  uint8_t* slot_cell;          // [cap] the same in sorted-slot order (written by k_perm)
  int4* items;                 // P2G work items (bucket, begin, end, 0)
  int32_t* n_items;
  int2* partials;              // scan tile partials
  unsigned long long* scan_state;  // one-pass scan: per tile, flag (2 bits) | count (31) | items (31)
  int32_t* scan_sync;          // one-pass scan: [0] tile ticket, [1] finished tiles
  int32_t n_tiles;             // one-pass scan CTAs launched (at least the live tiles)
  const int2* scan_tiles;      // one-pass scan: bucket range [x, y) of each live tile, in bucket order
  const int32_t* n_scan_tiles; // live tiles (device; the launch's extra CTAs return at once)
  int32_t scan_hold_tile0;     // failure-detection test only: tile 0 never publishes
  uint32_t scan_spin_limit;    // look-back wait limit (0: the default)
  uint32_t* pin;               // per-node bitmap of nodes touched by non-free particles (or null)
  int32_t* steps;              // per-scene substeps left (-1 unlimited, 0 frozen); null outside a substep
  int32_t n_scenes;
  float eps_norm;              // gs.EPS for Matrix.norm(eps)
  uint32_t* status;
  unsigned long long* fp64_count;
  const ForceFieldDev* ffs;    // external acceleration fields applied by k_grid_op (n_ffs > 0)
  int32_t n_ffs;
  const ColliderDev* colliders;  // kinematic colliders applied by k_grid_op (n_colliders > 0)
  int32_t n_colliders;
  double* collider_acc;        // [n_colliders][6] reaction force and torque
  int32_t fuse_grid;           // G2P applies the grid op while staging its tile and clears the other buffer
  int32_t grid_stage;          // k_grid_op: 0 whole grid op; 1 momentum -> velocity + fields [ff_begin, ff_end);
                               // 2 fields [ff_begin, ff_end) on velocities; 3 colliders, coupling, boundary
  int32_t ff_begin, ff_end;    // the force fields k_grid_op applies (stage 0: all)
  int32_t* nlist_reset;        // active-list length that k_perm resets at the end of a fused substep
  int32_t cpic_slots;          // CPIC collider slots (normal planes PF_CPIC + 3 * slot); 0: CPIC off
  uint32_t* cpic_mask;         // CPIC: per slot, the particle's nodes behind a collider (bit ox*9+oy*3+oz)
  ExtSetDev ext[2];            // coupled particle sets: [0] SPH, [1] PBD (applied in that order)
  unsigned long long* ff_step; // substeps since the force fields were set (NOISE draws), or null
  int32_t ff_step_advance;     // k_perm counts the substep (set only for the end of a substep)
  ColliderDev* colliders_rw;   // k_perm advances the tools' poses at the end of a substep (else null)
};

// Programmatic dependent launch (the substep kernels are launched with programmatic stream
// serialisation): a kernel may start while its predecessor drains; pdl_wait() returns once the
// predecessor grid has completed and its writes are visible, and must come before any read of
// them; pdl_trigger() lets the successor start launching once every CTA of this grid has passed it.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// Block key of a world position; returns false if the stencil would leave the grid.
__device__ __forceinline__ bool stencil_origin(const SceneDev& S, const float* x, int* b) {
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    if (!isfinite(x[d])) return false;
    const float t = __fsub_rn(__fmul_rn(x[d], S.inv_dx), 0.5f);
    const float f = floorf(t);
    if (f < -1e9f || f > 1e9f) return false;
    b[d] = (int)f - S.offset[d];
    if (b[d] < 0 || b[d] > S.res[d] - 3) return false;
  }
  return true;
}

// Grid op of one node (legacy_coupler.py:356-501 with MPM alone): v = p/m + dt g where the node
// holds mass, then the free-slip separating boundary on node positions (boundaries.py:22-32).
// (gx, gy, gz) is the node index within its scene's grid.
__device__ __forceinline__ bool grid_free_velocity(const SceneDev& S, float4 q, float* v) {
  v[0] = v[1] = v[2] = 0.f;
  if (!(q.w > S.eps)) return false;
  const float inv = 1.f / q.w;
  v[0] = inv * q.x + S.dt * S.grav[0];
  v[1] = inv * q.y + S.dt * S.grav[1];
  v[2] = inv * q.z + S.dt * S.grav[2];
  return true;
}

__device__ __forceinline__ void grid_boundary(const SceneDev& S, float* v, int gx, int gy, int gz) {
  const int g[3] = {gx, gy, gz};
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const float pos = (float)(g[d] + S.offset[d]) * S.dx;
    if (pos >= S.hi[d] && v[d] >= 0.f) v[d] *= -S.restitution;
    else if (pos <= S.lo[d] && v[d] <= 0.f) v[d] *= -S.restitution;
  }
}

__device__ __forceinline__ float4 grid_velocity(const SceneDev& S, float4 q, int gx, int gy, int gz) {
  float v[3];
  if (grid_free_velocity(S, q, v)) grid_boundary(S, v, gx, gy, gz);
  return make_float4(v[0], v[1], v[2], q.w);
}

__device__ __forceinline__ int64_t block_of(const SceneDev& S, int gx, int gy, int gz) {
  return S.block_base + ((int64_t)(gx >> 2) * S.bres[1] + (gy >> 2)) * S.bres[2] + (gz >> 2);
}

__device__ __forceinline__ int64_t node_addr(const SceneDev& S, int gx, int gy, int gz) {
  return block_of(S, gx, gy, gz) * BLK_NODES + (((gx & 3) * 4 + (gy & 3)) * 4 + (gz & 3));
}

// ---------------------------------------------------------------- kernels
__global__ void k_init_particles(KParams P, const int64_t* scene_pbegin, const int32_t* scene_first_mat,
                                 int64_t n_scenes);
__global__ void k_add_particles(KParams P, int64_t s0, int64_t s1, int64_t start, int64_t n_add, int32_t mat_local,
                                int32_t active, const float* pos);
__global__ void k_admit(KParams P, int32_t s, int64_t n0, int64_t n_add, const float* pos, const int32_t* mat_local);
__global__ void k_retire(KParams P, int32_t s);
__global__ void k_get_state(KParams P, int64_t s0, int64_t s1, float* pos, float* vel, float* C, float* F,
                            float* Jp, uint8_t* active);
__global__ void k_set_state(KParams P, int64_t s0, int64_t s1, const float* pos, const float* vel, const float* C,
                            const float* F, const float* Jp, const uint8_t* active);
__global__ void k_row_slots(KParams P, int64_t s0, int64_t s1, int32_t* row_slot, uint32_t* row_info);
__global__ void k_get_state_rows(KParams P, int64_t rows, const int32_t* row_slot, const uint32_t* row_info,
                                 float* pos, float* vel, float* C, float* F, float* Jp, uint8_t* active);
__global__ void k_set_state_rows(KParams P, int64_t rows, const uint32_t* row_info, const float* pos,
                                 const float* vel, const float* C, const float* F, const float* Jp,
                                 const uint8_t* active);
__global__ void k_particles_field(KParams P, int field, int write, int64_t s0, int64_t s1, int64_t start,
                                  int64_t n_sel, float* data);
__global__ void k_g2p(KParams P);   // G2P + re-keying, over the P2G work items
__global__ void k_keys(KParams P);  // re-keying only (after a state change)
__global__ void k_scan_onepass(KParams P);
__global__ void k_scan_single(KParams P);
__global__ void k_perm(KParams P);
__global__ void k_p2g(KParams P);
__global__ void k_p2g_cpic(KParams P);  // k_p2g with CPIC (thin-collider separation)
__global__ void k_g2p_cpic(KParams P);  // k_g2p with CPIC
__global__ void k_grid_op(KParams P);
__global__ void k_fill_plane(float* p, int64_t n, float v);
__global__ void k_ext_bin(KParams P, int k, int unbin);
__global__ void k_get_grid(KParams P, int64_t scene, float* out);
__global__ void k_node_positions(KParams P, float* pos, int32_t* scene);
// Soft particle-to-link constraint of one reference particle row (mpm_solver.py:1052-1128).
struct ConstraintDev {
  float local[3];   // offset in the link frame at attachment
  float target[3];  // current target position
  float stiffness;
  int32_t link;     // kinematic link index, or -1 (target stays where it was set)
  int32_t on;
  int32_t pad;
};
__global__ void k_set_constraints(KParams P, int64_t s0, int64_t s1, int64_t start, int64_t n, const uint8_t* mask,
                                  float stiffness, int32_t link, const float* link_pos, const float* link_quat,
                                  ConstraintDev* cons);
__global__ void k_remove_constraints(KParams P, int64_t s0, int64_t s1, int64_t start, int64_t n,
                                     const uint8_t* mask, ConstraintDev* cons);
__global__ void k_constraints(KParams P, ConstraintDev* cons, const float* links, int32_t n_links);
// Regular-lattice particle sampling on the device (utils/particle.py:180-278, 'regular' sampler).
struct LatticeDev {
  double lo[3], step[3], hi[3];  // per axis: first point, spacing, last point (np.linspace)
  int64_t n[3];
  int32_t shape;                 // 0 box, 1 sphere, 2 cylinder (z axis)
  int32_t pad;
  double center[3], radius;
};
__global__ void k_lattice_rows(LatticeDev L, int64_t* row_count);
__global__ void k_lattice_fill(LatticeDev L, const int64_t* row_offset, float* out);
__global__ void k_render_vverts(KParams P, int64_t s0, int64_t s1, const float* pos, const uint8_t* active,
                                int64_t n_vverts, int32_t n_supports, const int32_t* support_idx,
                                const float* support_w, float* vpos, uint8_t* vactive);
__global__ void k_render_nowhere(int64_t rows, const uint8_t* active, float* pos);
__global__ void k_count_touched(KParams P, unsigned long long* out);

}  // namespace gbmpm
