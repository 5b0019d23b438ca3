/*
 * gbmpm.h - C ABI of the GB300-native MLS-MPM substep library (libgbmpm.so).
 *
 * The reference (Genesis, genesis-world 0.4.5) has no native FFI for this path: its MPM
 * solver is Python written as Quadrants kernels, and the "plugin" boundary is the Solver
 * protocol that genesis/engine/simulator.py calls.  Every entry point below names the
 * reference kernel or method it replaces (file:line, paths relative to the Genesis
 * project root).  The Python package genesis_gb300 binds these with ctypes; a Genesis
 * maintainer would bind them the same way, from genesis/engine/solvers/mpm_solver.py.
 *
 * Conventions
 *  - Every function returns an mpm_status code (0 = OK).  No C++ exception crosses the ABI.
 *  - Array arguments are DEVICE pointers unless the name ends in _host.  They use the
 *    reference's layouts: pos/vel [B, N, 3], C/F [B, N, 3, 3] row-major, Jp [B, N],
 *    active [B, N] (uint8), all float32, where B is a range of scenes ("envs") and N the
 *    per-scene particle count.  Ragged scenes are laid out back to back in scene order.
 *  - `stream` is a cudaStream_t passed as void*; NULL means the legacy default stream.
 *    Work is enqueued on it; no entry point synchronises the host unless it says so.
 *  - No pointer passed in is retained after the call returns, except the coupled particle
 *    arrays of mpm_set_coupled_particles (the other solver's live state, read every grid op).
 */
#ifndef GBMPM_H
#define GBMPM_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status codes */
typedef enum mpm_status {
  MPM_OK = 0,
  MPM_ERR_BAD_ARG = 1,   /* invalid argument / configuration (reference: gs.raise_exception) */
  MPM_ERR_CUDA = 2,      /* a CUDA runtime call failed; mpm_last_error() has the text */
  MPM_ERR_OOM = 3,       /* device allocation failed */
  MPM_ERR_NAN = 4,       /* NaN in particle positions (mpm_solver.py:542-546) */
  MPM_ERR_OOB = 5,       /* a particle's stencil left the grid; the particle was skipped */
  MPM_ERR_TIMEOUT = 6,   /* a bounded device wait gave up */
  MPM_ERR_STATE = 7      /* call not valid in the context's current state */
} mpm_status;

/* Bits of the device status word returned by mpm_status_word(). */
#define MPM_STATUS_NAN 0x1u
#define MPM_STATUS_OOB 0x2u
#define MPM_STATUS_WAIT 0x4u /* a bounded device-side wait ran out (internal error; results invalid) */
#define MPM_STATUS_BAD_INDEX 0x8u /* an index array passed to a kernel held an out-of-range entry (skipped) */

/* ---------------------------------------------------------------- materials */
/* Material models of genesis/engine/materials/MPM/*.py */
typedef enum mpm_material_type {
  MPM_MAT_ELASTIC = 0,       /* elastic.py:32-60 (corotation; flag NEOHOOKEAN for the alternative) */
  MPM_MAT_LIQUID = 1,        /* liquid.py:30-49 */
  MPM_MAT_SAND = 2,          /* sand.py:38-84 (Drucker-Prager) */
  MPM_MAT_SNOW = 3,          /* snow.py:42-74 */
  MPM_MAT_ELASTOPLASTIC = 4, /* elasto_plastic.py:40-71 (flag VON_MISES selects the von Mises branch) */
  MPM_MAT_MUSCLE = 5         /* muscle.py:39-53 (flag NEOHOOKEAN selects the passive model) */
} mpm_material_type;

#define MPM_MATF_NEOHOOKEAN 0x1
#define MPM_MATF_VON_MISES 0x2

/* One registered material.  The derived constants follow base.py:77-88 (mu, lam),
 * sand.py:40-45 (alpha, default Jp 0) and muscle.py:46-50 (stiffness = E); the caller
 * (the Python facade) computes them exactly as the reference does. */
typedef struct mpm_material {
  int32_t type;          /* mpm_material_type */
  int32_t flags;         /* MPM_MATF_* */
  int32_t scene;         /* scene this material belongs to */
  int32_t reserved;
  double mu, lam;        /* Lame parameters (Liquid: mu = 0 unless viscous) */
  double rho;            /* density */
  double default_Jp;     /* 1, or 0 for Sand */
  double friction_alpha; /* Sand: sqrt(2/3)*2 sin(phi)/(3 - sin(phi)) */
  double yield_lower, yield_higher;  /* Snow / ElastoPlastic clamp */
  double von_mises_yield_stress;     /* ElastoPlastic von Mises */
  double stiffness;      /* Muscle actuation stiffness (= E) */
} mpm_material;

/* ---------------------------------------------------------------- scenes */
/* One independent MPM scene (a reference "env").  Derived values follow
 * MPMSolver.__init__ (mpm_solver.py:32-80): dx = 1/grid_density,
 * grid_res = round(density*ub) - round(density*lb) + 1, grid_offset = round(density*lb),
 * particle_volume = particle_size^3 * 1e3, boundary = [lb + 3dx, ub - 3dx]. */
typedef struct mpm_scene_config {
  double substep_dt;      /* SimOptions.dt / substeps (base_solver.py:25) */
  double gravity[3];
  double lower_bound[3];
  double upper_bound[3];
  double grid_density;
  double particle_size;
  double mass_eps;        /* grid-op mass threshold; the reference uses gs.EPS (fp32: 2^-23) */
  double restitution;     /* CubeBoundary restitution, 0 in the reference */
  int64_t n_particles;    /* particle capacity of this scene */
} mpm_scene_config;

typedef struct mpm_ctx mpm_ctx;

/* Create a context owning all device state for n_scenes scenes and n_materials
 * materials on CUDA device `device`.
 * Replaces MPMSolver.__init__/build + init_particle_fields/init_grid_fields
 * (mpm_solver.py:32-80, 82-148, 201-241) and LegacyCoupler.build for MPM. */
int mpm_ctx_create(const mpm_scene_config* scenes, int64_t n_scenes,
                   const mpm_material* materials, int32_t n_materials,
                   int32_t device, mpm_ctx** out);

/* Free all device state.  Replaces nothing (Quadrants frees fields at exit). */
int mpm_ctx_destroy(mpm_ctx* ctx);

/* Text of the last error on this context (or of the last failed create if ctx is NULL). */
const char* mpm_last_error(const mpm_ctx* ctx);

/* Add `n` particles of material `material` (index among the scene's own materials, in
 * registration order, like Material.idx) to scenes [scene_begin, scene_end),
 * at per-scene particle indices [particle_start, particle_start + n), with the same
 * positions `pos` [n, 3] in every scene.  Sets v = 0, F = I, C = 0, Jp = default_Jp,
 * actu = 0, free = true, muscle direction (0,0,1).
 * Replaces MPMSolver._kernel_add_particles (mpm_solver.py:806-838). */
int mpm_add_particles(mpm_ctx* ctx, int64_t scene_begin, int64_t scene_end,
                      int64_t particle_start, int64_t n, int32_t material, int32_t active,
                      const float* pos, void* stream);

/* Full particle state of scenes [scene_begin, scene_end) in reference layout.
 * Replaces MPMSolver._kernel_get_state / _kernel_set_state (mpm_solver.py:759-778,
 * 729-749) and MPMEntity.get_frame (mpm_entity.py:305-352).  Any pointer may be NULL to
 * skip that field.  set_state marks the particle ordering dirty (re-sorted before the
 * next substep). */
int mpm_get_state(mpm_ctx* ctx, int64_t scene_begin, int64_t scene_end,
                  float* pos, float* vel, float* C, float* F, float* Jp, uint8_t* active,
                  void* stream);
int mpm_set_state(mpm_ctx* ctx, int64_t scene_begin, int64_t scene_end,
                  const float* pos, const float* vel, const float* C, const float* F,
                  const float* Jp, const uint8_t* active, void* stream);

/* Per-particle field access over a contiguous per-scene particle range
 * [particle_start, particle_start + n) of scenes [scene_begin, scene_end); data is
 * [B, n, width].  Replaces _kernel_{set,get}_particles_{pos,vel,active,actu} and
 * _kernel_set_particles_{free,muscle_direction,muscle_group} (mpm_solver.py:840-1026).
 * MPM_FIELD_POS_RESET sets positions and resets v, F, C, Jp like
 * _kernel_set_particles_pos (mpm_solver.py:840-859). */
typedef enum mpm_field {
  MPM_FIELD_POS = 0,        /* float[3] */
  MPM_FIELD_VEL = 1,        /* float[3] */
  MPM_FIELD_C = 2,          /* float[9] */
  MPM_FIELD_F = 3,          /* float[9] */
  MPM_FIELD_JP = 4,         /* float[1] */
  MPM_FIELD_ACTIVE = 5,     /* float[1] read/written as 0/1 */
  MPM_FIELD_ACTU = 6,       /* float[1] */
  MPM_FIELD_FREE = 7,       /* float[1] 0/1 */
  MPM_FIELD_MUSCLE_DIR = 8, /* float[3] */
  MPM_FIELD_POS_RESET = 9   /* float[3], write only */
} mpm_field;
int mpm_set_particles(mpm_ctx* ctx, int32_t field, int64_t scene_begin, int64_t scene_end,
                      int64_t particle_start, int64_t n, const float* data, void* stream);
int mpm_get_particles(mpm_ctx* ctx, int32_t field, int64_t scene_begin, int64_t scene_end,
                      int64_t particle_start, int64_t n, float* data, void* stream);

/* Per-scene gravity [scene_end - scene_begin, 3] (host pointer).
 * Replaces Solver.set_gravity (base_solver.py:43-53). */
int mpm_set_gravity(mpm_ctx* ctx, int64_t scene_begin, int64_t scene_end,
                    const double* gravity_host);

/* Run n full substeps on every scene.  Replaces, per substep, Simulator.substep
 * (simulator.py:320-324) = MPMSolver.substep_pre_coupling (mpm_solver.py:503-515:
 * reset_grid_and_grad, compute_F_tmp, svd, p2g), LegacyCoupler.mpm_grid_op
 * (legacy_coupler.py:356-501, gravity + boundary, no coupling partners) and
 * MPMSolver.substep_post_coupling (mpm_solver.py:530-546: g2p, NaN check), plus
 * copy_frame (mpm_solver.py:556-565), which the double-buffered layout makes unnecessary.
 * The NaN check is recorded in the device status word instead of syncing every substep.
 * Captured as a CUDA graph after the first call with the same particle count. */
int mpm_substeps(mpm_ctx* ctx, int32_t n_substeps, void* stream);

/* The three phases of one substep, for callers that interleave coupling work the way
 * Simulator.substep does (simulator.py:320-324).  pre = particle sort (if needed) +
 * F update + SVD + material + P2G; grid_op = legacy_coupler.py:356-501 without partners;
 * post = G2P + boundary + NaN flag + re-keying for the next sort. */
int mpm_substep_pre(mpm_ctx* ctx, void* stream);
int mpm_substep_grid_op(mpm_ctx* ctx, void* stream);
int mpm_substep_post(mpm_ctx* ctx, void* stream);

/* The grid op in stages, in place of mpm_substep_grid_op, for a caller that applies its own
 * acceleration fields to the node velocities at their place in the field order (the reference's
 * force_fields.Custom, a user function called in legacy_coupler.py:376-378 like the built-in
 * fields).  stage 1 (after mpm_substep_pre): momentum -> velocity + gravity, then the force fields
 * [ff_begin, ff_end) of the mpm_set_force_fields list; stage 2 (repeatable): fields
 * [ff_begin, ff_end) on the velocities; stage 3: colliders, tools, SPH / PBD coupling and the
 * boundary, after which mpm_substep_post follows.  Between stages the caller may change the
 * velocities of nodes with mass > mass_eps in the buffer mpm_grid_nodes returns. */
int mpm_substep_grid_stage(mpm_ctx* ctx, int32_t stage, int32_t ff_begin, int32_t ff_end, void* stream);

/* The grid buffer of the current substep (valid from mpm_substep_pre to mpm_substep_post): *nodes
 * = device float4 per node (momentum or velocity xyz, mass), block-major, *n_nodes of them (every
 * scene's 4x4x4-node blocks, padding included).  Replaces reading MPMSolver.grid in place. */
int mpm_grid_nodes(mpm_ctx* ctx, float** nodes, int64_t* n_nodes);

/* World position pos [n_nodes][3] of every node of that buffer and its scene scene [n_nodes]
 * (-1 for block padding past the scene's grid; scene may be NULL); device arrays. */
int mpm_grid_node_positions(mpm_ctx* ctx, float* pos, int32_t* scene, void* stream);

/* Copy the dense grid of one scene into out [gx, gy, gz, 4] (x-major, float32):
 * after mpm_substep_pre it holds (momentum xyz, mass); after mpm_substep_grid_op it
 * holds (vel_out xyz, mass).  Replaces reading MPMSolver.grid (mpm_solver.py:137-148). */
int mpm_get_grid(mpm_ctx* ctx, int64_t scene, float* out, void* stream);

/* External acceleration fields of the grid op (engine/force_fields.py; applied at
 * legacy_coupler.py:381-383 as v += acc(x, v) dt for each field in order, after gravity and before
 * rigid coupling).  direction is normalised by the caller as the reference's constructors do.
 *   CONSTANT: acc = direction * strength
 *   WIND:     direction * strength inside the infinite cylinder of `radius` about the axis through
 *             center along direction, 0 outside
 *   POINT:    r = x - center, d = r / norm(r, eps); acc = strength d; acc += (acc - v) flow;
 *             acc *= 1 / (|r|_eps + 1)^falloff_pow
 *   DRAG:     -linear v - quadratic |v| v
 *   VORTEX:   about the z axis through center: falloff 1 below falloff_min, 1/(r - falloff_min + 1)^
 *             falloff_pow below falloff_max, 0 beyond; acc = falloff (strength_perpendicular
 *             (-ry, rx, 0) + strength_radial (-rx, -ry, 0)) - damping v
 *   NOISE:    (force_fields.py:232-259) acc_k = strength (2 u_k - 1), u_k uniform in [0, 1) drawn per
 *             node, component and substep: the top 24 bits of splitmix64 chained over (seed, substep
 *             counter, scene, world node index, component).  The counter counts substeps since the
 *             last mpm_set_force_fields.  Same distribution as the reference's qd.random, not the
 *             same numbers.
 *   TURBULENCE: (force_fields.py:372-421, 441-544) acc_k = strength perlin(perm[k], frequency, x),
 *             Perlin's improved noise over the 256-entry permutation perm[k] (the field's three
 *             PerlinNoiseField tables, built by the caller as the reference builds them);
 *             acc += (acc - v) flow
 * Inactive fields (active = 0) are skipped.  With any field set, the grid op runs as its own
 * kernel. */
#define MPM_FF_CONSTANT 0
#define MPM_FF_WIND 1
#define MPM_FF_POINT 2
#define MPM_FF_DRAG 3
#define MPM_FF_VORTEX 4
#define MPM_FF_NOISE 5
#define MPM_FF_TURBULENCE 6
typedef struct mpm_force_field {
  int32_t type;
  int32_t active;
  double direction[3];
  double center[3];
  double strength, radius, falloff_pow, flow;
  double linear, quadratic;
  double strength_perpendicular, strength_radial, falloff_min, falloff_max, damping;
  double frequency;      /* TURBULENCE */
  uint64_t seed;         /* NOISE */
  uint8_t perm[3][256];  /* TURBULENCE: permutation tables of the x, y, z noise fields */
} mpm_force_field;

/* Replace the force-field set (n may be 0); host array, copied before returning. */
int mpm_set_force_fields(mpm_ctx* ctx, int32_t n, const mpm_force_field* fields);

/* Kinematic rigid colliders coupled in the grid op (legacy_coupler.py:134-218, 284-347, called
 * from mpm_grid_op :389-403).  For every grid node with mass, after gravity and before the domain
 * boundary, each collider of the node's scene (in array order) with
 * influence = min(exp(-sdf / max(1e-10, softness)), 1) > 0.1 and an approaching relative velocity
 * (v - v_rigid) . n < 0 gets: tangential part reduced by friction * |normal part| (never
 * reversed), normal part scaled by -restitution, blended with the old relative velocity by the
 * influence; v_rigid = lin_vel + ang_vel x (x - com).  The reaction force -m dv / dt on the
 * collider (m = node mass / 1e3, the particle_volume_scale) and its torque about `com` are
 * accumulated on the device.  Sphere and plane SDFs are the reference's analytic ones
 * (utils/sdf.py:119-126, 372-378); the box SDF is analytic here (the reference samples a
 * precomputed SDF grid for boxes; MPM_COLLIDER_SDF does exactly that with a caller's grid).
 * With colliders set, the grid op runs as its own kernel.
 *
 * MPM_COLLIDER_SDF: a rigid geom whose SDF is a precomputed voxel grid (mpm_add_sdf_grid, with
 * gradients) - utils/sdf.py:105-185, 223-322: the point goes to the mesh frame (pos, quat), then
 * to voxel coordinates by T_mesh_to_sdf; inside the grid the value and the gradient are trilinear
 * interpolations, outside it the distance to the grid centre / cell_size + sdf_max and the
 * direction from the centre; normal = quat . gradient, normalised.
 *
 * MPM_COLLIDER_TOOL: a tool entity (engine/entities/tool_entity/mesh.py:84-177,
 * tool_entity.py:189-206), applied before the rigid colliders (legacy_coupler.py:349-354, 386-387).
 * Its voxel SDF (a grid without gradients) reads 1 outside the grid, its normal is a central
 * difference (delta 1e-2 voxels) taken back to the world frame; a node with sdf <= 0 or
 * influence > 0.1 that approaches the tool loses its inward relative velocity and tangential speed
 * by friction * |normal part|, blended by the influence (no restitution, no reaction force).  The
 * tool moves by itself: every substep its pose advances on the device from lin_vel and ang_vel
 * (pos += v dt, clamped to z >= floor_height; quat = rotvec(w dt) * quat, normalised), and the
 * collider velocity at x is (pose_next(pose^-1(x)) - x) / dt; mpm_get_collider_poses reads the
 * current poses.  Tools take no part in CPIC (the reference's CPIC sees rigid geoms only). */
#define MPM_COLLIDER_SPHERE 0 /* size[0] = radius */
#define MPM_COLLIDER_PLANE 1  /* size = plane normal in the collider frame; sdf = n . x_local */
#define MPM_COLLIDER_BOX 2    /* size = half extents */
#define MPM_COLLIDER_SDF 3    /* sdf_grid = id from mpm_add_sdf_grid (with gradients) */
#define MPM_COLLIDER_TOOL 4   /* sdf_grid = id from mpm_add_sdf_grid; lin_vel, ang_vel move it */
typedef struct mpm_collider {
  int32_t type;
  int32_t scene;        /* scene index, or -1: every scene */
  double pos[3];        /* collider position (world) */
  double quat[4];       /* orientation (w, x, y, z) */
  double size[3];
  double com[3];        /* point the angular velocity turns about (the link's root COM) */
  double lin_vel[3];
  double ang_vel[3];
  double friction;      /* coup_friction (a tool's friction) */
  double softness;      /* coup_softness */
  double restitution;   /* coup_restitution (unused by a tool) */
  int32_t sdf_grid;     /* MPM_COLLIDER_SDF / MPM_COLLIDER_TOOL: SDF grid id */
  int32_t pad;
  double floor_height;  /* MPM_COLLIDER_TOOL: ToolOptions.floor_height (FloorBoundary of the tool solver) */
} mpm_collider;

/* Replace the collider set (n may be 0); host array, copied before returning.  Resets the force
 * accumulators. */
int mpm_set_colliders(mpm_ctx* ctx, int32_t n, const mpm_collider* colliders);

/* Copy a voxel SDF grid to the device for MPM_COLLIDER_SDF / MPM_COLLIDER_TOOL colliders; *id_out
 * receives its id (0, 1, ... in call order).  values [res0][res1][res2] (x-major) in world
 * distance units, grads [res0][res1][res2][3] or NULL (a tool's grid); T_mesh_to_sdf is the 4x4
 * row-major transform from the mesh frame to voxel coordinates; cell_size and sdf_max enter the
 * outside-grid distance (utils/sdf.py:157-164).  Host arrays, copied before returning; grids live
 * until the context is destroyed (the reference's SDFInfo, rigid/sdf fields). */
int mpm_add_sdf_grid(mpm_ctx* ctx, const int32_t* res, const float* values, const float* grads,
                     const double* T_mesh_to_sdf, double cell_size, double sdf_max, int32_t* id_out);

/* Current pose of each collider: out_host [n][7] = pos (xyz), quat (wxyz); tools have advanced one
 * substep per substep since mpm_set_colliders.  Synchronises `stream`. */
int mpm_get_collider_poses(mpm_ctx* ctx, double* out_host, void* stream);

/* Force (xyz) and torque about com (xyz) exerted by the particles on each collider, summed over
 * the substeps since the last reset: out_host [n][6].  Synchronises `stream`. */
int mpm_get_collider_forces(mpm_ctx* ctx, double* out_host, int32_t reset, void* stream);

/* CPIC for thin colliders (MPMOptions.enable_CPIC; mpm_solver.py:389-411, 445-459,
 * legacy_coupler.py:62-66, 503-529): reserves n_slots collider slots of particle-side SDF normals
 * (3 floats per particle and slot, carried with the particle) and sets them to zero, as the
 * coupler's reset does; call again to reset them.  While colliders are set, P2G gives nothing
 * to a stencil node that a collider separates from the particle (its SDF normal at the node
 * points against the particle's stored one), and G2P takes there the particle's own velocity
 * collided with that collider (influence 1), the reaction going to the collider's accumulator.
 * Colliders beyond n_slots are rejected by mpm_set_colliders.  n_slots = 0 turns CPIC off.
 * Not available in pool mode. */
int mpm_enable_cpic(mpm_ctx* ctx, int32_t n_slots, void* stream);

/* MPM <-> SPH and MPM <-> PBD coupling in the grid op (legacy_coupler.py:404-498) with another
 * solver's particles.  In every grid op, after the colliders and before the domain boundary, a node
 * with MPM mass whose cell (|x_node - p|_inf < dx/2) holds particles of the set takes their mean
 * velocity, and each of those particles loses delta_mv / m_i, delta_mv = m_node (v_new - v_old)
 * (PBD: only particles with free != 0); the SPH set acts before the PBD set.
 * pos and vel [n_scenes][n][3], mass [n_scenes][n] and free [n_scenes][n] (PBD only; NULL: all
 * free) are device arrays that the caller keeps owning: they must stay valid until the set is
 * replaced or removed (n = 0).  Every grid op reads pos, mass and free and updates vel in place
 * (the caller's solver advances pos between substeps, e.g. through the split-phase entry points).
 * Not available in pool mode. */
#define MPM_COUPLED_SPH 0
#define MPM_COUPLED_PBD 1
int mpm_set_coupled_particles(mpm_ctx* ctx, int32_t kind, int64_t n, const float* pos, float* vel,
                              const float* mass, const uint8_t* free_, void* stream);

/* Soft particle-to-link constraints (mpm_solver.py:1052-1128; mpm_entity.py:631-690).
 * mpm_set_particle_constraints: for each scene b of [scene_begin, scene_end) and each particle
 * [particle_start, particle_start + n) of it with mask[b * n + i] != 0, attach the particle to
 * kinematic link `link_idx` (or to its current position if link_idx < 0): the target is the
 * current position, its offset in the link frame is kept.  link_pos [B,3] and link_quat [B,4]
 * (w, x, y, z) are the link poses at attachment, per scene.  After every G2P the target follows
 * the link's current pose (mpm_set_link_poses) and the velocity gets
 * dv = dt (-k (x - target) - 2 sqrt(k m) v) / m (m = the particle's real mass).
 * mpm_remove_particle_constraints clears the masked particles.  mask, link_pos and link_quat are
 * device arrays.  Not available in pool mode. */
int mpm_set_particle_constraints(mpm_ctx* ctx, int64_t scene_begin, int64_t scene_end, int64_t particle_start,
                                 int64_t n, const uint8_t* mask, double stiffness, int32_t link_idx,
                                 const float* link_pos, const float* link_quat, void* stream);
int mpm_remove_particle_constraints(mpm_ctx* ctx, int64_t scene_begin, int64_t scene_end, int64_t particle_start,
                                    int64_t n, const uint8_t* mask, void* stream);

/* Poses of the kinematic links that constraints follow, replacing the rigid solver's
 * links_state: poses_host [n_scenes][n_links][7] = (pos xyz, quat wxyz), host memory, copied
 * before returning.  Call whenever the links move (e.g. once per scene.step()). */
int mpm_set_link_poses(mpm_ctx* ctx, int32_t n_links, const float* poses_host);

/* Failure-detection test of the bounded device waits: runs the one-pass bucket scan with tile 0
 * withheld, so the next tile's look-back wait runs out (after 4096 polls) and sets
 * MPM_STATUS_WAIT in the status word; the kernel still completes and the context stays usable
 * (the sort is rebuilt before the next substep).  Needs a context with more than 4096 buckets. */
int mpm_test_wait_timeout(mpm_ctx* ctx, void* stream);

/* Device-side 'regular' particle sampling (utils/particle.py:180-278): the lattice of
 * np.linspace(lower + p/2, upper - p/2, max(1, round(extent / p))) per axis in row-major order,
 * kept by the reference's rejection test; positions as float32 (x, y, z) into out (device).
 * shape 0 box (size = extents), 1 sphere (size[0] = radius), 2 cylinder along z (size[0] =
 * radius, size[1] = height); pos = centre.  *n_out receives the count; with out == NULL only the
 * count is computed, and a too small capacity returns MPM_ERR_BAD_ARG after setting *n_out.
 * Synchronises `stream`. */
int mpm_sample_regular(int32_t shape, const double* pos, const double* size, double p_size, float* out,
                       int64_t capacity, int64_t* n_out, void* stream);

/* Render fields (mpm_solver.py:780-803, _kernel_update_render_fields) of scenes
 * [scene_begin, scene_end), in the reference [B, N] row order of mpm_get_state:
 *   pos_out [B,N,3]: the particle position, or the reference's "nowhere" point
 *     (-2333333, -6666666, -5201314) for an inactive particle; vel_out [B,N,3]; active_out [B,N];
 *   vvert_pos_out [B,V,3]: for each of n_vverts visual vertices, sum_j w[v,j] * x[support[v,j]]
 *     over its n_supports support particles (indices within the scene, weights from
 *     particle_entity.py:193-232), using the particles' actual positions; vvert_active_out [B,V]:
 *     the active flag of the first support.  support_idx [V, n_supports] int32 and
 *     support_w [V, n_supports] float are device arrays; an out-of-range support index is skipped
 *     and sets MPM_STATUS_BAD_INDEX.  n_vverts may be 0 (vvert pointers may then be NULL).
 * All pointers are device memory; outputs are written on `stream`. */
int mpm_render_fields(mpm_ctx* ctx, int64_t scene_begin, int64_t scene_end, float* pos_out, float* vel_out,
                      uint8_t* active_out, int64_t n_vverts, int32_t n_supports, const int32_t* support_idx,
                      const float* support_w, float* vvert_pos_out, uint8_t* vvert_active_out, void* stream);

/* Number of grid nodes with mass > mass_eps in the current grid buffer of all scenes
 * (device reduction; synchronises `stream`). */
int mpm_count_touched_nodes(mpm_ctx* ctx, int64_t* out_host, void* stream);

/* Read and optionally clear the device status word (MPM_STATUS_* bits) and the count of
 * particles whose SVD was redone in FP64.  Synchronises `stream`.
 * Replaces MPMSolver._is_state_valid (mpm_solver.py:483-489). */
int mpm_status_word(mpm_ctx* ctx, uint32_t* status_host, int64_t* fp64_svd_host,
                    int32_t clear, void* stream);

/* Tuning knobs (the autotuner sets these): P2G threads per CTA (64..256, multiple of 32) and
 * particles per thread (threads * ppt <= 1024; the P2G work chunk is their product), G2P
 * threads per CTA (64..256, multiple of 32; 0 keeps the current value), CUDA graphs on/off.
 * A new context starts at 128 P2G threads x 2 particles (64 x 1 below 65,536 particles), 128 G2P
 * threads, graphs on. */
int mpm_set_tuning(mpm_ctx* ctx, int32_t p2g_threads, int32_t particles_per_thread,
                   int32_t use_graph, int32_t g2p_threads);

/* Per-kernel timing: when enabled, mpm_substeps runs without a graph and brackets every
 * kernel with CUDA events on its launch stream; mpm_kernel_times synchronises and returns
 * accumulated milliseconds and launch counts for [P2G, grid op, G2P, scan, perm]. */
int mpm_set_profiling(mpm_ctx* ctx, int32_t enable);
int mpm_kernel_times(mpm_ctx* ctx, double* ms_host /*[5]*/, int64_t* counts_host /*[5]*/, int32_t reset);

/* ---------------------------------------------------------------- pool mode (serving)
 * A context whose scene slots are configured and retired while it runs, for a request
 * loop that keeps every live scene in one set of launches (continuous batching).  There is
 * no reference counterpart: Genesis builds one fixed scene per process (scene.py:841-905).
 * Slot s owns grid blocks [s*B, (s+1)*B) with B = ceil(max_grid_res/4)^3 and materials
 * [s*M, (s+1)*M) with M = max_materials_per_scene; particles of all slots share one pool. */
typedef struct mpm_pool_config {
  int64_t max_scenes;
  int64_t particle_capacity;
  int32_t max_grid_res;            /* largest grid nodes per axis of any admitted scene */
  int32_t max_materials_per_scene;
  int32_t with_muscle;             /* allocate actuation fields */
  int32_t reserved;
} mpm_pool_config;
int mpm_ctx_create_pool(const mpm_pool_config* cfg, int32_t device, mpm_ctx** out);

/* Configure free slot `slot` as `scene` with its materials and append its n particles
 * (device pos [n,3], per-particle material index among `materials` or NULL for 0).  The
 * scene advances for n_substeps substeps (-1: unlimited) and then stays frozen (its
 * particles are carried unchanged) until retired.  Synchronises `stream`. */
int mpm_scene_admit(mpm_ctx* ctx, int64_t slot, const mpm_scene_config* scene, const mpm_material* materials,
                    int32_t n_materials, int64_t n, const float* pos, const int32_t* mat_local,
                    int32_t n_substeps, void* stream);

/* Drop every particle of `slot` (they sort after all live particles and the next P2G does
 * not carry them) and free the slot.  Read its state first with mpm_get_state(slot, slot+1). */
int mpm_scene_retire(mpm_ctx* ctx, int64_t slot, void* stream);

/* Substeps left per slot ([max_scenes] host ints; 0 = finished/frozen, -1 = unlimited). */
int mpm_scene_steps_left(mpm_ctx* ctx, int32_t* out_host, void* stream);

/* ---------------------------------------------------------------- no-allocation substeps
 * No counterpart in the reference.  For callers that may not allocate device memory
 * (plug-ins whose host application owns every device allocation through its own pool,
 * real-time loops that forbid allocator calls after start-up, since cudaMalloc/cudaFree may
 * synchronise the device): n_substeps substeps of one scene on the caller's particle arrays, updated in place
 * (device pointers, reference layout: pos/vel [n,3], C/F [n,3,3], Jp [n]; mat [n] material
 * index or NULL for 0; active [n] or NULL for all).  No cudaMalloc/cudaFree: the grid lives
 * in a file-scope device array of at most 524288 nodes (8 MiB on every GPU that loads the
 * library); at most 16 materials, no Muscle; particles are not re-sorted (small scenes).
 * Grids beyond the limit are rejected with MPM_ERR_BAD_ARG.  All calls share the array:
 * calls that overlap on the GPU race.  The first call on a device looks up the array's
 * address with that device current; make it before any stream capture.  Only the device's
 * primary context is supported.  Synchronises `stream` at the end to read the status
 * (NaN / out-of-grid). */
int mpm_substeps_noalloc(const mpm_scene_config* scene, const mpm_material* materials, int32_t n_materials,
                         int64_t n, float* pos, float* vel, float* C, float* F, float* Jp,
                         const int32_t* mat, const uint8_t* active, int32_t n_substeps, void* stream);
/* Text of the calling thread's last failed mpm_substeps_noalloc call. */
const char* mpm_noalloc_last_error(void);

/* ---------------------------------------------------------------- differentiation
 * One differentiable substep of one scene of a single material - `neohookean` 0: corotated
 * Elastic, 1: neo-Hookean Elastic, 2: Liquid (liquid.py: the corotated stress with its mu, 0
 * unless viscous, and F_new = J^(1/3) I) - with per-particle Lame parameters mu[n], lam[n], and
 * its adjoint.
 * Replace the reference's Quadrants autodiff of the substep (p2g.grad, mpm_grid_op.grad,
 * g2p.grad, compute_F_tmp.grad: mpm_solver.py:517-554, legacy_coupler.py:998-1019) and its SVD
 * backward (mpm_solver.py:1229-1252).  Particle arrays use the reference layout; grid_pm,
 * grid_v, g_grid_v, g_grid_pm are caller buffers of res^3 float4 (res = the scene's grid);
 * status is a device uint32 (MPM_STATUS_* bits, or-ed).  mpm_diff_backward needs the grid of
 * the same substep in grid_pm/grid_v (run mpm_diff_forward on the same state first); it
 * writes dL/d(x, v, C, F) and adds into dL/d(mu, lam).  gF1 may be NULL. */
int mpm_diff_forward(const mpm_scene_config* scene, double rho, int32_t neohookean, int64_t n,
                     const float* x, const float* v, const float* C, const float* F,
                     const float* mu, const float* lam, float* x1, float* v1, float* C1, float* F1,
                     void* grid_pm, void* grid_v, uint32_t* status, void* stream);
int mpm_diff_backward(const mpm_scene_config* scene, double rho, int32_t neohookean, int64_t n,
                      const float* x, const float* v, const float* C, const float* F,
                      const float* mu, const float* lam, const float* gx1, const float* gv1,
                      const float* gC1, const float* gF1, float* gx, float* gv, float* gC, float* gF,
                      float* gmu, float* glam, void* grid_pm, void* grid_v, void* g_grid_v,
                      void* g_grid_pm, uint32_t* status, void* stream);

/* n_sub forward substeps in one call: state k in slot k % ring of x_seq [ring,n,3],
 * v_seq [ring,n,3], C_seq [ring,n,9], F_seq [ring,n,9] (slot 0 = input); with grids_per_substep
 * substep k leaves its grid at grid_pm/grid_v + k * res^3 float4, else one grid is reused. */
int mpm_diff_forward_seq(const mpm_scene_config* scene, double rho, int32_t neohookean, int64_t n, int32_t n_sub,
                         float* x_seq, float* v_seq, float* C_seq, float* F_seq, int32_t ring, const float* mu,
                         const float* lam, void* grid_pm, void* grid_v, int32_t grids_per_substep, uint32_t* status,
                         void* stream);

/* Adjoint of n_sub substeps kept by mpm_diff_forward_seq (all states and grids): g_seq holds two
 * packed gradient buffers of 24 n floats (dx, dv, dC, dF); buffer 0 carries dL/d(state n_sub) in
 * and dL/d(state 0) out; dL/d(mu, lam) accumulate into gmu, glam. */
int mpm_diff_backward_seq(const mpm_scene_config* scene, double rho, int32_t neohookean, int64_t n, int32_t n_sub,
                          const float* x_seq, const float* v_seq, const float* C_seq, const float* F_seq,
                          const float* mu, const float* lam, float* g_seq, float* gmu, float* glam, void* grid_pm,
                          void* grid_v, void* g_grid_v, void* g_grid_pm, uint32_t* status, void* stream);

/* mpm_diff_forward_seq / mpm_diff_backward_seq for scenes of several entities: per-particle
 * mass [n], material kind [n] (0 corotated Elastic, 1 neo-Hookean Elastic, 2 Liquid, 3 Sand,
 * 4 Snow) and aux [n,2] (Sand: friction alpha; Snow: 1 - yield_lower, 1 + yield_higher) instead of
 * one rho and one material; the state carries Jp (Jp_seq [ring,n]) and g_seq packs dL/dJp after
 * (dx, dv, dC, dF): [2, 25n].  Replace the same reference autodiff kernels, whose material dispatch
 * and particle mass are per particle (mpm_solver.py:341-375, particles_info.mass), and the SVD
 * backward of the plastic laws (backward_svd, mpm_solver.py:1229-1252). */
int mpm_diff_forward_seq_pp(const mpm_scene_config* scene, const float* mass, const int32_t* kind, const float* aux,
                            int64_t n, int32_t n_sub, float* x_seq, float* v_seq, float* C_seq, float* F_seq,
                            float* Jp_seq, int32_t ring, const float* mu, const float* lam, void* grid_pm, void* grid_v,
                            int32_t grids_per_substep, uint32_t* status, void* stream);
int mpm_diff_backward_seq_pp(const mpm_scene_config* scene, const float* mass, const int32_t* kind, const float* aux,
                             int64_t n, int32_t n_sub, const float* x_seq, const float* v_seq, const float* C_seq,
                             const float* F_seq, const float* Jp_seq, const float* mu, const float* lam, float* g_seq,
                             float* gmu, float* glam, void* grid_pm, void* grid_v, void* g_grid_v, void* g_grid_pm,
                             uint32_t* status, void* stream);

/* Tool entities in the differentiable form (tool_entity/mesh.py Mesh.collide in the grid op,
 * ToolEntity.advect between substeps; the reference differentiates both through its autodiff).
 * A tool: its SDF values (device, [res0][res1][res2], the layout of Mesh.sdf_voxels),
 * T_mesh_to_sdf (row-major 4x4; rows 0-2 used), Tool friction and coup_softness, the tool solver's
 * floor height.  tool_seq: device [(n_sub + 1)][n_tools][13] states (pos 3, quat wxyz 4, vel 3,
 * ang 3); the caller fills entry 0, the forward writes entries 1..n_sub.  The backward takes g_tool
 * [n_tools][12] with dL/d(pos, vel) of the last state in [0..5] and returns dL/d(pos, vel) of the
 * first state there ([6..11] is scratch).  The orientation and the angular velocity are carried
 * but not differentiated.  At most MPM_DIFF_MAX_TOOLS tools. */
#define MPM_DIFF_MAX_TOOLS 4
typedef struct mpm_diff_tool {
  const float* sdf;
  int32_t res[3];
  int32_t pad0;
  double T_mesh_to_sdf[16];
  double friction, softness, floor_height;
} mpm_diff_tool;
int mpm_diff_forward_seq_tools(const mpm_scene_config* scene, const float* mass, const int32_t* kind, const float* aux,
                               int64_t n, int32_t n_sub, float* x_seq, float* v_seq, float* C_seq, float* F_seq,
                               float* Jp_seq, int32_t ring, const float* mu, const float* lam,
                               const mpm_diff_tool* tools, int32_t n_tools, float* tool_seq, void* grid_pm,
                               void* grid_v, int32_t grids_per_substep, uint32_t* status, void* stream);
int mpm_diff_backward_seq_tools(const mpm_scene_config* scene, const float* mass, const int32_t* kind, const float* aux,
                                int64_t n, int32_t n_sub, const float* x_seq, const float* v_seq, const float* C_seq,
                                const float* F_seq, const float* Jp_seq, const float* mu, const float* lam,
                                const mpm_diff_tool* tools, int32_t n_tools, const float* tool_seq, float* g_tool,
                                float* g_seq, float* gmu, float* glam, void* grid_pm, void* grid_v, void* g_grid_v,
                                void* g_grid_pm, uint32_t* status, void* stream);

/* The general differentiable sequence: mpm_diff_forward_seq_pp / mpm_diff_backward_seq_pp plus
 * the optional parts of a scene in one record (zero-initialise it and fill what the scene has):
 * - tool entities: tools, n_tools, tool_seq and (backward) g_tool, as mpm_diff_forward_seq_tools
 *   takes them;
 * - force fields (legacy_coupler.py:381-383: v += acc(x, v) dt after gravity, before the tools;
 *   the reference differentiates them through its autodiff): host array of n_force_fields
 *   mpm_force_field records (at most MPM_DIFF_MAX_FORCE_FIELDS, inactive ones skipped, copied in
 *   the call); scene_index and ff_step (the fields' substep counter at the first substep) seed the
 *   noise draws as mpm_set_force_fields' fields draw them in env scene_index.  The backward
 *   carries dL/dv through each field's Jacobian in the node velocity (noise draws and node
 *   positions are constants);
 * - Muscle particles (kind 5: corotated, 6: neo-Hookean elastic plus the actuation stress
 *   stiffness * actu * (F m)(F m)^T of muscle.py:46-53, aux[0] = stiffness): actu [n] and
 *   muscle_dir [n][3] device arrays (both or neither; actu constant over the call), and for the
 *   backward g_actu [n], into which dL/dactu is added (mpm_entity.py _set_particles_actu_grad).
 * - kinematic rigid colliders (legacy_coupler.py:134-218, 284-347, called at :389-403 after the
 *   tools): host array of n_colliders mpm_collider records (at most MPM_DIFF_MAX_COLLIDERS; no
 *   MPM_COLLIDER_TOOL: tools go in the tool records), poses fixed over the call; SDF colliders
 *   name a grid registered with mpm_add_sdf_grid on sdf_ctx (NULL when none is of that type).
 *   The backward carries dL/dv through each collider's velocity update; poses are constants and no
 *   reaction force is accumulated.
 * - particle constraints (apply_particle_constraints, mpm_solver.py:1099-1128, after G2P):
 *   constraint_stiffness [n] (0: unconstrained) and constraint_target [n][3] device arrays, both or
 *   neither, fixed over the call (the targets the links' poses give); the backward carries dL/d(x, v)
 *   through the spring's velocity update.
 * - particle activity: active [n] device uint8 (NULL: all active); an inactive particle takes no
 *   part in P2G and G2P and keeps its state (mpm_solver.py p2g / g2p), its adjoint passes through.
 * Kinds 7 and 8 are ElastoPlastic (elasto_plastic.py:44-71) with clamped principal stretches
 * (aux = 1 - yield_lower, 1 + yield_higher) and with von Mises yield (aux[0] = yield stress / (2 mu)).
 * The backward needs the same record contents as the forward it reverses. */
#define MPM_DIFF_MAX_FORCE_FIELDS 8
#define MPM_DIFF_MAX_COLLIDERS 8
typedef struct mpm_diff_extras {
  const mpm_diff_tool* tools;
  int32_t n_tools;
  int32_t n_force_fields;
  float* tool_seq;
  float* g_tool;
  const mpm_force_field* force_fields;
  int32_t scene_index;
  int32_t pad0;
  uint64_t ff_step;
  const float* actu;
  const float* muscle_dir;
  float* g_actu;
  const mpm_collider* colliders;
  const mpm_ctx* sdf_ctx;
  int32_t n_colliders;
  int32_t pad1;
  const float* constraint_stiffness;
  const float* constraint_target;
  const uint8_t* active;
} mpm_diff_extras;
int mpm_diff_forward_seq_ex(const mpm_scene_config* scene, const float* mass, const int32_t* kind, const float* aux,
                            int64_t n, int32_t n_sub, float* x_seq, float* v_seq, float* C_seq, float* F_seq,
                            float* Jp_seq, int32_t ring, const float* mu, const float* lam, const mpm_diff_extras* ex,
                            void* grid_pm, void* grid_v, int32_t grids_per_substep, uint32_t* status, void* stream);
int mpm_diff_backward_seq_ex(const mpm_scene_config* scene, const float* mass, const int32_t* kind, const float* aux,
                             int64_t n, int32_t n_sub, const float* x_seq, const float* v_seq, const float* C_seq,
                             const float* F_seq, const float* Jp_seq, const float* mu, const float* lam,
                             const mpm_diff_extras* ex, float* g_seq, float* gmu, float* glam, void* grid_pm,
                             void* grid_v, void* g_grid_v, void* g_grid_pm, uint32_t* status, void* stream);

/* A differentiable substep in parts, for scenes with Custom force fields (a user function that acts
 * on the node velocities between grid stages, as mpm_substep_grid_stage splits the product grid op):
 * phase 0 clears grid_pm and runs P2G (writing F1, Jp1) and advances the tools (ex->tool_seq holds
 * this substep's [2][n_tools][13] states, entry 1 written); phase 1 runs grid stage `stage`:
 * 1 = velocity from grid_pm plus gravity and the fields [ff_begin, ff_end) of ex into grid_v,
 * 2 = the fields [ff_begin, ff_end) on grid_v, 3 = the tools, colliders and boundary on grid_v;
 * phase 2 runs G2P from grid_v (writing x1, v1, C1).  ex->ff_step is this substep's counter.
 * The adjoint runs the parts in reverse: phase 2 clears g_grid_v and writes the G2P adjoint (dL/dx
 * in gx, dL/d(node velocity) in g_grid_v); phase 1, stage 3 or 2, takes the velocity that stage began
 * from in vstage and turns g_grid_v into dL/d(that velocity) in place, stage 1 ends in g_grid_pm;
 * phase 0 runs the tools' chain and the P2G adjoint (adding to gx).  The caller applies each
 * Custom field's transposed Jacobian to g_grid_v between stages. */
int mpm_diff_substep_stage(const mpm_scene_config* scene, const float* mass, const int32_t* kind, const float* aux,
                           int64_t n, const float* x, const float* v, const float* C, const float* F, const float* Jp,
                           const float* mu, const float* lam, const mpm_diff_extras* ex, int32_t phase, int32_t stage,
                           int32_t ff_begin, int32_t ff_end, float* x1, float* v1, float* C1, float* F1, float* Jp1,
                           void* grid_pm, void* grid_v, uint32_t* status, void* stream);
int mpm_diff_substep_stage_adj(const mpm_scene_config* scene, const float* mass, const int32_t* kind,
                               const float* aux, int64_t n, const float* x, const float* v, const float* C,
                               const float* F, const float* Jp, const float* mu, const float* lam,
                               const mpm_diff_extras* ex, int32_t phase, int32_t stage, int32_t ff_begin,
                               int32_t ff_end, const void* vstage, const float* gx1, const float* gv1,
                               const float* gC1, const float* gF1, const float* gJp1, float* gx, float* gv, float* gC,
                               float* gF, float* gJp, float* gmu, float* glam, void* grid_pm, void* grid_v,
                               void* g_grid_v, void* g_grid_pm, uint32_t* status, void* stream);

/* ABI version of this header (1). */
int mpm_version(void);

/* Sizes: particles in use, number of grid blocks (4^3 nodes each), grid res of a scene. */
int mpm_get_info(const mpm_ctx* ctx, int64_t* n_particles, int64_t* n_blocks,
                 int64_t* n_scenes);
int mpm_scene_grid_res(const mpm_ctx* ctx, int64_t scene, int32_t* res3_host);

#ifdef __cplusplus
}
#endif
#endif /* GBMPM_H */
