// mpm_oracle.cpp - CPU restatement of the Genesis MLS-MPM substep.  TEST INFRASTRUCTURE:
// only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it, as the
// checker and as the timed CPU baseline.  It is never part of the product path.
//
// Parity status: the reference (genesis-world 0.4.5) runs on the Quadrants JIT, which is
// not installed here, so this restatement cannot be compared with the reference executing.
// Parity is pinned only through golden vectors produced by the reference's own material
// functions (tests/golden/), the reference's own closed-form constants, and physics
// known-answer tests; see the tests.  The SVD is unpinned (qd.svd is not vendored).
//
// What it follows (paths relative to the Genesis project root):
//   MPMSolver.__init__ constants      genesis/engine/solvers/mpm_solver.py:32-80
//   compute_F_tmp / svd               mpm_solver.py:293-307
//   p2g (material, stress, scatter)   mpm_solver.py:322-421
//   grid op                           genesis/engine/couplers/legacy_coupler.py:356-501
//   force fields                      genesis/engine/force_fields.py (constant, wind, point, drag, vortex)
//   rigid coupling (kinematic         legacy_coupler.py:166-218, 284-347; SDFs utils/sdf.py:119-126,
//     colliders)                      372-378 (sphere, plane); boxes use their exact distance
//   SPH / PBD grid coupling           legacy_coupler.py:404-498 (another solver's particles, by cell)
//   CPIC (thin colliders)             legacy_coupler.py:503-529 (particle-side normals),
//                                     mpm_solver.py:389-411 (P2G skips separated nodes), :445-459
//                                     (G2P takes the collided particle velocity there)
//   g2p + particle boundary           mpm_solver.py:423-481, engine/boundaries/boundaries.py:22-32
//   materials                         genesis/engine/materials/MPM/{base,elastic,liquid,sand,snow,
//                                     elasto_plastic,muscle}.py
// The accumulation order is particle order (deterministic) when threads == 1.  With
// threads > 1 the scatter uses atomic adds (like the reference's CPU backend) and is
// used only for timing.
//
// Non-free particles: the reference stores vel_in = 0 on their 27 nodes inside the
// scatter loop, racing with other particles' adds (mpm_solver.py:420-421).  This
// restatement resolves the race deterministically: such nodes end the scatter with zero
// momentum (the outcome when the store lands last), which is also what the CUDA path does.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

extern "C" {
typedef struct oracle_scene {
  double dt;
  double gravity[3];
  double lower_bound[3];
  double upper_bound[3];
  double grid_density;
  double particle_size;
  double eps;          // gs.EPS (grid-op mass threshold and Matrix.norm eps)
  double restitution;  // CubeBoundary restitution (0)
} oracle_scene;

// Kinematic rigid collider: same layout as mpm_collider of the library header.
typedef struct oracle_collider {
  int32_t type;  // 0 sphere (size[0] radius), 1 plane (size = normal, collider frame), 2 box (half extents)
  int32_t scene;
  double pos[3], quat[4], size[3], com[3], lin_vel[3], ang_vel[3];
  double friction, softness, restitution;
  int32_t sdf_grid;  // 3 (rigid geom with an SDF grid) and 4 (tool): index into the oracle's grids
  int32_t pad;
  double floor_height;  // tool: the tool solver's FloorBoundary height
} oracle_collider;

// External acceleration field: same layout as mpm_force_field of the library header.
typedef struct oracle_force_field {
  int32_t type;  // 0 constant, 1 wind, 2 point, 3 drag, 4 vortex, 5 noise, 6 turbulence
  int32_t active;
  double direction[3], center[3];
  double strength, radius, falloff_pow, flow, linear, quadratic;
  double strength_perpendicular, strength_radial, falloff_min, falloff_max, damping;
  double frequency;      // 6 turbulence
  uint64_t seed;         // 5 noise
  uint8_t perm[3][256];  // 6 turbulence: the x, y, z noise fields' permutations
} oracle_force_field;

typedef struct oracle_material {
  int32_t type;   // 0 elastic, 1 liquid, 2 sand, 3 snow, 4 elastoplastic, 5 muscle
  int32_t flags;  // 1 neohookean, 2 von Mises
  double mu, lam, rho, default_Jp, alpha, yield_lower, yield_higher, vm_yield, stiffness;
} oracle_material;
}

namespace {

template <typename T>
struct M3 {
  T a[9];
  T& operator()(int i, int j) { return a[i * 3 + j]; }
  T operator()(int i, int j) const { return a[i * 3 + j]; }
  static M3 zero() {
    M3 m;
    for (int k = 0; k < 9; ++k) m.a[k] = 0;
    return m;
  }
  static M3 eye() {
    M3 m = zero();
    m.a[0] = m.a[4] = m.a[8] = 1;
    return m;
  }
};

template <typename T>
M3<T> mul(const M3<T>& A, const M3<T>& B) {
  M3<T> C = M3<T>::zero();
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      for (int k = 0; k < 3; ++k) C(i, j) += A(i, k) * B(k, j);
  return C;
}
template <typename T>
M3<T> transpose(const M3<T>& A) {
  M3<T> C;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) C(i, j) = A(j, i);
  return C;
}
template <typename T>
M3<T> add(const M3<T>& A, const M3<T>& B, T sb = 1) {
  M3<T> C;
  for (int k = 0; k < 9; ++k) C.a[k] = A.a[k] + sb * B.a[k];
  return C;
}
template <typename T>
M3<T> scale(const M3<T>& A, T s) {
  M3<T> C;
  for (int k = 0; k < 9; ++k) C.a[k] = s * A.a[k];
  return C;
}
template <typename T>
M3<T> diag(T a, T b, T c) {
  M3<T> m = M3<T>::zero();
  m(0, 0) = a;
  m(1, 1) = b;
  m(2, 2) = c;
  return m;
}
template <typename T>
T det(const M3<T>& A) {
  return A(0, 0) * (A(1, 1) * A(2, 2) - A(1, 2) * A(2, 1)) - A(0, 1) * (A(1, 0) * A(2, 2) - A(1, 2) * A(2, 0)) +
         A(0, 2) * (A(1, 0) * A(2, 1) - A(1, 1) * A(2, 0));
}

// One-sided (Hestenes) Jacobi SVD iterated to convergence, then brought to the
// rotation-variant convention: det U = det V = +1, sig0 >= sig1 >= |sig2|, sign in sig2.
template <typename T>
void svd_hestenes(const M3<T>& A, M3<T>& U, M3<T>& S, M3<T>& V) {
  M3<T> W = A;
  V = M3<T>::eye();
  const T tol = std::numeric_limits<T>::epsilon();
  for (int sweep = 0; sweep < 60; ++sweep) {
    bool rotated = false;
    const int pq[3][2] = {{0, 1}, {0, 2}, {1, 2}};
    for (auto& e : pq) {
      const int p = e[0], q = e[1];
      T al = 0, be = 0, ga = 0;
      for (int i = 0; i < 3; ++i) {
        al += W(i, p) * W(i, p);
        be += W(i, q) * W(i, q);
        ga += W(i, p) * W(i, q);
      }
      if (std::fabs(ga) <= tol * std::sqrt(al * be) || ga == 0) continue;
      rotated = true;
      const T zeta = (be - al) / (2 * ga);
      const T t = (zeta >= 0 ? 1 : -1) / (std::fabs(zeta) + std::sqrt(1 + zeta * zeta));
      const T c = 1 / std::sqrt(1 + t * t), s = c * t;
      for (int i = 0; i < 3; ++i) {
        const T wp = W(i, p), wq = W(i, q);
        W(i, p) = c * wp - s * wq;
        W(i, q) = s * wp + c * wq;
        const T vp = V(i, p), vq = V(i, q);
        V(i, p) = c * vp - s * vq;
        V(i, q) = s * vp + c * vq;
      }
    }
    if (!rotated) break;
  }
  T sig[3];
  for (int k = 0; k < 3; ++k) sig[k] = std::sqrt(W(0, k) * W(0, k) + W(1, k) * W(1, k) + W(2, k) * W(2, k));
  // sort descending (same column swaps on W and V)
  for (int a = 0; a < 2; ++a)
    for (int b = a + 1; b < 3; ++b)
      if (sig[b] > sig[a]) {
        std::swap(sig[a], sig[b]);
        for (int i = 0; i < 3; ++i) {
          std::swap(W(i, a), W(i, b));
          std::swap(V(i, a), V(i, b));
        }
      }
  // U = W diag(1/sig), completing null directions orthonormally
  U = M3<T>::zero();
  const T small = sig[0] * std::numeric_limits<T>::epsilon() * 8;
  int rank = 0;
  for (int k = 0; k < 3; ++k)
    if (sig[k] > small && sig[k] > 0) {
      for (int i = 0; i < 3; ++i) U(i, k) = W(i, k) / sig[k];
      rank = k + 1;
    }
  for (int k = rank; k < 3; ++k) {
    // pick the basis vector least aligned with existing columns, Gram-Schmidt it
    T best[3] = {0, 0, 0};
    T bestn = -1;
    for (int e = 0; e < 3; ++e) {
      T v[3] = {0, 0, 0};
      v[e] = 1;
      for (int j = 0; j < k; ++j) {
        const T d = U(0, j) * v[0] + U(1, j) * v[1] + U(2, j) * v[2];
        for (int i = 0; i < 3; ++i) v[i] -= d * U(i, j);
      }
      const T n = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
      if (n > bestn) {
        bestn = n;
        for (int i = 0; i < 3; ++i) best[i] = v[i] / n;
      }
    }
    for (int i = 0; i < 3; ++i) U(i, k) = best[i];
  }
  if (det(V) < 0)
    for (int i = 0; i < 3; ++i) {
      V(i, 2) = -V(i, 2);
      U(i, 2) = -U(i, 2);
    }
  if (det(U) < 0) {
    for (int i = 0; i < 3; ++i) U(i, 2) = -U(i, 2);
    sig[2] = -sig[2];
  }
  S = diag(sig[0], sig[1], sig[2]);
}

// Matrix.norm(eps) = sqrt(|x|^2 + eps) (upstream Taichi definition; unverified here)
template <typename T>
T norm_eps(const T* v, T eps) {
  return std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2] + eps);
}

template <typename T>
struct Mat {
  int type, flags;
  T mu, lam, rho, default_Jp, alpha, yl, yh, vmy, stiffness;
};

// base.py:94-99 / elastic.py:48-53
template <typename T>
M3<T> stress_default(const Mat<T>& m, const M3<T>& U, const M3<T>& V, const M3<T>& F_new, T J) {
  M3<T> r = mul(U, transpose(V));
  M3<T> s = scale(mul(add(F_new, r, T(-1)), transpose(F_new)), 2 * m.mu);
  return add(s, scale(M3<T>::eye(), m.lam * J * (J - 1)));
}

// Material update: returns F_new, S_new, Jp_new (update_F_S_Jp of each material).
template <typename T>
void update_F_S_Jp(const Mat<T>& m, T J, const M3<T>& F_tmp, const M3<T>& U, const M3<T>& S, const M3<T>& V, T Jp,
                   T eps, M3<T>& F_new, M3<T>& S_new, T& Jp_new) {
  switch (m.type) {
    case 1:  // liquid.py:36-40
      F_new = scale(M3<T>::eye(), std::pow(J, T(1) / T(3)));
      S_new = S;
      Jp_new = Jp;
      return;
    case 2: {  // sand.py:47-78
      M3<T> So = M3<T>::zero();
      T e[3];
      for (int i = 0; i < 3; ++i) {
        e[i] = std::log(std::max(std::fabs(S(i, i)), T(1e-4)));
        So(i, i) = 1;
      }
      const T tr = e[0] + e[1] + e[2] + Jp;
      T eh[3];
      for (int i = 0; i < 3; ++i) eh[i] = e[i] - tr / 3;
      const T ehn = norm_eps(eh, eps);
      if (tr >= 0) {
        Jp_new = tr;
      } else {
        Jp_new = 0;
        const T dg = ehn + (3 * m.lam + 2 * m.mu) / (2 * m.mu) * tr * m.alpha;
        for (int i = 0; i < 3; ++i) So(i, i) = std::exp(e[i] - std::max(T(0), dg) / ehn * eh[i]);
      }
      S_new = So;
      F_new = mul(mul(U, S_new), transpose(V));
      return;
    }
    case 3: {  // snow.py:56-64
      S_new = M3<T>::zero();
      Jp_new = Jp;
      for (int d = 0; d < 3; ++d) {
        S_new(d, d) = std::min(std::max(S(d, d), 1 - m.yl), 1 + m.yh);
        Jp_new *= S(d, d) / S_new(d, d);
      }
      F_new = mul(mul(U, S_new), transpose(V));
      return;
    }
    case 4: {  // elasto_plastic.py:44-71
      if (m.flags & 2) {
        T s[3], e[3];
        for (int d = 0; d < 3; ++d) {
          s[d] = std::max(S(d, d), T(0.05));
          e[d] = std::log(s[d]);
        }
        const T mean = (e[0] + e[1] + e[2]) / 3;
        T eh[3];
        for (int d = 0; d < 3; ++d) eh[d] = e[d] - mean;
        const T ehn = norm_eps(eh, eps);
        const T dg = ehn - m.vmy / (2 * m.mu);
        if (dg > 0) {
          for (int d = 0; d < 3; ++d) e[d] -= (dg / ehn) * eh[d];
          S_new = diag(std::exp(e[0]), std::exp(e[1]), std::exp(e[2]));
          F_new = mul(mul(U, S_new), transpose(V));
        } else {
          S_new = diag(s[0], s[1], s[2]);
          F_new = F_tmp;
        }
      } else {
        S_new = M3<T>::zero();
        for (int d = 0; d < 3; ++d) S_new(d, d) = std::min(std::max(S(d, d), 1 - m.yl), 1 + m.yh);
        F_new = mul(mul(U, S_new), transpose(V));
      }
      Jp_new = Jp;
      return;
    }
    default:  // elastic.py:41-46 (elastic and muscle)
      F_new = F_tmp;
      S_new = S;
      Jp_new = Jp;
      return;
  }
}

template <typename T>
M3<T> update_stress(const Mat<T>& m, const M3<T>& U, const M3<T>& S, const M3<T>& V, const M3<T>& F_tmp,
                    const M3<T>& F_new, T J, T Jp, T actu, const T* mdir) {
  switch (m.type) {
    case 1:  // liquid.py:43-49 (uses F_tmp)
      return stress_default(m, U, V, F_tmp, J);
    case 2: {  // sand.py:74-84 (S = S_new)
      T lsum = 0;
      M3<T> center = M3<T>::zero();
      for (int i = 0; i < 3; ++i) {
        lsum += std::log(S(i, i));
        center(i, i) = 2 * m.mu * std::log(S(i, i)) * (1 / S(i, i));
      }
      for (int i = 0; i < 3; ++i) center(i, i) += m.lam * lsum * (1 / S(i, i));
      return mul(mul(mul(U, center), transpose(V)), transpose(F_new));
    }
    case 3: {  // snow.py:66-74 (Jp before the update)
      const T h = std::exp(10 * (1 - Jp));
      Mat<T> mh = m;
      mh.mu = m.mu * h;
      mh.lam = m.lam * h;
      return stress_default(mh, U, V, F_new, J);
    }
    case 4:  // base.py default stress
      return stress_default(m, U, V, F_new, J);
    default: {  // elastic.py:48-60, muscle.py:46-53
      M3<T> st;
      if (m.flags & 1)
        st = add(scale(mul(F_tmp, transpose(F_tmp)), m.mu), scale(M3<T>::eye(), m.lam * std::log(J) - m.mu));
      else
        st = stress_default(m, U, V, F_new, J);
      if (m.type == 5) {
        M3<T> AAt;
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j) AAt(i, j) = mdir[i] * mdir[j];
        st = add(st, scale(mul(mul(F_tmp, AAt), transpose(F_tmp)), m.stiffness * actu));
      }
      return st;
    }
  }
}

// Colliders applied in the grid op of every run (set by oracle_set_colliders) and the reaction
// force / torque they accumulated.
std::vector<oracle_collider> g_colliders;
std::vector<double> g_collider_acc;

std::vector<oracle_force_field> g_ffs;

// Substeps since the force fields were set: the noise field's draw counter.
uint64_t g_ff_step = 0;

// splitmix64 (Steele, Lea and Flood 2014) as a mixing function: the noise field's draws.
inline uint64_t splitmix64(uint64_t z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

// Perlin's improved noise over a 256-entry permutation (force_fields.py:441-544; the reference's
// 512-entry table is the permutation twice).
template <typename T>
T perlin(const uint8_t* p, T f, T x, T y, T z) {
  auto fade = [](T t) { return t * t * t * (t * (t * 6 - 15) + 10); };
  auto lerp = [](T t, T a, T b) { return a + t * (b - a); };
  auto grad = [](int h, T gx, T gy, T gz) {
    h &= 15;
    const T u = h < 8 ? gx : gy;
    const T w = h < 4 ? gy : ((h == 12 || h == 14) ? gx : gz);
    return ((h & 1) == 0 ? u : -u) + ((h & 2) == 0 ? w : -w);
  };
  x *= f;
  y *= f;
  z *= f;
  const T fx = std::floor(x), fy = std::floor(y), fz = std::floor(z);
  const int X = (int)fx & 255, Y = (int)fy & 255, Z = (int)fz & 255;
  x -= fx;
  y -= fy;
  z -= fz;
  const T u = fade(x), v = fade(y), w = fade(z);
  auto P = [&](int i) { return (int)p[i & 255]; };
  const int A = P(X) + Y, AA = P(A) + Z, AB = P(A + 1) + Z, B = P(X + 1) + Y, BA = P(B) + Z, BB = P(B + 1) + Z;
  return lerp(w,
              lerp(v, lerp(u, grad(P(AA), x, y, z), grad(P(BA), x - 1, y, z)),
                   lerp(u, grad(P(AB), x, y - 1, z), grad(P(BB), x - 1, y - 1, z))),
              lerp(v, lerp(u, grad(P(AA + 1), x, y, z - 1), grad(P(BA + 1), x - 1, y, z - 1)),
                   lerp(u, grad(P(AB + 1), x, y - 1, z - 1), grad(P(BB + 1), x - 1, y - 1, z - 1))));
}

// engine/force_fields.py _get_acc: Constant :73, Wind :122, Point :178, Drag :220, Noise :243,
// Vortex :319, Turbulence :400; gw is the node's world index (noise draws).
template <typename T>
void ff_acc(const oracle_force_field& f, const T* x, const T* v, T eps, T* a, const int64_t* gw) {
  a[0] = a[1] = a[2] = 0;
  const T dir[3] = {(T)f.direction[0], (T)f.direction[1], (T)f.direction[2]};
  const T r[3] = {x[0] - (T)f.center[0], x[1] - (T)f.center[1], x[2] - (T)f.center[2]};
  if (f.type == 0) {
    for (int k = 0; k < 3; ++k) a[k] = dir[k] * (T)f.strength;
  } else if (f.type == 1) {
    const T c[3] = {r[1] * dir[2] - r[2] * dir[1], r[2] * dir[0] - r[0] * dir[2], r[0] * dir[1] - r[1] * dir[0]};
    if (!(std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]) > (T)f.radius))
      for (int k = 0; k < 3; ++k) a[k] = dir[k] * (T)f.strength;
  } else if (f.type == 2) {
    const T rad = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2] + eps);
    const T fall = 1 / std::pow(rad + 1, (T)f.falloff_pow);
    for (int k = 0; k < 3; ++k) {
      T ak = (T)f.strength * (r[k] / rad);
      ak += (ak - v[k]) * (T)f.flow;
      a[k] = ak * fall;
    }
  } else if (f.type == 3) {
    const T vn = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    for (int k = 0; k < 3; ++k) a[k] = -(T)f.linear * v[k] - (T)f.quadratic * vn * v[k];
  } else if (f.type == 4) {
    const T rad = std::sqrt(r[0] * r[0] + r[1] * r[1]);
    T fall = 0;
    if (rad < (T)f.falloff_min) fall = 1;
    else if (rad < (T)f.falloff_max) fall = 1 / std::pow(rad - (T)f.falloff_min + 1, (T)f.falloff_pow);
    const T sp = (T)f.strength_perpendicular, sr = (T)f.strength_radial, dm = (T)f.damping;
    a[0] = fall * (sp * -r[1] + sr * -r[0]) - dm * v[0];
    a[1] = fall * (sp * r[0] + sr * -r[1]) - dm * v[1];
    a[2] = -dm * v[2];
  } else if (f.type == 5) {  // uniform in [-strength, strength) per node, component and substep
    const uint64_t node = ((uint64_t)((uint32_t)gw[0] & 0x1fffffu)) | ((uint64_t)((uint32_t)gw[1] & 0x1fffffu) << 21) |
                          ((uint64_t)((uint32_t)gw[2] & 0x1fffffu) << 42);
    const uint64_t h = splitmix64(splitmix64(splitmix64(splitmix64(f.seed) ^ g_ff_step) ^ 0ull) ^ node);
    for (int k = 0; k < 3; ++k) {
      const T u = (T)(splitmix64(h + (uint64_t)k) >> 40) * (T)(1.0 / 16777216.0);
      a[k] = (u * 2 - 1) * (T)f.strength;
    }
  } else if (f.type == 6) {
    for (int k = 0; k < 3; ++k) a[k] = perlin<T>(f.perm[k], (T)f.frequency, x[0], x[1], x[2]) * (T)f.strength;
    for (int k = 0; k < 3; ++k) a[k] += (a[k] - v[k]) * (T)f.flow;
  }
}

// gu.transform_by_quat with q = (w, x, y, z) (utils/geom.py:256-271).
template <typename T>
void quat_rot(const double* q, const T* v, T* o) {
  const T w = (T)q[0], x = (T)q[1], y = (T)q[2], z = (T)q[3];
  o[0] = v[0] * (x * x + w * w - y * y - z * z) + v[1] * (2 * x * y - 2 * w * z) + v[2] * (2 * x * z + 2 * w * y);
  o[1] = v[0] * (2 * w * z + 2 * x * y) + v[1] * (w * w - x * x + y * y - z * z) + v[2] * (-2 * w * x + 2 * y * z);
  o[2] = v[0] * (-2 * w * y + 2 * x * z) + v[1] * (2 * w * x + 2 * y * z) + v[2] * (w * w - x * x - y * y + z * z);
}

// Voxel SDF grids (oracle_add_sdf_grid): values [x][y][z], gradients [x][y][z][3] (rigid) or none
// (tool), T_mesh_to_sdf (4x4 row-major), cell size and maximum (utils/sdf.py SDFInfo).
struct SdfGridH {
  int64_t res[3];
  std::vector<double> val, grad;
  double T[16];
  double cell_size, sdf_max;
};
std::vector<SdfGridH> g_sdf_grids;

// qd_inv_transform_by_trans_quat then qd_transform_by_T: world -> mesh frame -> voxel frame.
template <typename T>
void to_voxels(const oracle_collider& c, const double* cpos, const double* cquat, const T* x, T* pm, T* pv) {
  const SdfGridH& g = g_sdf_grids[(size_t)c.sdf_grid];
  const T d[3] = {x[0] - (T)cpos[0], x[1] - (T)cpos[1], x[2] - (T)cpos[2]};
  const double qi[4] = {cquat[0], -cquat[1], -cquat[2], -cquat[3]};
  quat_rot(qi, d, pm);
  for (int r = 0; r < 3; ++r)
    pv[r] = (T)g.T[r * 4] * pm[0] + (T)g.T[r * 4 + 1] * pm[1] + (T)g.T[r * 4 + 2] * pm[2] + (T)g.T[r * 4 + 3];
}

// Sum over the 8 corner voxels (qd.ndrange(2, 2, 2) order) of prod(1 - |p - corner|) * value.
template <typename T>
T trilinear(const SdfGridH& g, const std::vector<double>& f, int comps, int comp, const T* p, const int64_t* base) {
  T acc = 0;
  for (int a = 0; a < 2; ++a)
    for (int b = 0; b < 2; ++b)
      for (int e = 0; e < 2; ++e) {
        const int64_t q[3] = {base[0] + a, base[1] + b, base[2] + e};
        T w = 1;
        for (int k = 0; k < 3; ++k) w *= 1 - std::fabs(p[k] - (T)q[k]);
        acc = acc + w * (T)f[(size_t)(((q[0] * g.res[1] + q[1]) * g.res[2] + q[2]) * comps + comp)];
      }
  return acc;
}

// Rigid geom SDF grid (utils/sdf.py:137-184, 223-296): signed distance; gradient in `gv`.
template <typename T>
T rigid_grid_sdf(const oracle_collider& c, const T* pv, T eps, T* gv) {
  const SdfGridH& g = g_sdf_grids[(size_t)c.sdf_grid];
  bool outside = false;
  for (int k = 0; k < 3; ++k) outside = outside || pv[k] >= (T)(g.res[k] - 1) || pv[k] <= 0;
  if (outside) {
    T d[3], l2 = 0;
    for (int k = 0; k < 3; ++k) {
      d[k] = pv[k] - (T)(g.res[k] - 1) / 2;
      l2 += d[k] * d[k];
    }
    for (int k = 0; k < 3; ++k) gv[k] = d[k] / std::sqrt(l2 + eps);
    return std::sqrt(l2) / (T)g.cell_size + (T)g.sdf_max;
  }
  int64_t base[3];
  for (int k = 0; k < 3; ++k) base[k] = std::min((int64_t)std::floor(pv[k]), g.res[k] - 2);
  for (int k = 0; k < 3; ++k) gv[k] = trilinear(g, g.grad, 3, k, pv, base);
  return trilinear(g, g.val, 1, 0, pv, base);
}

// Mesh.sdf_ of a tool (tool_entity/mesh.py:92-107): 1 when the base voxel leaves the grid.
template <typename T>
T tool_grid_sdf(const SdfGridH& g, const T* pv) {
  int64_t base[3];
  for (int k = 0; k < 3; ++k) {
    base[k] = (int64_t)std::floor(pv[k]);
    if (base[k] >= g.res[k] - 1 || base[k] < 0) return 1;
  }
  return trilinear(g, g.val, 1, 0, pv, base);
}

// ToolEntity.advect (tool_entity.py:193-206): pose one substep later, in double.
void tool_advance(const oracle_collider& c, double dt, double eps, double* pn, double* qn) {
  for (int k = 0; k < 3; ++k) pn[k] = c.pos[k] + c.lin_vel[k] * dt;
  pn[2] = std::max(pn[2], c.floor_height);  // FloorBoundary.impose_pos
  const double rv[3] = {c.ang_vel[0] * dt, c.ang_vel[1] * dt, c.ang_vel[2] * dt};
  const double th2 = rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2];
  double u[4] = {1, 0, 0, 0};
  if (th2 > eps * eps) {  // qd_rotvec_to_quat
    const double th = std::sqrt(th2);
    u[0] = std::cos(th / 2);
    for (int k = 0; k < 3; ++k) u[k + 1] = std::sin(th / 2) / th * rv[k];
    const double n2 = u[0] * u[0] + u[1] * u[1] + u[2] * u[2] + u[3] * u[3];
    for (int k = 0; k < 4; ++k) u[k] *= 0.5 * (3 - n2);
  }
  const double* v = c.quat;  // qd_transform_quat_by_quat(quat, u) = normalize(u * quat)
  const double q[4] = {u[0] * v[0] - u[1] * v[1] - u[2] * v[2] - u[3] * v[3],
                       u[0] * v[1] + u[1] * v[0] + u[2] * v[3] - u[3] * v[2],
                       u[0] * v[2] - u[1] * v[3] + u[2] * v[0] + u[3] * v[1],
                       u[0] * v[3] + u[1] * v[2] - u[2] * v[1] + u[3] * v[0]};
  const double len = std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  for (int k = 0; k < 4; ++k) qn[k] = q[k] / len;
}

// Mesh.collide (tool_entity/mesh.py:148-177) at node position x.
template <typename T>
void collide_tool(const oracle_collider& c, const T* x, T* v, T dt, T eps) {
  const SdfGridH& g = g_sdf_grids[(size_t)c.sdf_grid];
  T pm[3], pv[3];
  to_voxels(c, c.pos, c.quat, x, pm, pv);
  const T sd = tool_grid_sdf(g, pv);
  const T infl = std::min(std::exp(-sd / std::max(eps, (T)c.softness)), (T)1);
  if (!(sd <= 0 || infl > (T)0.1)) return;
  double pn[3], qn[4];
  tool_advance(c, (double)dt, (double)eps, pn, qn);
  T xn[3], vc[3];
  quat_rot(qn, pm, xn);
  for (int k = 0; k < 3; ++k) vc[k] = (xn[k] + (T)pn[k] - x[k]) / dt;
  T nv[3];
  for (int i = 0; i < 3; ++i) {  // Mesh.normal_: central differences, delta 1e-2 voxels
    T inc[3] = {pv[0], pv[1], pv[2]}, dec[3] = {pv[0], pv[1], pv[2]};
    inc[i] += (T)1e-2;
    dec[i] -= (T)1e-2;
    nv[i] = (tool_grid_sdf(g, inc) - tool_grid_sdf(g, dec)) / (2 * (T)1e-2);
  }
  T l = std::sqrt(nv[0] * nv[0] + nv[1] * nv[1] + nv[2] * nv[2] + eps);
  for (int k = 0; k < 3; ++k) nv[k] /= l;
  // R_voxels_to_mesh = inverse(T[:3, :3]) (Cramer's rule)
  const double* M = g.T;
  const double det = M[0] * (M[5] * M[10] - M[6] * M[9]) - M[1] * (M[4] * M[10] - M[6] * M[8]) +
                     M[2] * (M[4] * M[9] - M[5] * M[8]);
  const double R[9] = {(M[5] * M[10] - M[6] * M[9]) / det, (M[2] * M[9] - M[1] * M[10]) / det,
                       (M[1] * M[6] - M[2] * M[5]) / det,  (M[6] * M[8] - M[4] * M[10]) / det,
                       (M[0] * M[10] - M[2] * M[8]) / det, (M[2] * M[4] - M[0] * M[6]) / det,
                       (M[4] * M[9] - M[5] * M[8]) / det,  (M[1] * M[8] - M[0] * M[9]) / det,
                       (M[0] * M[5] - M[1] * M[4]) / det};
  T nm[3], n[3];
  for (int r = 0; r < 3; ++r) nm[r] = (T)R[r * 3] * nv[0] + (T)R[r * 3 + 1] * nv[1] + (T)R[r * 3 + 2] * nv[2];
  quat_rot(c.quat, nm, n);
  l = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2] + eps);
  for (int k = 0; k < 3; ++k) n[k] /= l;
  T rv[3];
  for (int k = 0; k < 3; ++k) rv[k] = v[k] - vc[k];
  const T nc = rv[0] * n[0] + rv[1] * n[1] + rv[2] * n[2];
  if (!(nc < 0)) return;
  T rt[3];
  for (int k = 0; k < 3; ++k) rt[k] = rv[k] - nc * n[k];
  const T rtn = std::sqrt(rt[0] * rt[0] + rt[1] * rt[1] + rt[2] * rt[2] + eps);
  const T keep = std::max((T)0, rtn + nc * (T)c.friction);
  for (int k = 0; k < 3; ++k) v[k] = vc[k] + rt[k] / rtn * keep * infl + rv[k] * (1 - infl);
}

// Signed distance and unit normal: sphere and plane as utils/sdf.py:119-126, 372-378; a box by
// its exact distance function (outside: the clamped offset; inside: the nearest face).
template <typename T>
T collider_sdf(const oracle_collider& c, const T* x, T eps, T* n) {
  if (c.type == 3) {  // SDF grid: utils/sdf.py sdf_func_world / sdf_func_normal_world
    T pm[3], pv[3], gv[3], gw[3];
    to_voxels(c, c.pos, c.quat, x, pm, pv);
    const T sd = rigid_grid_sdf(c, pv, eps, gv);
    quat_rot(c.quat, gv, gw);
    const T gn = std::sqrt(gw[0] * gw[0] + gw[1] * gw[1] + gw[2] * gw[2] + eps);
    for (int k = 0; k < 3; ++k) n[k] = gw[k] / gn;
    return sd;
  }
  T d[3] = {x[0] - (T)c.pos[0], x[1] - (T)c.pos[1], x[2] - (T)c.pos[2]};
  if (c.type == 0) {
    const T ln = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2] + eps);
    for (int k = 0; k < 3; ++k) n[k] = d[k] / ln;
    return std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]) - (T)c.size[0];
  }
  const double qi[4] = {c.quat[0], -c.quat[1], -c.quat[2], -c.quat[3]};
  T l[3], gl[3], g[3], sd;
  quat_rot(qi, d, l);
  if (c.type == 1) {
    sd = l[0] * (T)c.size[0] + l[1] * (T)c.size[1] + l[2] * (T)c.size[2];
    for (int k = 0; k < 3; ++k) gl[k] = (T)c.size[k];
  } else {
    T q[3], out2 = 0;
    int ax = 0;
    for (int k = 0; k < 3; ++k) {
      q[k] = std::fabs(l[k]) - (T)c.size[k];
      const T o = std::max(q[k], (T)0);
      out2 += o * o;
      if (q[k] > q[ax]) ax = k;
    }
    sd = std::sqrt(out2) + std::min(std::max(q[0], std::max(q[1], q[2])), (T)0);
    for (int k = 0; k < 3; ++k) {
      const T sg = l[k] < 0 ? (T)-1 : (T)1;
      gl[k] = out2 > 0 ? sg * std::max(q[k], (T)0) : (k == ax ? sg : (T)0);
    }
  }
  quat_rot(c.quat, gl, g);
  const T gn = std::sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2] + eps);
  for (int k = 0; k < 3; ++k) n[k] = g[k] / gn;
  return sd;
}

// _func_collide_in_rigid_geom (legacy_coupler.py:284-347): relative-velocity projection with
// friction and restitution along the normal n, blended by `influence`; the reaction on collider
// ci goes to its accumulator.
template <typename T>
void collide_in(size_t ci, const T* x, T* v, T mass, const T* n, T influence, T dt, T eps) {
  const oracle_collider& c = g_colliders[ci];
  const T r[3] = {x[0] - (T)c.com[0], x[1] - (T)c.com[1], x[2] - (T)c.com[2]};
  const T w[3] = {(T)c.ang_vel[0], (T)c.ang_vel[1], (T)c.ang_vel[2]};
  const T vr[3] = {w[1] * r[2] - w[2] * r[1] + (T)c.lin_vel[0], w[2] * r[0] - w[0] * r[2] + (T)c.lin_vel[1],
                   w[0] * r[1] - w[1] * r[0] + (T)c.lin_vel[2]};
  T rv[3];
  for (int k = 0; k < 3; ++k) rv[k] = v[k] - vr[k];
  const T rvn = rv[0] * n[0] + rv[1] * n[1] + rv[2] * n[2];
  if (!(rvn < 0)) return;
  T rt[3];
  for (int k = 0; k < 3; ++k) rt[k] = rv[k] - rvn * n[k];
  const T rtn = std::sqrt(rt[0] * rt[0] + rt[1] * rt[1] + rt[2] * rt[2] + eps);
  const T mag = std::max((T)0, rtn + rvn * (T)c.friction);
  T f[3];
  for (int k = 0; k < 3; ++k) {
    const T rnew = rt[k] / rtn * mag - n[k] * rvn * (T)c.restitution;
    const T nv = vr[k] + rnew * influence + rv[k] * (1 - influence);
    f[k] = -mass * (nv - v[k]) / dt;
    v[k] = nv;
  }
  double* acc = g_collider_acc.data() + ci * 6;
  const double tq[3] = {(double)(r[1] * f[2] - r[2] * f[1]), (double)(r[2] * f[0] - r[0] * f[2]),
                        (double)(r[0] * f[1] - r[1] * f[0])};
  for (int k = 0; k < 3; ++k) {
#pragma omp atomic
    acc[k] += (double)f[k];
#pragma omp atomic
    acc[3 + k] += tq[k];
  }
}

// _func_collide_with_rigid (legacy_coupler.py:134-218): every collider of the scene whose SDF
// influence exceeds 0.1 at x, in order.
template <typename T>
void collide_node(int scene, const T* x, T* v, T mass, T dt, T eps) {
  for (const oracle_collider& c : g_colliders)  // tools first (legacy_coupler.py:386-387)
    if (c.type == 4 && (c.scene < 0 || c.scene == scene)) collide_tool<T>(c, x, v, dt, eps);
  for (size_t ci = 0; ci < g_colliders.size(); ++ci) {
    const oracle_collider& c = g_colliders[ci];
    if (c.type == 4 || (c.scene >= 0 && c.scene != scene)) continue;
    T n[3];
    const T sd = collider_sdf(c, x, eps, n);
    const T influence = std::min(std::exp(-sd / std::max((T)1e-10, (T)c.softness)), (T)1);
    if (!(influence > (T)0.1)) continue;
    collide_in<T>(ci, x, v, mass, n, influence, dt, eps);
  }
}

// Another solver's particles coupled in the grid op, [0] SPH and [1] PBD (set by
// oracle_set_coupled); velocities are updated in place across runs.
struct ExtSet {
  std::vector<double> pos, vel, mass;
  std::vector<uint8_t> free_;
  int64_t n = 0;
};
ExtSet g_ext[2];

// legacy_coupler.py:404-498: the node at x (MPM mass m) takes the mean velocity of the set's
// particles with |x - p|_inf < dx/2; each of them loses m (v_new - v_old) / m_i (PBD: free only).
template <typename T>
void couple_ext(const T* x, T* v, T m, T dx) {
  for (int k = 0; k < 2; ++k) {
    ExtSet& E = g_ext[k];
    if (E.n == 0) continue;
    auto inside = [&](int64_t i) {
      for (int d = 0; d < 3; ++d)
        if (!(std::fabs(x[d] - (T)E.pos[i * 3 + d]) < (T)0.5 * dx)) return false;
      return true;
    };
    T sv[3] = {0, 0, 0};
    int64_t cnt = 0;
    for (int64_t i = 0; i < E.n; ++i)
      if (inside(i)) {
        for (int d = 0; d < 3; ++d) sv[d] += (T)E.vel[i * 3 + d];
        ++cnt;
      }
    if (cnt == 0) continue;
    T dmv[3];
    for (int d = 0; d < 3; ++d) {
      const T vn = sv[d] / (T)cnt;
      dmv[d] = m * (vn - v[d]);
      v[d] = vn;
    }
    for (int64_t i = 0; i < E.n; ++i)
      if (inside(i) && (k == 0 || E.free_.empty() || E.free_[i]))
        for (int d = 0; d < 3; ++d) E.vel[i * 3 + d] -= (double)(dmv[d] / (T)E.mass[i]);
  }
}

// CPIC state: per particle and collider, the last SDF normal seen on the particle's side
// (mpm_rigid_normal, legacy_coupler.py:65), zero until the first substep.
bool g_cpic = false;
std::vector<double> g_cpic_normal;

// First collider of the scene (in order) whose normal at world point xc points against the
// particle's stored normal (mpm_solver.py:392-409), or -1.
template <typename T>
int cpic_separating(int scene, const double* pn, const T* xc, T eps) {
  const size_t nc = g_colliders.size();
  for (size_t ci = 0; ci < nc; ++ci) {
    const oracle_collider& c = g_colliders[ci];
    if (c.type == 4 || (c.scene >= 0 && c.scene != scene)) continue;
    T n[3];
    collider_sdf(c, xc, eps, n);
    if ((T)pn[ci * 3] * n[0] + (T)pn[ci * 3 + 1] * n[1] + (T)pn[ci * 3 + 2] * n[2] < 0) return (int)ci;
  }
  return -1;
}

template <typename T>
struct Scene {
  T dt, dx, inv_dx, p_vol, eps, restitution;
  T g[3], lo[3], hi[3];
  int64_t res[3], off[3];
};

template <typename T>
Scene<T> make_scene(const oracle_scene& c) {
  Scene<T> S;
  const double dx = 1.0 / c.grid_density;
  S.dt = (T)c.dt;
  S.dx = (T)dx;
  S.inv_dx = (T)c.grid_density;
  S.p_vol = (T)(c.particle_size * c.particle_size * c.particle_size * 1e3);
  S.eps = (T)c.eps;
  S.restitution = (T)c.restitution;
  for (int d = 0; d < 3; ++d) {
    S.g[d] = (T)c.gravity[d];
    S.lo[d] = (T)(c.lower_bound[d] + 3 * dx);
    S.hi[d] = (T)(c.upper_bound[d] - 3 * dx);
    const int64_t lo = (int64_t)std::nearbyint(c.grid_density * c.lower_bound[d]);
    const int64_t hi = (int64_t)std::nearbyint(c.grid_density * c.upper_bound[d]);
    S.res[d] = hi - lo + 1;
    S.off[d] = lo;
  }
  return S;
}

template <typename T>
inline void atomic_add(T& dst, T v, bool atomic) {
  if (atomic) {
#pragma omp atomic
    dst += v;
  } else {
    dst += v;
  }
}

template <typename T>
int run(const oracle_scene* sc, const oracle_material* mats, int n_mats, int64_t n, T* pos, T* vel, T* C, T* F,
        T* Jp, const int32_t* mat, const uint8_t* active, const uint8_t* free_, const T* actu, const T* mdir,
        int n_substeps, T* grid_out, int64_t* n_touched, int threads) {
  const Scene<T> S = make_scene<T>(*sc);
  std::vector<Mat<T>> M(n_mats);
  for (int i = 0; i < n_mats; ++i) {
    const oracle_material& m = mats[i];
    M[i] = {m.type, m.flags, (T)m.mu, (T)m.lam, (T)m.rho, (T)m.default_Jp, (T)m.alpha, (T)m.yield_lower,
            (T)m.yield_higher, (T)m.vm_yield, (T)m.stiffness};
  }
  const int64_t rx = S.res[0], ry = S.res[1], rz = S.res[2];
  const int64_t nn = rx * ry * rz;
  std::vector<T> gm(nn), gp(nn * 3), gv(nn * 3);
  std::vector<uint8_t> pin;
  bool any_pinned = false;
  for (int64_t i = 0; i < n && free_; ++i) any_pinned = any_pinned || (active[i] && !free_[i]);
  if (any_pinned) pin.assign(nn, 0);
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#endif
  const bool par = threads > 1;
  const T stress_scale = (T)(-(double)S.dt * (double)S.p_vol * 4.0 * (double)S.inv_dx * (double)S.inv_dx);
  const size_t ncol = g_colliders.size();
  const bool cpic = g_cpic && ncol > 0;
  std::vector<int16_t> cflag;  // cpic_flag: separating collider of each particle's 27 nodes, or -1
  if (cpic) {
    if (g_cpic_normal.size() != (size_t)n * ncol * 3) g_cpic_normal.assign((size_t)n * ncol * 3, 0.0);
    cflag.assign((size_t)n * 27, -1);
  }
  for (int step = 0; step < n_substeps; ++step) {
    if (cpic) {  // mpm_surface_to_particle (legacy_coupler.py:513-529): keep the particle's side
#pragma omp parallel for schedule(static) if (par)
      for (int64_t i = 0; i < n; ++i) {
        if (!active[i]) continue;
        for (size_t ci = 0; ci < ncol; ++ci) {
          const oracle_collider& c = g_colliders[ci];
          if (c.type == 4 || (c.scene >= 0 && c.scene != 0)) continue;
          T nr[3];
          collider_sdf(c, pos + i * 3, S.eps, nr);
          double* pn = g_cpic_normal.data() + ((size_t)i * ncol + ci) * 3;
          if ((T)pn[0] * nr[0] + (T)pn[1] * nr[1] + (T)pn[2] * nr[2] >= 0)
            for (int k = 0; k < 3; ++k) pn[k] = (double)nr[k];
        }
      }
    }
    // reset_grid_and_grad (mpm_solver.py:577-587)
    std::fill(gm.begin(), gm.end(), T(0));
    std::fill(gp.begin(), gp.end(), T(0));
    std::fill(gv.begin(), gv.end(), T(0));
    int bad = 0;
    // p2g
#pragma omp parallel for schedule(static) if (par) reduction(| : bad)
    for (int64_t i = 0; i < n; ++i) {
      if (!active[i]) continue;
      const Mat<T>& m = M[mat[i]];
      const T mass = S.p_vol * m.rho;
      M3<T> Cm, Fm;
      std::memcpy(Cm.a, C + i * 9, sizeof(T) * 9);
      std::memcpy(Fm.a, F + i * 9, sizeof(T) * 9);
      const M3<T> F_tmp = mul(add(M3<T>::eye(), Cm, S.dt), Fm);
      M3<T> U, Sg, V;
      svd_hestenes(F_tmp, U, Sg, V);
      const T J = det(Sg);
      M3<T> F_new, S_new;
      T Jp_new;
      update_F_S_Jp(m, J, F_tmp, U, Sg, V, Jp[i], S.eps, F_new, S_new, Jp_new);
      const T md[3] = {mdir ? mdir[i * 3] : T(0), mdir ? mdir[i * 3 + 1] : T(0), mdir ? mdir[i * 3 + 2] : T(1)};
      M3<T> stress = update_stress(m, U, S_new, V, F_tmp, F_new, J, Jp[i], actu ? actu[i] : T(0), md);
      std::memcpy(F + i * 9, F_new.a, sizeof(T) * 9);
      Jp[i] = Jp_new;
      stress = scale(stress, stress_scale);
      const M3<T> affine = add(stress, Cm, mass);
      int64_t base[3];
      T fx[3], w[3][3];
      for (int d = 0; d < 3; ++d) {
        const T xs = pos[i * 3 + d] * S.inv_dx;
        base[d] = (int64_t)std::floor(xs - T(0.5));
        fx[d] = xs - (T)base[d];
        w[0][d] = T(0.5) * (T(1.5) - fx[d]) * (T(1.5) - fx[d]);
        w[1][d] = T(0.75) - (fx[d] - 1) * (fx[d] - 1);
        w[2][d] = T(0.5) * (fx[d] - T(0.5)) * (fx[d] - T(0.5));
        const int64_t lo = base[d] - S.off[d];
        if (lo < 0 || lo + 2 >= S.res[d]) bad = 1;
      }
      if (bad) continue;
      const bool is_free = !free_ || free_[i];
      for (int ox = 0; ox < 3; ++ox)
        for (int oy = 0; oy < 3; ++oy)
          for (int oz = 0; oz < 3; ++oz) {
            const int o[3] = {ox, oy, oz};
            T dpos[3];
            T weight = 1;
            for (int d = 0; d < 3; ++d) {
              dpos[d] = ((T)o[d] - fx[d]) * S.dx;
              weight *= w[o[d]][d];
            }
            const int64_t I = ((base[0] - S.off[0] + ox) * ry + (base[1] - S.off[1] + oy)) * rz + (base[2] - S.off[2] + oz);
            if (!is_free) pin[I] = 1;
            if (cpic) {  // a node behind a thin collider gets nothing from this particle (:389-412)
              const T xc[3] = {(T)(base[0] + ox) * S.dx, (T)(base[1] + oy) * S.dx, (T)(base[2] + oz) * S.dx};
              const int sep = cpic_separating<T>(0, g_cpic_normal.data() + (size_t)i * ncol * 3, xc, S.eps);
              cflag[(size_t)i * 27 + ox * 9 + oy * 3 + oz] = (int16_t)sep;
              if (sep >= 0) continue;
            }
            for (int r = 0; r < 3; ++r) {
              const T a = affine(r, 0) * dpos[0] + affine(r, 1) * dpos[1] + affine(r, 2) * dpos[2];
              atomic_add(gp[I * 3 + r], weight * (mass * vel[i * 3 + r] + a), par);
            }
            atomic_add(gm[I], weight * mass, par);
          }
    }
    if (bad) return 5;
    if (any_pinned)
      for (int64_t I = 0; I < nn; ++I)
        if (pin[I]) {
          gp[I * 3] = gp[I * 3 + 1] = gp[I * 3 + 2] = 0;
          pin[I] = 0;
        }
    if (grid_out && step == n_substeps - 1)
      for (int64_t I = 0; I < nn; ++I) {
        grid_out[I * 4 + 0] = gp[I * 3 + 0];
        grid_out[I * 4 + 1] = gp[I * 3 + 1];
        grid_out[I * 4 + 2] = gp[I * 3 + 2];
        grid_out[I * 4 + 3] = gm[I];
      }
    // grid op (legacy_coupler.py:367-373, 501)
    int64_t touched = 0;
#pragma omp parallel for schedule(static) if (par) reduction(+ : touched)
    for (int64_t I = 0; I < nn; ++I) {
      if (!(gm[I] > S.eps)) continue;
      ++touched;
      const int64_t idx[3] = {I / (ry * rz), (I / rz) % ry, I % rz};
      T v[3];
      for (int d = 0; d < 3; ++d) v[d] = (1 / gm[I]) * gp[I * 3 + d] + S.dt * S.g[d];
      if (!g_colliders.empty() || !g_ffs.empty() || g_ext[0].n > 0 || g_ext[1].n > 0) {
        T x[3];
        for (int d = 0; d < 3; ++d) x[d] = (T)(idx[d] + S.off[d]) * S.dx;
        for (const oracle_force_field& f : g_ffs) {  // force fields (legacy_coupler.py:381-383)
          if (!f.active) continue;
          T a[3];
          const int64_t gw[3] = {idx[0] + S.off[0], idx[1] + S.off[1], idx[2] + S.off[2]};
          ff_acc<T>(f, x, v, S.eps, a, gw);
          for (int d = 0; d < 3; ++d) v[d] += a[d] * S.dt;
        }
        collide_node<T>(0, x, v, gm[I] / (T)1e3, S.dt, S.eps);  // rigid coupling (:389-403)
        couple_ext<T>(x, v, gm[I] / (T)1e3, S.dx);               // SPH, then PBD (:404-498)
      }
      for (int d = 0; d < 3; ++d) {
        const T p = (T)(idx[d] + S.off[d]) * S.dx;
        if (p >= S.hi[d] && v[d] >= 0) v[d] *= -S.restitution;
        else if (p <= S.lo[d] && v[d] <= 0) v[d] *= -S.restitution;
        gv[I * 3 + d] = v[d];
      }
    }
    if (n_touched && step == n_substeps - 1) *n_touched = touched;
    // g2p (mpm_solver.py:431-481)
    int nan = 0;
#pragma omp parallel for schedule(static) if (par) reduction(| : nan)
    for (int64_t i = 0; i < n; ++i) {
      if (!active[i]) continue;
      int64_t base[3];
      T fx[3], w[3][3];
      for (int d = 0; d < 3; ++d) {
        const T xs = pos[i * 3 + d] * S.inv_dx;
        base[d] = (int64_t)std::floor(xs - T(0.5));
        fx[d] = xs - (T)base[d];
        w[0][d] = T(0.5) * (T(1.5) - fx[d]) * (T(1.5) - fx[d]);
        w[1][d] = T(0.75) - (fx[d] - 1) * (fx[d] - 1);
        w[2][d] = T(0.5) * (fx[d] - T(0.5)) * (fx[d] - T(0.5));
      }
      T nv[3] = {0, 0, 0};
      M3<T> nC = M3<T>::zero();
      for (int ox = 0; ox < 3; ++ox)
        for (int oy = 0; oy < 3; ++oy)
          for (int oz = 0; oz < 3; ++oz) {
            const int o[3] = {ox, oy, oz};
            T dpos[3];
            T weight = 1;
            for (int d = 0; d < 3; ++d) {
              dpos[d] = (T)o[d] - fx[d];
              weight *= w[o[d]][d];
            }
            const int64_t I = ((base[0] - S.off[0] + ox) * ry + (base[1] - S.off[1] + oy)) * rz + (base[2] - S.off[2] + oz);
            T gvel[3] = {gv[I * 3], gv[I * 3 + 1], gv[I * 3 + 2]};
            const int sep = cpic ? cflag[(size_t)i * 27 + ox * 9 + oy * 3 + oz] : -1;
            if (sep >= 0) {  // the particle's own velocity, collided with that collider (:445-459)
              for (int r = 0; r < 3; ++r) gvel[r] = vel[i * 3 + r];
              T pn[3];
              for (int k = 0; k < 3; ++k) pn[k] = (T)g_cpic_normal[((size_t)i * ncol + sep) * 3 + k];
              collide_in<T>((size_t)sep, pos + i * 3, gvel, M[mat[i]].rho * S.p_vol * weight / (T)1e3, pn, (T)1,
                            S.dt, S.eps);
            }
            for (int r = 0; r < 3; ++r) {
              const T g = gvel[r];
              nv[r] += weight * g;
              for (int c = 0; c < 3; ++c) nC(r, c) += 4 * S.inv_dx * weight * g * dpos[c];
            }
          }
      T np[3];
      for (int d = 0; d < 3; ++d) np[d] = pos[i * 3 + d] + S.dt * nv[d];
      for (int d = 0; d < 3; ++d) {
        if (np[d] >= S.hi[d] && nv[d] >= 0) nv[d] *= -S.restitution;
        else if (np[d] <= S.lo[d] && nv[d] <= 0) nv[d] *= -S.restitution;
        if (std::isnan(np[d])) nan = 1;
        np[d] = std::max(std::min(np[d], S.hi[d]), S.lo[d]);
      }
      for (int d = 0; d < 3; ++d) {
        pos[i * 3 + d] = np[d];
        vel[i * 3 + d] = nv[d];
      }
      std::memcpy(C + i * 9, nC.a, sizeof(T) * 9);
    }
    if (nan) return 4;
    ++g_ff_step;  // the noise field draws anew every substep
    for (oracle_collider& c : g_colliders)  // tools move (ToolEntity.advect)
      if (c.type == 4) {
        double pn[3], qn[4];
        tool_advance(c, (double)S.dt, (double)S.eps, pn, qn);
        std::memcpy(c.pos, pn, sizeof(pn));
        std::memcpy(c.quat, qn, sizeof(qn));
      }
  }
  return 0;
}

}  // namespace

extern "C" {

int oracle_substeps_f64(const oracle_scene* sc, const oracle_material* mats, int n_mats, int64_t n, double* pos,
                        double* vel, double* C, double* F, double* Jp, const int32_t* mat, const uint8_t* active,
                        const uint8_t* free_, const double* actu, const double* mdir, int n_substeps,
                        double* grid_out, int64_t* n_touched, int threads) {
  return run<double>(sc, mats, n_mats, n, pos, vel, C, F, Jp, mat, active, free_, actu, mdir, n_substeps, grid_out,
                     n_touched, threads);
}

int oracle_substeps_f32(const oracle_scene* sc, const oracle_material* mats, int n_mats, int64_t n, float* pos,
                        float* vel, float* C, float* F, float* Jp, const int32_t* mat, const uint8_t* active,
                        const uint8_t* free_, const float* actu, const float* mdir, int n_substeps, float* grid_out,
                        int64_t* n_touched, int threads) {
  return run<float>(sc, mats, n_mats, n, pos, vel, C, F, Jp, mat, active, free_, actu, mdir, n_substeps, grid_out,
                    n_touched, threads);
}

void oracle_svd_f64(const double* A, double* U, double* sig, double* V) {
  M3<double> a, u, s, v;
  std::memcpy(a.a, A, sizeof(a.a));
  svd_hestenes(a, u, s, v);
  std::memcpy(U, u.a, sizeof(u.a));
  std::memcpy(V, v.a, sizeof(v.a));
  for (int k = 0; k < 3; ++k) sig[k] = s(k, k);
}

// Material update + stress of one particle (for golden-vector checks of the material code).
void oracle_material_f64(const oracle_material* mm, const double* F_tmp, double Jp, double actu, const double* mdir,
                         double eps, double* F_new, double* Jp_new, double* stress) {
  Mat<double> m = {mm->type, mm->flags, mm->mu, mm->lam, mm->rho, mm->default_Jp, mm->alpha,
                   mm->yield_lower, mm->yield_higher, mm->vm_yield, mm->stiffness};
  M3<double> Ft, U, S, V, Fn, Sn;
  std::memcpy(Ft.a, F_tmp, sizeof(Ft.a));
  svd_hestenes(Ft, U, S, V);
  const double J = det(S);
  double jn;
  update_F_S_Jp(m, J, Ft, U, S, V, Jp, eps, Fn, Sn, jn);
  M3<double> st = update_stress(m, U, Sn, V, Ft, Fn, J, Jp, actu, mdir);
  std::memcpy(F_new, Fn.a, sizeof(Fn.a));
  *Jp_new = jn;
  std::memcpy(stress, st.a, sizeof(st.a));
}

// Colliders for the following runs (n = 0 removes them); resets the force accumulators.
void oracle_set_colliders(int n, const oracle_collider* c) {
  g_colliders.assign(c, c + n);
  g_collider_acc.assign((size_t)n * 6, 0.0);
}

// CPIC for the following runs (MPMOptions.enable_CPIC); clears the particle-side normals.
void oracle_set_cpic(int enable) {
  g_cpic = enable != 0;
  g_cpic_normal.clear();
}

// Coupled particle set `kind` (0 SPH, 1 PBD) for the following runs: pos/vel [n][3], mass [n],
// free [n] or NULL (PBD); n = 0 removes it.
void oracle_set_coupled(int kind, int64_t n, const double* pos, const double* vel, const double* mass,
                        const uint8_t* free_) {
  ExtSet& E = g_ext[kind & 1];
  E.n = n;
  E.pos.assign(pos, pos + (n > 0 ? n * 3 : 0));
  E.vel.assign(vel, vel + (n > 0 ? n * 3 : 0));
  E.mass.assign(mass, mass + (n > 0 ? n : 0));
  if (free_ && n > 0) E.free_.assign(free_, free_ + n);
  else E.free_.clear();
}

// Current velocities of coupled set `kind`: out [n][3].
void oracle_coupled_vel(int kind, double* out) {
  const ExtSet& E = g_ext[kind & 1];
  for (size_t i = 0; i < E.vel.size(); ++i) out[i] = E.vel[i];
}

// Force fields for the following runs (n = 0 removes them).
void oracle_set_force_fields(int n, const oracle_force_field* f) {
  g_ffs.assign(f, f + n);
  g_ff_step = 0;
}

// Voxel SDF grid for collider types 3 and 4; returns its index (0, 1, ... in call order).
int oracle_add_sdf_grid(const int32_t* res, const float* values, const float* grads, const double* T_mesh_to_sdf,
                        double cell_size, double sdf_max) {
  SdfGridH g;
  for (int k = 0; k < 3; ++k) g.res[k] = res[k];
  const size_t nv = (size_t)res[0] * res[1] * res[2];
  g.val.assign(values, values + nv);
  if (grads) g.grad.assign(grads, grads + 3 * nv);
  std::memcpy(g.T, T_mesh_to_sdf, sizeof(g.T));
  g.cell_size = cell_size;
  g.sdf_max = sdf_max;
  g_sdf_grids.push_back(std::move(g));
  return (int)g_sdf_grids.size() - 1;
}

// Drops every SDF grid (ids restart at 0).
void oracle_clear_sdf_grids() { g_sdf_grids.clear(); }

// Current collider poses (tools advance every substep): out [n][7] = pos, quat.
void oracle_collider_poses(double* out) {
  for (size_t i = 0; i < g_colliders.size(); ++i) {
    std::memcpy(out + i * 7, g_colliders[i].pos, sizeof(double) * 3);
    std::memcpy(out + i * 7 + 3, g_colliders[i].quat, sizeof(double) * 4);
  }
}

// Reaction force and torque accumulated on each collider: out [n][6].
void oracle_collider_forces(double* out) {
  for (size_t i = 0; i < g_collider_acc.size(); ++i) out[i] = g_collider_acc[i];
}

int oracle_grid_res(const oracle_scene* sc, int64_t* res3) {
  const Scene<double> S = make_scene<double>(*sc);
  for (int d = 0; d < 3; ++d) res3[d] = S.res[d];
  return 0;
}

}  // extern "C"
