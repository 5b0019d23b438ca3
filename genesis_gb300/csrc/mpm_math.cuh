// mpm_math.cuh - per-particle MLS-MPM math shared by the CUDA kernels (and compiled on the
// host by the unit tests): 3x3 SVD, the six material models, quadratic B-spline weights.
//
// Everything here is a function of one particle and lives in registers.  Matrices are
// row-major float[9].  The templates run in float (the product path) and in double (the
// SVD fallback for particles whose FP32 factorisation fails its residual check).
#pragma once

#include <math.h>
#include <stdint.h>

#ifdef __CUDACC__
#define GB_HD __host__ __device__ __forceinline__
#else
#define GB_HD inline
#endif

namespace gbmpm {

GB_HD float gsqrt(float x) { return sqrtf(x); }
GB_HD double gsqrt(double x) { return sqrt(x); }
GB_HD float gabs(float x) { return fabsf(x); }
GB_HD double gabs(double x) { return fabs(x); }
GB_HD float glog(float x) { return logf(x); }
GB_HD double glog(double x) { return log(x); }
GB_HD float gexp(float x) { return expf(x); }
GB_HD double gexp(double x) { return exp(x); }
GB_HD float gpow(float x, float y) { return powf(x, y); }
GB_HD double gpow(double x, double y) { return pow(x, y); }
template <typename T> GB_HD T gmin(T a, T b) { return a < b ? a : b; }

// Rotation helpers: the angle of a Jacobi rotation only has to shrink the off-diagonal, so
// float uses the fast reciprocal-based division; what must stay accurate is c^2 + s^2 = 1,
// so the float cosine is rsqrt refined by one Newton step.  double keeps exact operations.
GB_HD float gdiv_fast(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fdividef(a, b);
#else
  return a / b;
#endif
}
GB_HD double gdiv_fast(double a, double b) { return a / b; }
GB_HD float grsqrt_acc(float x) {
#ifdef __CUDA_ARCH__
  const float r = rsqrtf(x);
  return r * (1.5f - 0.5f * x * r * r);
#else
  return 1.f / sqrtf(x);
#endif
}
GB_HD double grsqrt_acc(double x) { return 1.0 / sqrt(x); }
// sqrt of a positive argument for a rotation angle (only the convergence rate depends on it)
GB_HD float gsqrt_fast(float x) {
#ifdef __CUDA_ARCH__
  return x * rsqrtf(x);
#else
  return sqrtf(x);
#endif
}
GB_HD double gsqrt_fast(double x) { return sqrt(x); }
template <typename T> GB_HD T gmax(T a, T b) { return a > b ? a : b; }

// ------------------------------------------------------------------------------------
// 3x3 SVD, rotation-variant convention: A = U diag(sig) V^T with det U = det V = +1,
// |sig0| >= |sig1| >= |sig2| (approximately), sig0, sig1 >= 0 and sig2 carrying the sign of
// det A.  This is the convention of the Sifakis/McAdams SVD that Taichi-derived `svd`
// returns for 3x3 (mpm_solver.py:305 calls qd.svd).
//
// Method (McAdams, Selle, Tamstorf, Teran, Sifakis 2011, "Computing the singular value
// decomposition of 3x3 matrices with minimal branching and elementary floating point
// operations", structure of sections 2-4): symmetric eigen-analysis of A^T A by cyclic
// Jacobi sweeps (here with exact Jacobi rotations, Golub & Van Loan Alg. 8.5.1, instead of
// the paper's approximate quaternion rotations), V from the accumulated rotations, column
// sort of B = A V by norm, then Givens QR of B giving U and the singular values.
// ------------------------------------------------------------------------------------

template <typename T> struct Eps;
template <> struct Eps<float> { static constexpr float v = 1.1920929e-7f; };
template <> struct Eps<double> { static constexpr double v = 2.220446049250313e-16; };

// One Jacobi rotation zeroing the symmetric entry (p,q); r is the third index.  An entry
// already below the rounding level of its diagonal pair is left alone (the classical
// Jacobi threshold): rotating it would swap exact degeneracies (F = I) for rounding noise
// in U and V, which the corotated stress 2 mu (F - U V^T) F^T amplifies by mu.
template <typename T>
GB_HD bool jacobi_rotate(T& app, T& aqq, T& apq, T& arp, T& arq, T* V, int p, int q) {
  if (!(apq * apq > Eps<T>::v * Eps<T>::v * gabs(app * aqq))) return false;  // |apq| > eps sqrt|app aqq|
  const T theta = gdiv_fast(aqq - app, T(2) * apq);
  const T at = gabs(theta);
  T t = (at < T(1e18)) ? gdiv_fast(T(1), at + gsqrt_fast(theta * theta + T(1))) : gdiv_fast(T(0.5), at);
  if (theta < T(0)) t = -t;
  const T c = grsqrt_acc(t * t + T(1));
  const T s = t * c;
  app -= t * apq;
  aqq += t * apq;
  apq = T(0);
  const T rp = c * arp - s * arq;
  const T rq = s * arp + c * arq;
  arp = rp;
  arq = rq;
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    const T vp = V[r * 3 + p], vq = V[r * 3 + q];
    V[r * 3 + p] = c * vp - s * vq;
    V[r * 3 + q] = s * vp + c * vq;
  }
  return true;
}

// Swap columns i and j of B and V and negate the new column j (keeps det V = +1).
template <typename T>
GB_HD void swap_neg_cols(T* B, T* V, T* nrm, int i, int j) {
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    T b = B[r * 3 + i];
    B[r * 3 + i] = B[r * 3 + j];
    B[r * 3 + j] = -b;
    T v = V[r * 3 + i];
    V[r * 3 + i] = V[r * 3 + j];
    V[r * 3 + j] = -v;
  }
  T n = nrm[i];
  nrm[i] = nrm[j];
  nrm[j] = n;
}

// Givens rotation on rows j, i of B (i > j) zeroing B[i][j]; accumulates Q <- Q G^T.
template <typename T>
GB_HD void givens_qr_step(T* B, T* Q, int j, int i) {
  const T a = B[j * 3 + j], b = B[i * 3 + j];
  const T r2 = a * a + b * b;
  T c = T(1), s = T(0);
  if (r2 > T(0)) {
    const T inv = grsqrt_acc(r2);  // c^2 + s^2 = 1 to rounding
    c = a * inv;
    s = b * inv;
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const T bj = B[j * 3 + k], bi = B[i * 3 + k];
    B[j * 3 + k] = c * bj + s * bi;
    B[i * 3 + k] = -s * bj + c * bi;
    const T qj = Q[k * 3 + j], qi = Q[k * 3 + i];
    Q[k * 3 + j] = c * qj + s * qi;
    Q[k * 3 + i] = -s * qj + c * qi;
  }
}

// Returns the off-diagonal residual of the final triangular factor relative to |sig0|
// (a convergence measure: 0 for an exact factorisation).
template <typename T, int SWEEPS>
GB_HD T svd3(const T* A, T* U, T* sig, T* V) {
  // S = A^T A (symmetric)
  T s00 = 0, s11 = 0, s22 = 0, s01 = 0, s02 = 0, s12 = 0;
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    const T a0 = A[r * 3 + 0], a1 = A[r * 3 + 1], a2 = A[r * 3 + 2];
    s00 += a0 * a0;
    s11 += a1 * a1;
    s22 += a2 * a2;
    s01 += a0 * a1;
    s02 += a0 * a2;
    s12 += a1 * a2;
  }
#pragma unroll
  for (int k = 0; k < 9; ++k) V[k] = (k % 4 == 0) ? T(1) : T(0);
#pragma unroll
  for (int sweep = 0; sweep < SWEEPS; ++sweep) {
    // a sweep that rotates nothing leaves S unchanged, so every later sweep would skip too
    bool any = jacobi_rotate(s00, s11, s01, s02, s12, V, 0, 1);
    any = jacobi_rotate(s00, s22, s02, s01, s12, V, 0, 2) || any;
    any = jacobi_rotate(s11, s22, s12, s01, s02, V, 1, 2) || any;
    if (!any) break;
  }
  // B = A V
  T B[9];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c)
      B[r * 3 + c] = A[r * 3 + 0] * V[0 * 3 + c] + A[r * 3 + 1] * V[1 * 3 + c] + A[r * 3 + 2] * V[2 * 3 + c];
  T nrm[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) nrm[c] = B[c] * B[c] + B[3 + c] * B[3 + c] + B[6 + c] * B[6 + c];
  if (nrm[0] < nrm[1]) swap_neg_cols(B, V, nrm, 0, 1);
  if (nrm[0] < nrm[2]) swap_neg_cols(B, V, nrm, 0, 2);
  if (nrm[1] < nrm[2]) swap_neg_cols(B, V, nrm, 1, 2);
#pragma unroll
  for (int k = 0; k < 9; ++k) U[k] = (k % 4 == 0) ? T(1) : T(0);
  givens_qr_step(B, U, 0, 1);
  givens_qr_step(B, U, 0, 2);
  givens_qr_step(B, U, 1, 2);
  sig[0] = B[0];
  sig[1] = B[4];
  sig[2] = B[8];
  const T off = gabs(B[1]) + gabs(B[2]) + gabs(B[5]);
  const T scale = gabs(sig[0]);
  return scale > T(0) ? off / scale : off;
}

// Whether a factorisation from svd3 is accurate enough to use: its residual (relative to |sig0|)
// is below tol, and so is the rotation error it implies for the polar factor U V^T, which is
// about the off-diagonal residual over the smallest pair sum |sig1| + |sig2| (a deformation
// compressed to nearly nothing in two directions has an ill-determined FP32 rotation even when
// the residual is small).  NaN fails.
template <typename T>
GB_HD bool svd_accurate(T res, const T* sig, T tol) {
  return res <= tol && res * gabs(sig[0]) <= tol * (gabs(sig[1]) + gabs(sig[2]));
}

// ------------------------------------------------------------------------------------
// Small matrix helpers (row-major 3x3)
// ------------------------------------------------------------------------------------
template <typename T>
GB_HD void mat_mul(const T* A, const T* B, T* C) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      C[i * 3 + j] = A[i * 3 + 0] * B[0 * 3 + j] + A[i * 3 + 1] * B[1 * 3 + j] + A[i * 3 + 2] * B[2 * 3 + j];
}
// C = A B^T
template <typename T>
GB_HD void mat_mul_bt(const T* A, const T* B, T* C) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      C[i * 3 + j] = A[i * 3 + 0] * B[j * 3 + 0] + A[i * 3 + 1] * B[j * 3 + 1] + A[i * 3 + 2] * B[j * 3 + 2];
}
// C = U diag(d) V^T
template <typename T>
GB_HD void usvt(const T* U, const T* d, const T* V, T* C) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      C[i * 3 + j] = U[i * 3 + 0] * d[0] * V[j * 3 + 0] + U[i * 3 + 1] * d[1] * V[j * 3 + 1] +
                     U[i * 3 + 2] * d[2] * V[j * 3 + 2];
}

// ------------------------------------------------------------------------------------
// Materials (genesis/engine/materials/MPM/*.py).  Constants are precomputed on the host
// the way the reference folds its Python-level arithmetic before compiling the kernel.
// ------------------------------------------------------------------------------------
enum : int32_t {
  MT_ELASTIC = 0,
  MT_LIQUID = 1,
  MT_SAND = 2,
  MT_SNOW = 3,
  MT_ELASTOPLASTIC = 4,
  MT_MUSCLE = 5,
};
enum : int32_t { MF_NEOHOOKEAN = 1, MF_VON_MISES = 2 };

struct MaterialDev {
  int32_t type, flags, scene, pad0;
  float mu, lam, mass, default_Jp;
  float alpha, sand_coef, clamp_lo, clamp_hi;  // sand_coef = (3 lam + 2 mu) / (2 mu)
  float vm_ratio, stiffness, pad1, pad2;       // vm_ratio = yield_stress / (2 mu)
};

// Corotated stress 2 mu (Fe - U V^T) Fe^T + lam J (J - 1) I  (base.py:94-99, elastic.py:48-53)
template <typename T>
GB_HD void stress_corotated(T mu, T lam, const T* Fe, const T* U, const T* V, T J, T* P) {
  T R[9], D[9];
  mat_mul_bt(U, V, R);
#pragma unroll
  for (int k = 0; k < 9; ++k) D[k] = Fe[k] - R[k];
  mat_mul_bt(D, Fe, P);
  const T p = lam * J * (J - T(1));
#pragma unroll
  for (int k = 0; k < 9; ++k) P[k] = T(2) * mu * P[k];
  P[0] += p;
  P[4] += p;
  P[8] += p;
}

// Neo-Hookean stress mu F F^T + (lam log J - mu) I  (elastic.py:55-60)
template <typename T>
GB_HD void stress_neohookean(T mu, T lam, const T* Ft, T J, T* P) {
  mat_mul_bt(Ft, Ft, P);
#pragma unroll
  for (int k = 0; k < 9; ++k) P[k] *= mu;
  const T p = lam * glog(J) - mu;
  P[0] += p;
  P[4] += p;
  P[8] += p;
}

// Material update + stress of one particle: mpm_solver.py:339-375 dispatch, stress before
// the -dt*vol*4*inv_dx^2 scale.  eps is gs.EPS (used by Matrix.norm(eps) = sqrt(|x|^2+eps)).
template <typename T>
GB_HD void material_update(const MaterialDev& M, const T* Ft, const T* U, const T* sig, const T* V,
                           T Jp, T actu, const T* mdir, T eps, T* F_new, T& Jp_new, T* P) {
  const T J = sig[0] * sig[1] * sig[2];
  const T mu = T(M.mu), lam = T(M.lam);
  Jp_new = Jp;
  switch (M.type) {
    case MT_LIQUID: {  // liquid.py:36-49
      const T j3 = gpow(J, T(1) / T(3));
#pragma unroll
      for (int k = 0; k < 9; ++k) F_new[k] = (k % 4 == 0) ? j3 : T(0);
      stress_corotated(mu, lam, Ft, U, V, J, P);
      break;
    }
    case MT_SAND: {  // sand.py:47-84
      T e[3], S[3];
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        e[i] = glog(gmax(gabs(sig[i]), T(1e-4)));
        S[i] = T(1);
      }
      const T tr = e[0] + e[1] + e[2] + Jp;
      T eh[3];
#pragma unroll
      for (int i = 0; i < 3; ++i) eh[i] = e[i] - tr / T(3);
      const T ehn = gsqrt(eh[0] * eh[0] + eh[1] * eh[1] + eh[2] * eh[2] + eps);
      if (tr >= T(0)) {
        Jp_new = tr;
      } else {
        Jp_new = T(0);
        const T dg = ehn + T(M.sand_coef) * tr * T(M.alpha);
#pragma unroll
        for (int i = 0; i < 3; ++i) S[i] = gexp(e[i] - gmax(T(0), dg) / ehn * eh[i]);
      }
      usvt(U, S, V, F_new);
      T lsum = glog(S[0]) + glog(S[1]) + glog(S[2]);
      T c[3];
#pragma unroll
      for (int i = 0; i < 3; ++i) c[i] = T(2) * mu * glog(S[i]) * (T(1) / S[i]) + lam * lsum * (T(1) / S[i]);
      T W[9];
      usvt(U, c, V, W);
      mat_mul_bt(W, F_new, P);
      break;
    }
    case MT_SNOW: {  // snow.py:56-74
      T S[3];
      T jp = Jp;
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        S[i] = gmin(gmax(sig[i], T(M.clamp_lo)), T(M.clamp_hi));
        jp *= sig[i] / S[i];
      }
      Jp_new = jp;
      usvt(U, S, V, F_new);
      const T h = gexp(T(10) * (T(1) - Jp));
      stress_corotated(mu * h, lam * h, F_new, U, V, J, P);
      break;
    }
    case MT_ELASTOPLASTIC: {  // elasto_plastic.py:44-71, stress base.py:94-99
      if (M.flags & MF_VON_MISES) {
        T e[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) e[i] = glog(gmax(sig[i], T(0.05)));
        const T m3 = (e[0] + e[1] + e[2]) / T(3);
        T eh[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) eh[i] = e[i] - m3;
        const T ehn = gsqrt(eh[0] * eh[0] + eh[1] * eh[1] + eh[2] * eh[2] + eps);
        const T dg = ehn - T(M.vm_ratio);
        if (dg > T(0)) {
          T S[3];
#pragma unroll
          for (int i = 0; i < 3; ++i) S[i] = gexp(e[i] - (dg / ehn) * eh[i]);
          usvt(U, S, V, F_new);
        } else {
#pragma unroll
          for (int k = 0; k < 9; ++k) F_new[k] = Ft[k];
        }
      } else {
        T S[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) S[i] = gmin(gmax(sig[i], T(M.clamp_lo)), T(M.clamp_hi));
        usvt(U, S, V, F_new);
      }
      stress_corotated(mu, lam, F_new, U, V, J, P);
      break;
    }
    case MT_MUSCLE:  // muscle.py:46-53 on top of elastic.py
    case MT_ELASTIC:
    default: {  // elastic.py:41-60
#pragma unroll
      for (int k = 0; k < 9; ++k) F_new[k] = Ft[k];
      if (M.flags & MF_NEOHOOKEAN)
        stress_neohookean(mu, lam, Ft, J, P);
      else
        stress_corotated(mu, lam, F_new, U, V, J, P);
      if (M.type == MT_MUSCLE) {
        // stiffness * actu * F (m m^T) F^T = stiffness * actu * (F m)(F m)^T
        T fm[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) fm[i] = Ft[i * 3 + 0] * mdir[0] + Ft[i * 3 + 1] * mdir[1] + Ft[i * 3 + 2] * mdir[2];
        const T k = T(M.stiffness) * actu;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j) P[i * 3 + j] += k * fm[i] * fm[j];
      }
      break;
    }
  }
}

// Quadratic B-spline weights of one axis (mpm_solver.py:381, 437)
template <typename T>
GB_HD void bspline_w(T fx, T* w) {
  w[0] = T(0.5) * (T(1.5) - fx) * (T(1.5) - fx);
  w[1] = T(0.75) - (fx - T(1)) * (fx - T(1));
  w[2] = T(0.5) * (fx - T(0.5)) * (fx - T(0.5));
}

}  // namespace gbmpm
