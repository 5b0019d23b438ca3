// mpm_adjoint.cuh - adjoint of the plastic material updates (Sand, Snow) of one particle, for the
// differentiable substep.  Host and device (the CPU tests compile it with g++ and check it against
// FP64 central differences of material_update).
//
// Both materials are isotropic functions of F_tmp = U diag(s) V^T (s signed, rotation-variant
// SVD): F_new = U diag(sn) V^T and the stress P = U diag(tau) U^T with per-axis sn(s, Jp, mu, lam),
// tau(s, Jp, mu, lam) and a scalar Jp_new:
//   Sand (sand.py:47-84):  e = log max(|s|, 1e-4), tr = sum e + Jp, e^ = e - tr/3,
//     |e^| = sqrt(|e^|^2 + eps); tr >= 0: sn = 1, Jp_new = tr; else Jp_new = 0 and
//     sn = exp(e - max(0, dg)/|e^| e^), dg = |e^| + (3 lam + 2 mu)/(2 mu) tr alpha;
//     tau_i = 2 mu log sn_i + lam sum_j log sn_j   (U c V^T F_new^T with c_i = tau_i / sn_i).
//   Snow (snow.py:56-74):  sn = clamp(s, 1 - yl, 1 + yh), Jp_new = Jp prod s/sn, J = prod s,
//     h = exp(10 (1 - Jp)), tau_i = 2 mu h (sn_i - 1) sn_i + lam h J (J - 1)
//     (the corotated stress 2 mu h (F_new - U V^T) F_new^T + lam h J (J-1) I).
//   ElastoPlastic (elasto_plastic.py:44-71), Jp unchanged, tau_i = 2 mu (sn_i - 1) sn_i + lam J (J - 1):
//     clamped (MT_ELASTOPLASTIC): sn = clamp(s, 1 - yl, 1 + yh);
//     von Mises (EP_VON_MISES): e = log max(s, 0.05), e^ = e - mean(e), |e^| = sqrt(|e^|^2 + eps),
//     dg = |e^| - yield_stress / (2 mu); dg > 0: sn = exp(e - dg/|e^| e^), else sn = s.
// The per-axis functions and their Jacobians w.r.t. (s0, s1, s2, Jp, mu, lam) come from forward-
// mode dual numbers.  The off-diagonal part of the adjoint uses the divided differences
// (f_i - f_j)/(s_i - s_j), taken from the Jacobian (J_ii - J_ij) when s_i and s_j nearly coincide
// (and the quotient itself across a clamp bound), so the adjoint stays finite at F = I where the
// generic SVD backward (mpm_solver.py:1229-1252) divides by s_j^2 - s_i^2:
//   F_new:  dF_new^_ij = (a+b)/2 dA_ij + (a-b)/2 dA_ji,  a = (f_i-f_j)/(s_i-s_j), b = (f_i+f_j)/(s_i+s_j)
//   P:      (U^T dP U)_ij = q (s_j dA_ij + s_i dA_ji)/(s_i + s_j),  q = (tau_i - tau_j)/(s_i - s_j)
// with dA = U^T dF_tmp V; the diagonal follows the Jacobian.
#pragma once

#include "mpm_math.cuh"

namespace gbmpm {

// ---------------------------------------------------------------- dual numbers (6 tangents)
constexpr int ND = 6;  // d/d s0, s1, s2, Jp, mu, lam

template <typename T>
struct Dual {
  T v;
  T d[ND];
};

template <typename T> GB_HD Dual<T> dconst(T v) {
  Dual<T> r;
  r.v = v;
#pragma unroll
  for (int k = 0; k < ND; ++k) r.d[k] = T(0);
  return r;
}
template <typename T> GB_HD Dual<T> dvar(T v, int k) {
  Dual<T> r = dconst(v);
  r.d[k] = T(1);
  return r;
}
template <typename T> GB_HD Dual<T> operator+(const Dual<T>& a, const Dual<T>& b) {
  Dual<T> r;
  r.v = a.v + b.v;
#pragma unroll
  for (int k = 0; k < ND; ++k) r.d[k] = a.d[k] + b.d[k];
  return r;
}
template <typename T> GB_HD Dual<T> operator-(const Dual<T>& a, const Dual<T>& b) {
  Dual<T> r;
  r.v = a.v - b.v;
#pragma unroll
  for (int k = 0; k < ND; ++k) r.d[k] = a.d[k] - b.d[k];
  return r;
}
template <typename T> GB_HD Dual<T> operator*(const Dual<T>& a, const Dual<T>& b) {
  Dual<T> r;
  r.v = a.v * b.v;
#pragma unroll
  for (int k = 0; k < ND; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
  return r;
}
template <typename T> GB_HD Dual<T> operator/(const Dual<T>& a, const Dual<T>& b) {
  Dual<T> r;
  r.v = a.v / b.v;
  const T ib = T(1) / b.v;
#pragma unroll
  for (int k = 0; k < ND; ++k) r.d[k] = (a.d[k] - r.v * b.d[k]) * ib;
  return r;
}
template <typename T> GB_HD Dual<T> operator*(T s, const Dual<T>& a) {
  Dual<T> r;
  r.v = s * a.v;
#pragma unroll
  for (int k = 0; k < ND; ++k) r.d[k] = s * a.d[k];
  return r;
}
template <typename T> GB_HD Dual<T> dlog(const Dual<T>& a) {
  Dual<T> r;
  r.v = glog(a.v);
  const T ia = T(1) / a.v;
#pragma unroll
  for (int k = 0; k < ND; ++k) r.d[k] = a.d[k] * ia;
  return r;
}
template <typename T> GB_HD Dual<T> dexp(const Dual<T>& a) {
  Dual<T> r;
  r.v = gexp(a.v);
#pragma unroll
  for (int k = 0; k < ND; ++k) r.d[k] = a.d[k] * r.v;
  return r;
}
template <typename T> GB_HD Dual<T> dsqrt(const Dual<T>& a) {
  Dual<T> r;
  r.v = gsqrt(a.v);
  const T h = T(0.5) / r.v;
#pragma unroll
  for (int k = 0; k < ND; ++k) r.d[k] = a.d[k] * h;
  return r;
}

// ---------------------------------------------------------------- principal-axis material laws
// type: MT_SAND, MT_SNOW, MT_ELASTOPLASTIC or EP_VON_MISES; p0, p1: sand alpha ((3 lam + 2 mu)/(2 mu)
// is derived here); snow and clamped ElastoPlastic clamp_lo, clamp_hi; von Mises yield_stress/(2 mu).
constexpr int EP_VON_MISES = 64 + MT_ELASTOPLASTIC;
template <typename T>
GB_HD void plastic_principal(int type, const Dual<T>* s, const Dual<T>& Jp, const Dual<T>& mu, const Dual<T>& lam,
                             T p0, T p1, T eps, Dual<T>* sn, Dual<T>* tau, Dual<T>& Jpn) {
  const Dual<T> two = dconst(T(2));
  if (type == MT_SAND) {
    Dual<T> e[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const T a = gabs(s[i].v);
      if (a > T(1e-4)) {
        e[i] = dlog(s[i].v < T(0) ? T(-1) * s[i] : s[i]);
      } else {
        e[i] = dconst(glog(T(1e-4)));
      }
    }
    const Dual<T> tr = e[0] + e[1] + e[2] + Jp;
    const Dual<T> third = dconst(T(1) / T(3));
    Dual<T> eh[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) eh[i] = e[i] - tr * third;
    const Dual<T> ehn = dsqrt(eh[0] * eh[0] + eh[1] * eh[1] + eh[2] * eh[2] + dconst(eps));
    if (tr.v >= T(0)) {
      Jpn = tr;
#pragma unroll
      for (int i = 0; i < 3; ++i) sn[i] = dconst(T(1));
    } else {
      Jpn = dconst(T(0));
      const Dual<T> coef = (dconst(T(3)) * lam + two * mu) / (two * mu);
      const Dual<T> dg = ehn + coef * tr * dconst(p0);
      if (dg.v > T(0)) {
#pragma unroll
        for (int i = 0; i < 3; ++i) sn[i] = dexp(e[i] - dg / ehn * eh[i]);
      } else {
#pragma unroll
        for (int i = 0; i < 3; ++i) sn[i] = dexp(e[i]);
      }
    }
    Dual<T> l[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) l[i] = dlog(sn[i]);
    const Dual<T> L = l[0] + l[1] + l[2];
#pragma unroll
    for (int i = 0; i < 3; ++i) tau[i] = two * mu * l[i] + lam * L;
  } else if (type == MT_ELASTOPLASTIC || type == EP_VON_MISES) {
    Jpn = Jp;
    if (type == MT_ELASTOPLASTIC) {
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        if (s[i].v < p0) sn[i] = dconst(p0);
        else if (s[i].v > p1) sn[i] = dconst(p1);
        else sn[i] = s[i];
      }
    } else {
      Dual<T> e[3];
#pragma unroll
      for (int i = 0; i < 3; ++i) e[i] = s[i].v > T(0.05) ? dlog(s[i]) : dconst(glog(T(0.05)));
      const Dual<T> m3 = (e[0] + e[1] + e[2]) / dconst(T(3));
      Dual<T> eh[3];
#pragma unroll
      for (int i = 0; i < 3; ++i) eh[i] = e[i] - m3;
      const Dual<T> ehn = dsqrt(eh[0] * eh[0] + eh[1] * eh[1] + eh[2] * eh[2] + dconst(eps));
      const Dual<T> dg = ehn - dconst(p0);
      if (dg.v > T(0)) {
#pragma unroll
        for (int i = 0; i < 3; ++i) sn[i] = dexp(e[i] - (dg / ehn) * eh[i]);
      } else {
#pragma unroll
        for (int i = 0; i < 3; ++i) sn[i] = s[i];
      }
    }
    const Dual<T> J = s[0] * s[1] * s[2];
    const Dual<T> lj = lam * J * (J - dconst(T(1)));
#pragma unroll
    for (int i = 0; i < 3; ++i) tau[i] = two * mu * (sn[i] - dconst(T(1))) * sn[i] + lj;
  } else {  // MT_SNOW
    Jpn = Jp;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      if (s[i].v < p0) sn[i] = dconst(p0);
      else if (s[i].v > p1) sn[i] = dconst(p1);
      else sn[i] = s[i];
      Jpn = Jpn * s[i] / sn[i];
    }
    const Dual<T> J = s[0] * s[1] * s[2];
    const Dual<T> h = dexp(dconst(T(10)) * (dconst(T(1)) - Jp));
    const Dual<T> lj = lam * h * J * (J - dconst(T(1)));
#pragma unroll
    for (int i = 0; i < 3; ++i) tau[i] = two * mu * h * (sn[i] - dconst(T(1))) * sn[i] + lj;
  }
}

// (f_i - f_j)/(s_i - s_j) of a symmetric per-axis function f with Jacobian d f_i / d s_k: the quotient
// itself when s_i and s_j are apart (its cancellation error stays near float rounding / 1e-4) or lie
// on different smooth pieces of f (a clamp bound between them), else the mean of the one-sided
// limits d f_i/d s_i - d f_i/d s_j and d f_j/d s_j - d f_j/d s_i (second order).
template <typename T>
GB_HD T divided_difference(const T* s, const T* f, T jii, T jij, T jjj, T jji, int i, int j, bool same_piece) {
  const T ds = s[i] - s[j];
  const T scale = gabs(s[i]) + gabs(s[j]);
  const T rel = sizeof(T) == 8 ? T(1e-6) : T(1e-4);
  if (!same_piece || gabs(ds) > rel * scale) return (f[i] - f[j]) / ds;
  return T(0.5) * ((jii - jij) + (jjj - jji));
}

template <typename T> GB_HD T signmax(T a, T e) { return a >= T(0) ? gmax(a, e) : -gmax(-a, e); }

// Adjoint of (F_new, Jp_new, P) = plastic update of (F_tmp = U diag(s) V^T, Jp): given gFn = dL/dF_new,
// gP = dL/dP (P before the stress scale) and gJpn = dL/dJp_new, writes dL/dF_tmp into gFt and returns
// dL/dJp, dL/dmu, dL/dlam through gJp, gmu, glam (added).
template <typename T>
GB_HD void plastic_adjoint(int type, const T* U, const T* s, const T* V, T Jp, T mu, T lam, T p0, T p1, T eps,
                           const T* gFn, const T* gP, T gJpn, T* gFt, T& gJp, T& gmu, T& glam) {
  Dual<T> sd[3], sn[3], tau[3], Jpn;
#pragma unroll
  for (int i = 0; i < 3; ++i) sd[i] = dvar(s[i], i);
  plastic_principal<T>(type, sd, dvar(Jp, 3), dvar(mu, 4), dvar(lam, 5), p0, p1, eps, sn, tau, Jpn);
  // G^ = U^T gFn V,  P^ = U^T gP U
  T G[9], Ph[9], tmp[9];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      tmp[i * 3 + j] = gFn[i * 3 + 0] * V[0 * 3 + j] + gFn[i * 3 + 1] * V[1 * 3 + j] + gFn[i * 3 + 2] * V[2 * 3 + j];
    }
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      G[i * 3 + j] = U[0 * 3 + i] * tmp[0 * 3 + j] + U[1 * 3 + i] * tmp[1 * 3 + j] + U[2 * 3 + i] * tmp[2 * 3 + j];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      tmp[i * 3 + j] = gP[i * 3 + 0] * U[0 * 3 + j] + gP[i * 3 + 1] * U[1 * 3 + j] + gP[i * 3 + 2] * U[2 * 3 + j];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      Ph[i * 3 + j] = U[0 * 3 + i] * tmp[0 * 3 + j] + U[1 * 3 + i] * tmp[1 * 3 + j] + U[2 * 3 + i] * tmp[2 * 3 + j];
  // diagonal: d/d(s, Jp, mu, lam) of <G, diag(sn)> + <P^, diag(tau)> + gJpn Jp_new
  T g[ND];
#pragma unroll
  for (int k = 0; k < ND; ++k) {
    T a = gJpn * Jpn.d[k];
#pragma unroll
    for (int i = 0; i < 3; ++i) a += G[i * 4] * sn[i].d[k] + Ph[i * 4] * tau[i].d[k];
    g[k] = a;
  }
  T A[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) A[k] = T(0);
  A[0] = g[0];
  A[4] = g[1];
  A[8] = g[2];
  gJp += g[3];
  gmu += g[4];
  glam += g[5];
  // off-diagonal pairs
  const T f[3] = {sn[0].v, sn[1].v, sn[2].v};
  const T t[3] = {tau[0].v, tau[1].v, tau[2].v};
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = i + 1; j < 3; ++j) {
      // Snow and the clamped ElastoPlastic clamp each axis on its own: a bound may lie between s_i
      // and s_j; von Mises floors each log strain at 0.05
      bool same = true;
      if (type == MT_SNOW || type == MT_ELASTOPLASTIC)
        same = (s[i] < p0) == (s[j] < p0) && (s[i] > p1) == (s[j] > p1);
      else if (type == EP_VON_MISES)
        same = (s[i] > T(0.05)) == (s[j] > T(0.05));
      const T a = divided_difference(s, f, sn[i].d[i], sn[i].d[j], sn[j].d[j], sn[j].d[i], i, j, same);
      const T b = (f[i] + f[j]) / signmax(s[i] + s[j], T(1e-6));
      A[i * 3 + j] += T(0.5) * (a + b) * G[i * 3 + j] + T(0.5) * (a - b) * G[j * 3 + i];
      A[j * 3 + i] += T(0.5) * (a - b) * G[i * 3 + j] + T(0.5) * (a + b) * G[j * 3 + i];
      const T q = divided_difference(s, t, tau[i].d[i], tau[i].d[j], tau[j].d[j], tau[j].d[i], i, j, same);
      const T w = q * (Ph[i * 3 + j] + Ph[j * 3 + i]) / signmax(s[i] + s[j], T(1e-6));
      A[i * 3 + j] += w * s[j];
      A[j * 3 + i] += w * s[i];
    }
  // gFt = U A V^T
  T UA[9];
  mat_mul(U, A, UA);
  mat_mul_bt(UA, V, gFt);
}

}  // namespace gbmpm
