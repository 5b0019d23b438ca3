// Host build of the device math header (genesis_gb300/csrc/mpm_math.cuh) so that the CPU
// tests can check the CUDA path's SVD and material code against the oracle without a GPU.
#include "../genesis_gb300/csrc/mpm_adjoint.cuh"

using namespace gbmpm;

extern "C" {

float shim_svd3_f32(const float* A, float* U, float* sig, float* V) { return svd3<float, 4>(A, U, sig, V); }

double shim_svd3_f64(const double* A, double* U, double* sig, double* V) { return svd3<double, 8>(A, U, sig, V); }

// material update in float exactly as the P2G kernel runs it (FP32 SVD, FP64 re-solve if needed)
void shim_material_f32(int type, int flags, double mu, double lam, double alpha, double sand_coef, double clamp_lo,
                       double clamp_hi, double vm_ratio, double stiffness, const float* Ft, float Jp, float actu,
                       const float* mdir, float eps, float* F_new, float* Jp_new, float* P) {
  MaterialDev M{};
  M.type = type;
  M.flags = flags;
  M.mu = (float)mu;
  M.lam = (float)lam;
  M.alpha = (float)alpha;
  M.sand_coef = (float)sand_coef;
  M.clamp_lo = (float)clamp_lo;
  M.clamp_hi = (float)clamp_hi;
  M.vm_ratio = (float)vm_ratio;
  M.stiffness = (float)stiffness;
  float U[9], s[3], V[9];
  float res = svd3<float, 4>(Ft, U, s, V);
  if (!(res <= 1e-5f)) {
    double Ad[9], Ud[9], sd[3], Vd[9];
    for (int k = 0; k < 9; ++k) Ad[k] = Ft[k];
    svd3<double, 8>(Ad, Ud, sd, Vd);
    for (int k = 0; k < 9; ++k) {
      U[k] = (float)Ud[k];
      V[k] = (float)Vd[k];
    }
    for (int k = 0; k < 3; ++k) s[k] = (float)sd[k];
  }
  float jn;
  material_update<float>(M, Ft, U, s, V, Jp, actu, mdir, eps, F_new, jn, P);
  *Jp_new = jn;
}

void shim_bspline_w(float fx, float* w) { bspline_w<float>(fx, w); }

// Sand (type 2: p0 = alpha) / Snow (type 3: p0, p1 = clamp bounds) / clamped ElastoPlastic (type 4:
// p0, p1 = clamp bounds) / von Mises ElastoPlastic (EP_VON_MISES: p0 = yield stress / (2 mu)) update in
// double, and its adjoint (T = double or float) for the same F_tmp, Jp.
static MaterialDev plastic_material(int type, double mu, double lam, double p0, double p1) {
  MaterialDev M{};
  M.type = type == EP_VON_MISES ? MT_ELASTOPLASTIC : type;
  M.flags = type == EP_VON_MISES ? MF_VON_MISES : 0;
  M.mu = (float)mu;
  M.lam = (float)lam;
  if (type == MT_SAND) {
    M.alpha = (float)p0;
    M.sand_coef = (float)((3.0 * lam + 2.0 * mu) / (2.0 * mu));
  } else if (type == EP_VON_MISES) {
    M.vm_ratio = (float)p0;
  } else {
    M.clamp_lo = (float)p0;
    M.clamp_hi = (float)p1;
  }
  return M;
}

void shim_plastic_forward_f64(int type, double mu, double lam, double p0, double p1, double eps, const double* Ft,
                              double Jp, double* Fn, double* Jpn, double* P) {
  MaterialDev M = plastic_material(type, mu, lam, p0, p1);
  double U[9], s[3], V[9];
  svd3<double, 8>(Ft, U, s, V);
  const double mdir[3] = {0, 0, 1};
  double jn;
  // material_update<double> reads the float fields of M; mu/lam are passed in double through them
  material_update<double>(M, Ft, U, s, V, Jp, 0.0, mdir, eps, Fn, jn, P);
  *Jpn = jn;
}

void shim_plastic_adjoint_f64(int type, double mu, double lam, double p0, double p1, double eps, const double* Ft,
                              double Jp, const double* gFn, const double* gP, double gJpn, double* gFt, double* gJp,
                              double* gmu, double* glam) {
  double U[9], s[3], V[9];
  svd3<double, 8>(Ft, U, s, V);
  double a = 0, b = 0, c = 0;
  plastic_adjoint<double>(type, U, s, V, Jp, (double)(float)mu, (double)(float)lam, (double)(float)p0,
                          (double)(float)p1, eps, gFn, gP, gJpn, gFt, a, b, c);
  *gJp = a;
  *gmu = b;
  *glam = c;
}

void shim_plastic_adjoint_f32(int type, double mu, double lam, double p0, double p1, float eps, const float* Ft,
                              float Jp, const float* gFn, const float* gP, float gJpn, float* gFt, float* gJp) {
  float U[9], s[3], V[9];
  svd3<float, 4>(Ft, U, s, V);
  float a = 0, b = 0, c = 0;
  plastic_adjoint<float>(type, U, s, V, Jp, (float)mu, (float)lam, (float)p0, (float)p1, eps, gFn, gP, gJpn, gFt, a,
                         b, c);
  *gJp = a;
}
}
