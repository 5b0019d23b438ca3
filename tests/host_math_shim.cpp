// Host build of the device math header (genesis_gb300/csrc/mpm_math.cuh) so that the CPU
// tests can check the CUDA path's SVD and material code against the oracle without a GPU.
#include "../genesis_gb300/csrc/mpm_math.cuh"

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
}
