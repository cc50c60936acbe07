// Closed-form absorbers beside the line sums, float64:
//   co_ddb     (constituents/co/co_ddb.py:22-99): CO lines with a Voigt
//              (Hui rational approximation), Van Vleck-Weisskopf or
//              pressure-blended shape, chosen by other_dict['coshape'];
//   clouds_idp (constituents/clouds/clouds_idp.py:6-101): Rayleigh
//              absorption of cloud particles, 3 k fraction (-Im K).
// A CO catalogue has tens of lines, so these run once per (layer,
// frequency) in float64 (the Voigt real part in the far wings cancels to
// |f - f0| / gamma, up to ~1e5 at millibar pressures: float32 would lose
// it).  The forward kernel writes [2][nL][nf] in cm^-1 before the line-sum
// kernel, whose assembly adds them with their scales.  The adjoint kernel
// evaluates the same code on values carrying d/dT and d/dP (forward-mode)
// and contracts with d loss / d alpha per layer.
#include "rb_args.cuh"

namespace rb {

// ------------------------------------------------------------------ scalars
// A float64 value with its derivatives along T and P.
struct DTP {
  double v, t, p;
};
__device__ __forceinline__ double val(double x) { return x; }
__device__ __forceinline__ double val(const DTP& x) { return x.v; }
template <class S> __device__ __forceinline__ S cst(double v);
template <> __device__ __forceinline__ double cst<double>(double v) { return v; }
template <> __device__ __forceinline__ DTP cst<DTP>(double v) { return DTP{v, 0.0, 0.0}; }

__device__ __forceinline__ DTP operator+(DTP a, DTP b) { return {a.v + b.v, a.t + b.t, a.p + b.p}; }
__device__ __forceinline__ DTP operator-(DTP a, DTP b) { return {a.v - b.v, a.t - b.t, a.p - b.p}; }
__device__ __forceinline__ DTP operator-(DTP a) { return {-a.v, -a.t, -a.p}; }
__device__ __forceinline__ DTP operator*(DTP a, DTP b) {
  return {a.v * b.v, a.t * b.v + a.v * b.t, a.p * b.v + a.v * b.p};
}
__device__ __forceinline__ DTP operator/(DTP a, DTP b) {
  const double q = a.v / b.v;
  return {q, (a.t - q * b.t) / b.v, (a.p - q * b.p) / b.v};
}
__device__ __forceinline__ DTP operator+(DTP a, double b) { return {a.v + b, a.t, a.p}; }
__device__ __forceinline__ DTP operator+(double b, DTP a) { return {a.v + b, a.t, a.p}; }
__device__ __forceinline__ DTP operator-(DTP a, double b) { return {a.v - b, a.t, a.p}; }
__device__ __forceinline__ DTP operator-(double b, DTP a) { return {b - a.v, -a.t, -a.p}; }
__device__ __forceinline__ DTP operator*(DTP a, double b) { return {a.v * b, a.t * b, a.p * b}; }
__device__ __forceinline__ DTP operator*(double b, DTP a) { return {a.v * b, a.t * b, a.p * b}; }
__device__ __forceinline__ DTP operator/(DTP a, double b) { return {a.v / b, a.t / b, a.p / b}; }
__device__ __forceinline__ DTP operator/(double b, DTP a) {
  const double q = b / a.v;
  return {q, -q * a.t / a.v, -q * a.p / a.v};
}
__device__ __forceinline__ double sqrt_(double x) { return sqrt(x); }
__device__ __forceinline__ DTP sqrt_(DTP x) {
  const double r = sqrt(x.v);
  const double h = 0.5 / r;
  return {r, h * x.t, h * x.p};
}
__device__ __forceinline__ double exp_(double x) { return exp(x); }
__device__ __forceinline__ DTP exp_(DTP x) {
  const double e = exp(x.v);
  return {e, e * x.t, e * x.p};
}
__device__ __forceinline__ double pow_(double x, double e) { return pow(x, e); }
__device__ __forceinline__ DTP pow_(DTP x, double e) {
  const double r = pow(x.v, e);
  const double d = e * r / x.v;
  return {r, d * x.t, d * x.p};
}

// Real part of n / d for complex n = (nr, ni), d = (dr, di) (Smith's
// scaling: no overflow of |d|^2).
template <class S>
__device__ __forceinline__ S re_div(S nr, S ni, S dr, S di) {
  if (fabs(val(dr)) >= fabs(val(di))) {
    const S q = di / dr;
    return (nr + ni * q) / (dr + di * q);
  }
  const S q = dr / di;
  return (nr * q + ni) / (dr * q + di);
}

// ------------------------------------------------------------------ co_ddb
// Voigt coefficients of co_ddb.py:25-28 (Hui, Armstrong & Wray 1978
// rational approximation of the complex probability function):
// w(xi) = sum a_j xi^j / sum b_j xi^j, a_7 = 0, b_7 = 1.
__device__ constexpr double VOIGT_A[8] = {122.60793178, 214.38238869, 181.92853309, 93.15558046,
                                          30.18014220,  5.91262621,   0.56418958,   0.0};
__device__ constexpr double VOIGT_B[8] = {122.60793178, 352.73062511, 457.33447878, 348.70391772,
                                          170.35400182, 53.99290691,  10.47985711,  1.0};
constexpr double CO_COEF = 7.244E+21;   // co_ddb.py:6
constexpr double CO_T0 = 296.0;
constexpr double CO_HCK = 1.438396;
constexpr double GHZ_D = 29.9792458;
constexpr double PI_D = 3.14159265358979323846;
constexpr double SQRT_PI_D = 1.7724538509055160273;

template <class S>
__device__ S co_alpha(const ExtraArgs& a, int L, S T, S P, double f) {
  const int nL = a.nL;
  const double* X = a.X;
  const S Ph2 = P * X[X_H2 * nL + L], Phe = P * X[X_HE * nL + L], Pco = P * X[X_CO * nL + L];
  const S Tr = CO_T0 / T;
  const S gamma = pow_(Tr, 0.7) * (1.960 * Ph2 + 1.200 * Phe + 6.000 * Pco);   // co_ddb.py:44-50
  const S g2 = gamma * gamma;
  S w = (P - 0.001) / (0.1 - 0.001);                                           // co_ddb.py:57-61
  if (val(w) < 0.0) w = cst<S>(0.0);
  else if (val(w) > 1.0) w = cst<S>(1.0);
  const int shape = a.cfg.coshape;
  const bool do_voigt = val(P) <= 0.1 || shape == CO_VOIGT || shape == CO_DIFF;
  const bool do_vvw = val(P) >= 0.001 || shape == CO_VVW || shape == CO_DIFF;
  const double f2 = f * f;
  S betaD = cst<S>(1.0), vscale = cst<S>(0.0), xr = cst<S>(0.0);
  if (do_voigt) {                                   // Doppler width, co_ddb.py:70
    betaD = 4.3e-7 * sqrt_(T / 28.0) * f;
    vscale = GHZ_D / (SQRT_PI_D * betaD);
    xr = gamma / betaD;
  }
  const S invT = 1.0 / T;
  S acc = cst<S>(0.0);
  for (int l = 0; l < a.nco; ++l) {
    const double f0 = a.co_f0[l];
    S sV = cst<S>(0.0), sW = cst<S>(0.0);
    if (do_voigt) {                                 // co_ddb.py:68-79
      const S xi_r = xr, xi_i = (f - f0) / betaD;
      S nr = cst<S>(VOIGT_A[6]), ni = cst<S>(0.0);
      S dr = cst<S>(VOIGT_B[7]), di = cst<S>(0.0);
      for (int j = 6; j >= 0; --j) {
        const S tr = dr * xi_r - di * xi_i;
        di = dr * xi_i + di * xi_r;
        dr = tr + VOIGT_B[j];
      }
      for (int j = 5; j >= 0; --j) {
        const S tr = nr * xi_r - ni * xi_i;
        ni = nr * xi_i + ni * xi_r;
        nr = tr + VOIGT_A[j];
      }
      sV = vscale * re_div(nr, ni, dr, di);
    }
    if (do_vvw) {                                   // co_ddb.py:81-85, zeta = delta = 0
      const double c2 = f0 * f0;
      const S num = gamma * f2 + gamma * (c2 + g2);
      const S dd = (f2 - c2) - g2;
      const S den = dd * dd + (4.0 * f2) * g2;
      sW = (GHZ_D * 2.0 * (f / f0) * (f / f0) / PI_D) * (num / den);
    }
    switch (shape) {                                // co_ddb.py:86-93
      case CO_VOIGT: acc = acc + sV; break;
      case CO_VVW: acc = acc + sW; break;
      case CO_DIFF: acc = acc + (sV - sW); break;
      default: {
        const S ITG = a.co_I0[l] * exp_(-((invT - 1.0 / CO_T0) * (a.co_E[l] * CO_HCK)));
        acc = acc + (w * sW + (1.0 - w) * sV) * ITG;
      }
    }
  }
  return (CO_COEF / CO_T0) * (Pco * pow_(Tr, 3.5)) * acc;                     // co_ddb.py:95
}

// ------------------------------------------------------------------ clouds_idp
// Imaginary part of the dielectric constant of ice below 0 C, log-log
// interpolated in frequency (clouds_idp.py:68-69,88-99).
__device__ constexpr double ICE_FR[9] = {1.0E8, 3.0E8, 1.0E9, 2.0E9, 3.0E9, 5.0E9, 1.0E10, 3.0E10, 1.0E11};
__device__ constexpr double ICE_EIMAG[9] = {8.0E-3, 1.5E-3, 8.0E-4, 1.0E-3, 1.2E-3, 1.5E-3, 3.0E-3, 8.0E-3, 2.0E-2};

// Dielectric constant e = E1 - i E2 of water (clouds_idp.py:75-101).
template <class S>
__device__ void water(double f, S T, S& E1, S& E2) {
  const S Tc = T - 273.0;
  const double fHz = f * 1.0E9;
  if (val(Tc) >= 0.0) {
    const S Tc2 = Tc * Tc, Tc3 = Tc2 * Tc;
    const S RelT = 1.1109E-10 - Tc * 3.824E-12 + Tc2 * 6.938E-14 - Tc3 * 5.096E-16;
    S E0 = 88.045 - 0.4147 * Tc + Tc2 * 6.295E-4 + Tc3 * 1.075E-5;
    if (val(E0) < 0.0) E0 = cst<S>(0.0);
    const double EINF = 4.9;
    const S x = fHz * RelT;
    const S q = 1.0 + x * x;
    E1 = EINF + (E0 - EINF) / q;
    E2 = x * (E0 - EINF) / q;
    if (val(E2) < 0.0) E2 = cst<S>(0.0);
  } else {
    E1 = cst<S>(3.17);
    const double LF = log10(fHz);
    int j = 0;
    for (; j < 8; ++j)
      if (ICE_FR[j + 1] >= fHz) break;
    if (j == 8) j = 7;                 // the reference loop ends on its last index
    const double LF0 = log10(ICE_FR[j]), LF1 = log10(ICE_FR[j + 1]);
    const double DLF = (LF - LF0) / (LF1 - LF0);
    const double X0 = log10(ICE_EIMAG[j]), X1 = log10(ICE_EIMAG[j + 1]);
    E2 = cst<S>(pow(10.0, X0 + DLF * (X1 - X0)));
  }
}

// -Im K, K = (e - 1) / (e + 2), e = E1 - i E2 (clouds_idp.py:64-68).
template <class S>
__device__ __forceinline__ S neg_im_K(S E1, S E2) {
  const S a = E1 + 2.0;
  return (3.0 * E2) / (a * a + E2 * E2);
}

// Constant refractive index n = nr - i ni: e = n^2.
__device__ __forceinline__ double neg_im_K_n(double nr, double ni) {
  return neg_im_K<double>(nr * nr - ni * ni, 2.0 * nr * ni);
}

template <class S>
__device__ S cloud_alpha(const ExtraArgs& a, int L, S T, double f) {
  const int nL = a.nL, m = a.cfg.cloud_mask;
  const double* X = a.X;
  const double k3 = 3.0 * (2.0 * PI_D * f / GHZ_D);    // 3 k, k in cm^-1
  S alpha = cst<S>(0.0);
  if (m & (CL_ICE | CL_WATER)) {
    S E1, E2;
    water(f, T, E1, E2);
    const S mk = neg_im_K(E1, E2);
    if (m & CL_ICE) alpha = alpha + (k3 * (X[X_CL_H2O * nL + L] / 0.9)) * mk;
    if (m & CL_WATER) alpha = alpha + (k3 * (X[X_CL_SOLN * nL + L] / 1.0)) * mk;
  }
  if (m & CL_NH4SH) alpha = alpha + k3 * (X[X_CL_NH4SH * nL + L] / 1.2) * neg_im_K_n(1.7, 0.005);
  if (m & CL_NH3ICE) alpha = alpha + k3 * (X[X_CL_NH3 * nL + L] / 1.6) * neg_im_K_n(1.3, 0.0001);
  if (m & CL_H2SICE) alpha = alpha + k3 * (X[X_CL_H2S * nL + L] / 1.5) * neg_im_K_n(1.15, 0.0001);
  if (m & CL_CH4) alpha = alpha + k3 * (X[X_CL_CH4 * nL + L] / 1.0) * neg_im_K_n(1.3, 0.00001);
  if (val(alpha) < 0.0) alpha = cst<S>(0.0);             // clouds_idp.py:53-55
  return alpha;
}

// ------------------------------------------------------------------ kernels
__global__ void __launch_bounds__(256) rb_alpha_extra_kernel(ExtraArgs a) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (size_t)a.nL * a.nf) return;
  const int L = (int)(idx / a.nf), j = (int)(idx % a.nf);
  const double f = a.freqs[j], T = a.T[L], P = a.P[L];
  a.out[idx] = a.cfg.use_co ? co_alpha<double>(a, L, T, P, f) : 0.0;
  a.out[(size_t)a.nL * a.nf + idx] = a.cfg.use_clouds ? cloud_alpha<double>(a, L, T, f) : 0.0;
}

// One CTA per layer: sum over frequencies of d loss / d alpha times the
// scaled derivatives of the co and cloud terms (cm^-1).
constexpr int EXTRA_VJP_THREADS = 128;

__global__ void __launch_bounds__(EXTRA_VJP_THREADS) rb_extra_vjp_kernel(ExtraArgs a) {
  const int L = blockIdx.x;
  __shared__ double red[2][EXTRA_VJP_THREADS / 32];
  const DTP T{a.T[L], 1.0, 0.0}, P{a.P[L], 0.0, 1.0};
  const double sco = a.scale ? a.scale[(size_t)L * NGAS + GAS_CO] : 1.0;
  const double scl = a.scale ? a.scale[(size_t)L * NGAS + GAS_CLOUDS] : 1.0;
  double gt = 0.0, gp = 0.0;
  for (int j = threadIdx.x; j < a.nf; j += blockDim.x) {
    const double g = (double)a.galpha[(size_t)L * a.nf + j];
    if (g == 0.0) continue;
    const double f = a.freqs[j];
    if (a.cfg.use_co) {
      const DTP c = co_alpha<DTP>(a, L, T, P, f);
      gt += g * sco * c.t;
      gp += g * sco * c.p;
    }
    if (a.cfg.use_clouds) {
      const DTP c = cloud_alpha<DTP>(a, L, T, f);
      gt += g * scl * c.t;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    gt += __shfl_xor_sync(0xffffffffu, gt, o);
    gp += __shfl_xor_sync(0xffffffffu, gp, o);
  }
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    red[0][w] = gt;
    red[1][w] = gp;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double st = 0.0, sp = 0.0;
    for (int k = 0; k < EXTRA_VJP_THREADS / 32; ++k) {
      st += red[0][k];
      sp += red[1][k];
    }
    a.grad[2 * L] = st;
    a.grad[2 * L + 1] = sp;
  }
}

cudaError_t launch_extra(const ExtraArgs& a, cudaStream_t st) {
  const size_t n = (size_t)a.nL * a.nf;
  if (n == 0) return cudaSuccess;
  rb_alpha_extra_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_extra_vjp(const ExtraArgs& a, cudaStream_t st) {
  if (a.nL == 0) return cudaSuccess;
  rb_extra_vjp_kernel<<<a.nL, EXTRA_VJP_THREADS, 0, st>>>(a);
  return cudaGetLastError();
}

}  // namespace rb
