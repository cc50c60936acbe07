// Brightness temperature along each ray: the trapezoidal optical-depth scan
// of Brightness.single (brightness.py:53-117) for sm_103a.
//
// One thread per (ray, frequency); a CTA covers a tile of consecutive
// frequencies of one ray, so the per-segment loads of ds / layer index /
// temperature are warp-uniform and the absorption loads alpha[layer][f0..f31]
// are one 128-byte line of the [nL][nf] float32 table (L2 resident).
//
// Per segment i (layers ii = layer4ds[i], ii1 = layer4ds[i+1], ds in cm):
//   tau_{i+1} = tau_i + (a0 + a1) ds / 2                   double-float
//   W_{i+1}   = a1 exp(-tau_{i+1})      or 2 a1 E2(tau_{i+1}) for 'disc'
//   intW     += (W_{i+1} + W_i) ds / 2                      compensated fp32
//   TbL      += (T1 W_{i+1} + T0 W_i) ds / 2                compensated fp32
// and Tb = T_cmb if TbL < T_cmb else TbL / intW (brightness.py:107-117).
// The last ds of the path is not used, as in the reference loop.
#include "rb_args.cuh"
#include <math_constants.h>

namespace rb {

constexpr double T_CMB = 2.725;   // utils.py:77

// Exponential integral E2(x), x >= 0, float64.
// x <= 1: power series  E2(x) = 1 + x (ln x - 1 + gamma) - sum_{k>=2} (-x)^k / ((k-1) k!)
//         (Abramowitz & Stegun 5.1.12 with the n = 2 digamma term).
// x > 1:  continued fraction of A&S 5.1.22 evaluated by the modified Lentz
//         method (Thompson & Barnett 1986).
__device__ double expint2(double x) {
  if (x == 0.0) return 1.0;
  if (!(x > 0.0)) return CUDART_NAN;
  if (x > 740.0) return 0.0;
  if (x <= 1.0) {
    const double euler = 0.57721566490153286061;
    double sum = 0.0;
    double term = x;   // (-x)^k / k!, starting at k = 1: -x ... built below
    double fact = -x;  // (-x)^1 / 1!
    for (int kk = 2; kk < 60; ++kk) {
      fact *= -x / kk;                 // (-x)^k / k!
      term = fact / (kk - 1);
      sum += term;
      if (fabs(term) < 1e-18 * fabs(sum) + 1e-300) break;
    }
    return 1.0 + x * (log(x) - 1.0 + euler) - sum;
  }
  const double tiny = 1e-300;
  const int n = 2;
  double bb = x + n;
  double c = 1.0 / tiny;
  double d = 1.0 / bb;
  double h = d;
  for (int i = 1; i < 200; ++i) {
    const double an = -(double)i * (n - 1 + i);
    bb += 2.0;
    d = 1.0 / (an * d + bb);
    c = bb + an / c;
    const double del = c * d;
    h *= del;
    if (fabs(del - 1.0) < 1e-16) break;
  }
  return h * exp(-x);
}


__device__ __forceinline__ void kahan_add(float& s, float& c, float v) {
  const float y = v - c;
  const float t = s + y;
  c = (t - s) - y;
  s = t;
}

__device__ __forceinline__ int wrap_layer(int l, int nL) { return l < 0 ? l + nL : l; }

__global__ void __launch_bounds__(128) rb_tb_kernel(TbArgs a) {
  const int ray = blockIdx.y;
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (ray >= a.nb) return;
  const bool valid = f < a.nf;
  const int fi = valid ? f : 0;
  const int nseg = a.nseg[ray];
  const double* ds = a.ds + (size_t)ray * a.max_seg;
  const int* lay = a.layer + (size_t)ray * a.max_seg;
  const size_t pbase = ((size_t)ray * a.nf + fi) * a.max_seg;
  float th = 0.f, tl = 0.f;          // tau (double-float)
  float W0 = 0.f;
  float iw = 0.f, iwc = 0.f, tb = 0.f, tbc = 0.f;
  if (valid && a.tau) {
    a.tau[pbase] = 0.0;
    a.W[pbase] = 0.0;
    a.TbL[pbase] = 0.0;
  }
  // layer indices follow Python semantics: negative values wrap
  int ii = nseg > 0 ? wrap_layer(lay[0], a.nL) : 0;
  float T0 = nseg > 0 ? (float)a.T[ii] : 0.f;
  float a0 = nseg > 0 ? a.alpha32[(size_t)ii * a.nf + fi] : 0.f;
  for (int i = 0; i + 1 < nseg; ++i) {
    const int ii1 = wrap_layer(lay[i + 1], a.nL);
    const float d = (float)(ds[i] * 1.0e5);   // km -> cm
    const float hd = 0.5f * d;
    const float a1 = a.alpha32[(size_t)ii1 * a.nf + fi];
    const float T1 = (float)a.T[ii1];
    const float dtau = (a0 + a1) * hd;
    float s, e;
    two_sum(th, dtau, s, e);
    e += tl;
    th = s + e;
    tl = e - (th - s);
    float W1;
    if (a.disc)
      W1 = (float)(2.0 * (double)a1 * expint2((double)th + (double)tl));
    else
      W1 = a1 * __expf(-th);
    kahan_add(iw, iwc, (W1 + W0) * hd);
    kahan_add(tb, tbc, fmaf(T1, W1, T0 * W0) * hd);
    if (valid && a.tau) {
      const size_t p = pbase + i + 1;
      a.tau[p] = (double)th + (double)tl;
      a.W[p] = (double)W1;
      a.TbL[p] = (double)tb - (double)tbc;
    }
    W0 = W1;
    T0 = T1;
    a0 = a1;
  }
  if (!valid) return;
  const double TbL = (double)tb - (double)tbc;
  const double IW = (double)iw - (double)iwc;
  a.Tb[(size_t)ray * a.nf + f] = (TbL < T_CMB) ? T_CMB : TbL / IW;
  if (a.intW) a.intW[(size_t)ray * a.nf + f] = IW;
}

// Weighted sum over rays (disc quadrature), one thread per frequency.
__global__ void rb_disc_avg_kernel(int nb, int nf, const double* Tb, const double* w, double* out) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  double s = 0.0;
  for (int r = 0; r < nb; ++r) s += w[r] * Tb[(size_t)r * nf + f];
  out[f] = s;
}

__global__ void rb_e2_kernel(int n, const double* x, double* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = expint2(x[i]);
}

cudaError_t launch_tb(const TbArgs& a, cudaStream_t st) {
  if (a.nb <= 0 || a.nf <= 0) return cudaSuccess;
  dim3 grid((a.nf + 127) / 128, a.nb);
  rb_tb_kernel<<<grid, 128, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_disc_avg(int nb, int nf, const double* Tb, const double* w, double* out,
                            cudaStream_t st) {
  rb_disc_avg_kernel<<<(nf + 127) / 128, 128, 0, st>>>(nb, nf, Tb, w, out);
  return cudaGetLastError();
}

cudaError_t launch_e2(int n, const double* x, double* out, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  rb_e2_kernel<<<(n + 127) / 128, 128, 0, st>>>(n, x, out);
  return cudaGetLastError();
}

}  // namespace rb
