// Absorption coefficient of every (layer, frequency): the per-gas line sums
// of radioBEAR's Jupiter formalisms, restated for sm_103a.
//
//   rb_layer_prep_kernel  one warp per layer, float64: partial pressures,
//                         width / shift / coupling coefficients, strength
//                         prefactors and the per-family log-strength offset M.
//   rb_alpha_kernel       one CTA per (layer, frequency tile); one thread per
//                         frequency.  Lines are staged in shared-memory chunks
//                         (one line per thread computes its layer-dependent
//                         record), then every thread sweeps the chunk for its
//                         frequency.  Sums are float32 with compensated
//                         accumulation; the prefactor, unit conversion, clamp,
//                         blend and scaling are applied in float64.
//
// Numerics (per line l, frequency f, F = f^2):
//   Ben-Reuven  S_l [(g-z) F + (g+z) K_l] / [(F - K_l)^2 + 4 F g^2],
//               K_l = (fo+d)^2 + g^2 - z^2      (nh3_hs.py:216-225, h2s_ddb.py:270-272)
//   Gross       S_l g / [(F - fo^2)^2 + 4 F g^2]          (nh3_hs.py:260-263)
//   VVW         S_l df [1/((f-fo)^2+df^2) + 1/((f+fo)^2+df^2) - 2/(750^2+df^2)]
//                                                         (h2o_bk.py:174-187)
// with the common factor f^2 (and the 1/fo^2 of (f/fo)^2, folded into S_l)
// taken out of the sum.  F - K is evaluated as a double-float difference for
// lines whose centre lies within [0.75 fmin, 1.3 fmax] of the warp's
// frequencies (there FP32 would cancel); elsewhere plain FP32 is exact to a
// few ulp.  Pairs of lines share one reciprocal:
//   n1/d1 + n2/d2 = (n1 d2 + n2 d1) / (d1 d2).
#include "rb_args.cuh"
#include <math_constants.h>

namespace rb {

// nh3_hs.py:44-56
__device__ constexpr double HS_HC = 19.858252418E-24;
__device__ constexpr double HS_KB = 1.38E-23;
__device__ constexpr double HS_COEF = 1.0E6 * 6.02297E23 / 8.31432E7;
__device__ constexpr double HS_TO = 300.0;
__device__ constexpr double GHZ_INVCM = 29.9792458;
__device__ constexpr double GEISA_COEF = 7.244E+21;
__device__ constexpr double HCK = 1.438396;
__device__ constexpr double DB_PER_INVCM = 434294.5;
__device__ constexpr double INV_CON[2] = {0.9301, 0.9862};

// Inversion coefficient sets (nh3_hs.py:139-168): gnu_H2, gnu_He, gnu_NH3,
// GAMMA_H2, GAMMA_He, GAMMA_NH3, zeta_H2, zeta_He, zeta_NH3, Z_H2, Z_He,
// Z_NH3, d
__device__ constexpr double INV_SET[2][13] = {
    {1.640, 0.75, 0.852, 0.7756, 0.666, 1.0, 1.262, 0.3, 0.5296, 0.7964, 0.667, 1.554, -0.0498},
    {1.7465, 0.9779, 0.7298, 0.8202, 1.0, 1.0, 1.2163, 0.0291, 0.5152, 0.8873, 0.8994,
     2.0 / 3.0, -0.0627}};


__device__ double scale_pass(const LineTable& t, double cE, int lane) {
  // FP32 estimate of max_l (lnI_l + cE*E_l); the value only sets the scale.
  float m = -CUDART_INF_F;
  float ce = (float)cE;
  for (int i = lane; i < t.n; i += 32) m = fmaxf(m, fmaf(ce, t.E32[i], t.lnI32[i]));
  for (int o = 16; o; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  return isfinite(m) ? (double)m : 0.0;
}

__global__ void __launch_bounds__(32) rb_layer_prep_kernel(PrepArgs a) {
  const int L = blockIdx.x;
  const int lane = threadIdx.x;
  if (L >= a.nL) return;
  __shared__ LayerParams sp;
  const double P = a.P[L], T = a.T[L];
  const double* X = a.X;
  const int nL = a.nL;
  const double Ph2 = P * X[X_H2 * nL + L], Phe = P * X[X_HE * nL + L];
  const double Pch4 = P * X[X_CH4 * nL + L], Pnh3 = P * X[X_NH3 * nL + L];
  const double Ph2o = P * X[X_H2O * nL + L], Ph2s = P * X[X_H2S * nL + L];
  const double Pph3 = P * X[X_PH3 * nL + L];
  const double Tdiv = HS_TO / T;
  const double cE_hs = -(1.0 / T - 1.0 / HS_TO) * HS_HC / HS_KB;
  const double hs_pref = HS_COEF * (Pnh3 / HS_TO) * pow(HS_TO / T, 3.5) * GHZ_INVCM;
  if (lane == 0) {
    sp.P = P;
    sp.T = T;
    for (int f = 0; f < NFAM; ++f) {
      sp.fam[f].fac = 0.0;
      sp.fam[f].M = 0.0;
      sp.fam[f].cE = 0.0;
      for (int s = 0; s < 2; ++s)
        for (int k = 0; k < 8; ++k) sp.fam[f].c[s][k] = 0.f;
    }
    // NH3 formalism choice (nh3_hs_sjs.py:6-26)
    int mode = a.cfg.nh3_mode;
    sp.use_hs = 0;
    sp.use_sjs = 0;
    sp.blendW = 0.0;
    if (mode == NH3_HS) {
      sp.use_hs = 1;
    } else if (mode == NH3_SJS) {
      sp.use_sjs = 1;
      sp.blendW = 1.0;
    } else if (mode == NH3_HS_SJS) {
      if (P < 400.0) {
        sp.use_hs = 1;
      } else if (P > 2000.0) {
        sp.use_sjs = 1;
        sp.blendW = 1.0;
      } else {
        sp.use_hs = 1;
        sp.use_sjs = 1;
        sp.blendW = (P - 400.0) / (2000.0 - 400.0);
      }
    }
  }
  __syncwarp();
  // ---- per-family scalar tasks, one lane each (float64)
  if (lane < 2) {  // NH3 inversion, coefficient set = lane
    const double* c = INV_SET[lane];
    LayerFam& F = sp.fam[FAM_NH3_INV];
    const double t295 = 295.0 / T;
    F.c[lane][0] = (float)(c[0] * Ph2 * pow(Tdiv, c[3]) + c[1] * Phe * pow(Tdiv, c[4]));
    F.c[lane][1] = (float)(c[2] * Pnh3 * pow(t295, c[5]));
    F.c[lane][2] = 0.f;
    F.c[lane][3] = (float)(c[6] * Ph2 * pow(Tdiv, c[9]) + c[7] * Phe * pow(Tdiv, c[10]));
    F.c[lane][4] = (float)(c[8] * Pnh3 * pow(t295, c[11]));
    F.c[lane][5] = 0.f;
    F.c[lane][6] = (float)c[12];
    F.c[lane][7] = 0.f;
    if (lane == 0) {
      F.cE = cE_hs;
      F.fac = hs_pref * (2.0 / CUDART_PI);   // times Con of the set, applied at the end
    }
  } else if (lane == 2) {  // NH3 rotational (nh3_hs.py:232-265)
    LayerFam& F = sp.fam[FAM_NH3_ROT];
    F.c[0][1] = (float)(0.2984 * Ph2 * pow(Tdiv, 0.8730));
    F.c[0][2] = (float)(0.75 * Phe * pow(Tdiv, 2.0 / 3.0));
    F.c[0][3] = (float)(3.1789 * Pnh3 * pow(Tdiv, 1.0));
    F.cE = cE_hs;
    F.fac = 2.4268 * hs_pref * (4.0 / CUDART_PI);
  } else if (lane == 3) {  // NH3 nu2 (nh3_hs.py:269-302); per-line widths 1.4/0.68/9.5
    LayerFam& F = sp.fam[FAM_NH3_V2];
    F.c[0][1] = (float)(Ph2 * pow(Tdiv, 0.73));
    F.c[0][2] = (float)(Phe * pow(Tdiv, 0.5716));
    F.c[0][3] = (float)(Pnh3 * pow(Tdiv, 1.0));
    F.cE = cE_hs;
    F.fac = 1.1206 * hs_pref * (4.0 / CUDART_PI);
  } else if (lane == 4) {  // NH3 sjs (nh3_sjs.py:37-124)
    LayerFam& F = sp.fam[FAM_NH3_SJS];
    const double T0 = 296.0;
    const double rexp = 8.79 * exp(-T / 83.0);
    double GH2a = pow(exp(9.024 - T / 20.3) - 0.9918 + Ph2, rexp);
    // Joiner: {GH2, GHe, GNH3, ZH2, ZHe, ZNH3, D}
    double J[7] = {1.690, 0.750, 0.6, 1.350, 0.300, 0.200, -0.45};
    double S[7];
    if (GH2a < 1e-12) {
      for (int k = 0; k < 7; ++k) S[k] = J[k];
    } else {
      double g = 2.122 * exp(-T / 116.8) / GH2a;
      g = 2.34 * (1.0 - g);
      S[0] = g;
      S[1] = 0.46 + T / 3000.0;
      S[2] = 0.74;
      S[3] = 5.7465 - 7.7644 * g + 9.1931 * g * g - 5.6816 * g * g * g + 1.2307 * g * g * g * g;
      S[4] = 0.28 - T / 1750.0;
      S[5] = 0.50;
      S[6] = -0.45;
    }
    const double tt = pow(T0 / T, 2.0 / 3.0);
    for (int s = 0; s < 2; ++s) {
      const double* c = s == 0 ? J : S;
      sp.sjs[s][0] = tt * (c[0] * Ph2 + c[1] * Phe);   // gamma = [0] + [1]*G0
      sp.sjs[s][1] = tt * (c[2] * Pnh3);
      sp.sjs[s][2] = tt * (c[3] * Ph2 + c[4] * Phe);   // zeta  = [2] + [3]*G0
      sp.sjs[s][3] = tt * (c[5] * Pnh3);
      sp.sjs[s][4] = c[6] * Pnh3;                      // delta
      sp.sjs[s][5] = 0.0;
      sp.sjs[s][6] = 0.0;
      sp.sjs[s][7] = 0.0;
    }
    const double Pscale = 1.0 + P / 1.0E5;
    F.cE = -(1.0 / T - 1.0 / T0) * HCK;
    F.fac = GEISA_COEF * (Pnh3 / T0) * pow(T0 / T, 3.5) * Pscale * GHZ_INVCM * 2.0 / CUDART_PI;
  } else if (lane == 5) {  // H2S (h2s_ddb.py:42-87)
    LayerFam& F = sp.fam[FAM_H2S];
    const double T0 = 296.0;
    const double t7 = pow(T0 / T, 0.7);
    F.c[0][0] = (float)(t7 * (1.960 * Ph2 + 1.200 * Phe));
    F.c[0][1] = (float)(t7 * Ph2s);
    F.c[0][5] = 1.f;                     // zeta = gamma
    F.c[0][7] = (float)(1.28 * Ph2s);    // delta
    F.cE = -(1.0 / T - 1.0 / T0) * HCK;
    F.fac = GEISA_COEF * (Ph2s / T0) * pow(T0 / T, 3.5) * GHZ_INVCM * 2.0 / CUDART_PI;
  } else if (lane == 6) {  // PH3 (ph3_jh.py:64-108)
    LayerFam& F = sp.fam[FAM_PH3];
    const double T0 = 300.0;
    F.c[0][1] = (float)(pow(T0 / T, 2.0 / 3.0) * (3.2930 * Ph2 + 1.6803 * Phe));
    F.c[0][2] = (float)(pow(T0 / T, 1.0) * 4.2157 * Pph3);
    F.cE = -(1.0 / T - 1.0 / T0) * HCK;
    F.fac = GEISA_COEF * (Pph3 / T0) * pow(T0 / T, 3.5) * GHZ_INVCM * 2.0 / CUDART_PI;
  } else if (lane == 7) {  // H2O lines (h2o_bk.py:80-99)
    LayerFam& F = sp.fam[FAM_H2O];
    const double Theta = 300.0 / T;
    const double M_amu = 8.314472 / 0.46151805;
    double density = (M_amu * Ph2o) / (8.314472e-5 * T);
    density = 0.997317 * (density / M_amu) * 6.0221415e23 * (1.0 / 1e6);
    F.c[0][0] = (float)log2(Theta);
    F.c[0][1] = (float)Ph2o;
    F.c[0][2] = (float)Ph2;
    F.c[0][3] = (float)Phe;
    F.cE = 1.0 - Theta;
    F.fac = 4.342945 * 1e-4 * density * pow(Theta, 2.5) / DB_PER_INVCM;
    // continuum (h2o_bk.py:102-121), coefficient of f^2, in cm^-1
    const double Cf_he = (1.0 / 0.001) * (1.0 / 0.001) * 1.03562010226e-10;
    const double Cf_h2 = (1.0 / 0.001) * (1.0 / 0.001) * 5.07722009423e-11;
    const double Cs1 = 3.1e-07 * pow(Theta, 12.0);
    const double th3 = pow(Theta, 3.0);
    const double foreign = Cf_he * Phe * Ph2o * th3 + Cf_h2 * Ph2 * Ph2o * th3;
    const double selfc = Cs1 * ((Ph2o / 0.001) * (Ph2o / 0.001));
    sp.h2o_cont = (4.342945 * foreign + 4.342945 * selfc) / DB_PER_INVCM;
  } else if (lane == 8) {  // H2 CIA (h2_jj_ddb.py:7-38)
    const double th = 273.0 / T;
    double pre;
    if (a.cfg.h2state == 'n') {
      pre = pow(T / 40.0, 2.5);
      if (pre > 1.0) pre = 1.0;
    } else {
      pre = pow(T / 55.0, 2.7);
      if (pre > 1.0) pre = 1.0;
      pre *= pow(T / 120.0, 0.55);
      if (pre > 1.0) pre = 1.0;
    }
    sp.h2_cia = 3.9522E-14 * Ph2 * pre *
                (Ph2 * pow(th, 3.12) + 1.382 * Phe * pow(th, 2.24) + 9.322 * Pch4 * pow(th, 3.34));
  }
  __syncwarp();
  // ---- log-strength offsets (whole warp per family)
  for (int f = 0; f < NFAM; ++f) {
    if (a.tab[f].n == 0) continue;
    double M = scale_pass(a.tab[f], sp.fam[f].cE, lane);
    if (lane == 0) {
      sp.fam[f].M = M;
      sp.fam[f].fac *= exp(M);
    }
  }
  __syncwarp();
  // copy out
  const int words = sizeof(LayerParams) / 4;
  const unsigned* src = reinterpret_cast<const unsigned*>(&sp);
  unsigned* dst = reinterpret_cast<unsigned*>(a.out + L);
  for (int i = lane; i < words; i += 32) dst[i] = src[i];
}

// ------------------------------------------------------------------ alpha

constexpr int CHUNK_MAX = 256;

// Strength of line li in this layer, S' = exp(lnI + cE E - M), split as
// 2^round(t) * 2^(t-round(t)) so the float argument stays small.
__device__ __forceinline__ float line_strength(const LineTable& t, const LayerFam& F, int li) {
  const double a = (t.lnI[li] + F.cE * t.E[li] - F.M) * 1.4426950408889634;
  const double ti = rint(a);
  if (ti < -160.0) return 0.f;
  const float frac = (float)(a - ti);
  return ldexpf(exp2f(frac), (int)ti);
}

struct BrRec {
  float4* r;    // {KH, G4, Na, Nb}
  float* kl;    // KL
};

__device__ __forceinline__ void br_record(const LineTable& t, const float* c, int li, float S,
                                          float4& rec, float& kl) {
  const float w1 = t.w1 ? t.w1[li] : 0.f;
  const float w2 = t.w2 ? t.w2[li] : 0.f;
  const float g = c[0] + c[1] * w1 + c[2] * w2;
  const float z = c[3] + c[4] * w1 + c[5] * g;
  const float d = c[6] * g + c[7];
  const float fo = t.ch[li];
  const float small = fmaf(2.f * fo + d, d, (g - z) * (g + z));   // 2 fo d + d^2 + g^2 - z^2
  float KH, e;
  two_sum(t.c2h[li], small, KH, e);
  kl = e + t.c2l[li];
  rec = make_float4(KH, 4.f * g * g, S * (g - z), S * (g + z) * (KH + kl));
}

template <bool PRECISE>
__device__ __forceinline__ void br_sweep(const float4* __restrict__ rec, const float* __restrict__ kl,
                                         int b, int e, float FH, float FL, KahanAcc& acc) {
  int l = b;
  int cnt = 0;
  for (; l + 1 < e; l += 2) {
    const float4 r1 = rec[l], r2 = rec[l + 1];
    float d1 = FH - r1.x, d2 = FH - r2.x;
    if (PRECISE) {
      d1 += FL - kl[l];
      d2 += FL - kl[l + 1];
    }
    const float den1 = fmaf(d1, d1, r1.y * FH);
    const float den2 = fmaf(d2, d2, r2.y * FH);
    const float n1 = fmaf(r1.z, FH, r1.w);
    const float n2 = fmaf(r2.z, FH, r2.w);
    const float N = fmaf(n1, den2, n2 * den1);
    acc.part = fmaf(N, rcp_approx(den1 * den2), acc.part);
    if (++cnt == 16) {
      acc.flush();
      cnt = 0;
    }
  }
  if (l < e) {
    const float4 r1 = rec[l];
    float d1 = FH - r1.x;
    if (PRECISE) d1 += FL - kl[l];
    const float den1 = fmaf(d1, d1, r1.y * FH);
    acc.part = fmaf(fmaf(r1.z, FH, r1.w), rcp_approx(den1), acc.part);
  }
  acc.flush();
}

// Gross: record {KH, G4, S*g, KL}
template <bool PRECISE>
__device__ __forceinline__ void gross_sweep(const float4* __restrict__ rec, int b, int e, float FH,
                                            float FL, KahanAcc& acc) {
  int l = b;
  int cnt = 0;
  for (; l + 1 < e; l += 2) {
    const float4 r1 = rec[l], r2 = rec[l + 1];
    float d1 = FH - r1.x, d2 = FH - r2.x;
    if (PRECISE) {
      d1 += FL - r1.w;
      d2 += FL - r2.w;
    }
    const float den1 = fmaf(d1, d1, r1.y * FH);
    const float den2 = fmaf(d2, d2, r2.y * FH);
    const float N = fmaf(r1.z, den2, r2.z * den1);
    acc.part = fmaf(N, rcp_approx(den1 * den2), acc.part);
    if (++cnt == 16) {
      acc.flush();
      cnt = 0;
    }
  }
  if (l < e) {
    const float4 r1 = rec[l];
    float d1 = FH - r1.x;
    if (PRECISE) d1 += FL - r1.w;
    acc.part = fmaf(r1.z, rcp_approx(fmaf(d1, d1, r1.y * FH)), acc.part);
  }
  acc.flush();
}

// VVW: record {ch, cl, df^2, S*df}; per line 1/den1 + 1/den2.
template <bool PRECISE>
__device__ __forceinline__ void vvw_sweep(const float4* __restrict__ rec, int b, int e, float fh,
                                          float fl, KahanAcc& acc) {
  int cnt = 0;
  for (int l = b; l < e; ++l) {
    const float4 r = rec[l];
    float dm = fh - r.x;
    if (PRECISE) dm += fl - r.y;
    const float dp = fh + r.x;
    const float den1 = fmaf(dm, dm, r.z);
    const float den2 = fmaf(dp, dp, r.z);
    acc.part = fmaf(r.w * (den1 + den2), rcp_approx(den1 * den2), acc.part);
    if (++cnt == 32) {
      acc.flush();
      cnt = 0;
    }
  }
  acc.flush();
}

__device__ __forceinline__ int2 clamp_range(int2 nr, int c0, int c1) {
  return make_int2(max(c0, min(c1, nr.x)), max(c0, min(c1, nr.y)));
}

__global__ void __launch_bounds__(256) rb_alpha_kernel(AlphaArgs a) {
  const int L = blockIdx.x;
  const int tile = blockIdx.y;
  const int tid = threadIdx.x;
  const int nthr = blockDim.x;
  const int warp = tid >> 5;
  const int j = tile * nthr + tid;
  const bool valid = j < a.nf;
  __shared__ float4 s_rec[2][CHUNK_MAX];
  __shared__ float s_kl[2][CHUNK_MAX];
  __shared__ float s_red[8];
  const LayerParams& lp = a.lp[L];

  const double f = valid ? a.freqs[j] : 1.0;
  const double fhs = valid ? a.freqs_hs[j] : 1.0;
  const double F64 = f * f, Fhs64 = fhs * fhs;
  float FH, FL, FHhs, FLhs, fh, fl;
  split_double(F64, FH, FL);
  split_double(Fhs64, FHhs, FLhs);
  split_double(f, fh, fl);
  const int2* nearw = a.near + ((size_t)tile * a.nwarps_tile + warp) * NFAM;

  KahanAcc acc_inv, acc_rot, acc_v2, acc_sjs, acc_h2o, acc_h2s, acc_ph3;
  acc_inv.init(); acc_rot.init(); acc_v2.init(); acc_sjs.init();
  acc_h2o.init(); acc_h2s.init(); acc_ph3.init();
  float base_h2o = 0.f;

  const bool nh3_on = a.cfg.nh3_mode != NH3_OFF;
  // ---------------- Ben-Reuven families with layer-level coefficients
  const int br_fams[3] = {FAM_NH3_INV, FAM_H2S, FAM_PH3};
  for (int q = 0; q < 3; ++q) {
    const int fam = br_fams[q];
    if (fam == FAM_NH3_INV && !(nh3_on && lp.use_hs)) continue;
    if (fam == FAM_H2S && !a.cfg.use_h2s) continue;
    if (fam == FAM_PH3 && !a.cfg.use_ph3) continue;
    const LineTable& t = a.tab[fam];
    const LayerFam& LF = lp.fam[fam];
    const bool two = fam == FAM_NH3_INV;
    const int set = (two && fhs > 30.0) ? 1 : 0;
    const float fH = (fam == FAM_NH3_INV) ? FHhs : FH;
    const float fL = (fam == FAM_NH3_INV) ? FLhs : FL;
    KahanAcc& acc = fam == FAM_NH3_INV ? acc_inv : (fam == FAM_H2S ? acc_h2s : acc_ph3);
    const int2 nr = nearw[fam];
    for (int c0 = 0; c0 < t.n; c0 += nthr) {
      const int c1 = min(t.n, c0 + nthr);
      const int li = c0 + tid;
      if (li < c1) {
        const float S = line_strength(t, LF, li);
        float4 r;
        float kl;
        br_record(t, LF.c[0], li, S, r, kl);
        s_rec[0][tid] = r;
        s_kl[0][tid] = kl;
        if (two) {
          br_record(t, LF.c[1], li, S, r, kl);
          s_rec[1][tid] = r;
          s_kl[1][tid] = kl;
        }
      }
      __syncthreads();
      const int n = c1 - c0;
      const int2 rr = clamp_range(nr, c0, c1);
      const float4* rec = s_rec[set];
      const float* kl = s_kl[set];
      br_sweep<false>(rec, kl, 0, rr.x - c0, fH, fL, acc);
      br_sweep<true>(rec, kl, rr.x - c0, rr.y - c0, fH, fL, acc);
      br_sweep<false>(rec, kl, rr.y - c0, n, fH, fL, acc);
      __syncthreads();
    }
  }
  // ---------------- Gross families (nh3_hs rotational, nu2)
  if (nh3_on && lp.use_hs) {
    for (int fam = FAM_NH3_ROT; fam <= FAM_NH3_V2; ++fam) {
      const LineTable& t = a.tab[fam];
      const LayerFam& LF = lp.fam[fam];
      KahanAcc& acc = fam == FAM_NH3_ROT ? acc_rot : acc_v2;
      const int2 nr = nearw[fam];
      for (int c0 = 0; c0 < t.n; c0 += nthr) {
        const int c1 = min(t.n, c0 + nthr);
        const int li = c0 + tid;
        if (li < c1) {
          const float S = line_strength(t, LF, li);
          const float g = LF.c[0][1] * t.w1[li] + LF.c[0][2] * t.w2[li] + LF.c[0][3] * t.w3[li];
          s_rec[0][tid] = make_float4(t.c2h[li], 4.f * g * g, S * g, t.c2l[li]);
        }
        __syncthreads();
        const int n = c1 - c0;
        const int2 rr = clamp_range(nr, c0, c1);
        gross_sweep<false>(s_rec[0], 0, rr.x - c0, FHhs, FLhs, acc);
        gross_sweep<true>(s_rec[0], rr.x - c0, rr.y - c0, FHhs, FLhs, acc);
        gross_sweep<false>(s_rec[0], rr.y - c0, n, FHhs, FLhs, acc);
        __syncthreads();
      }
    }
  }
  // ---------------- nh3_sjs (frequency-dependent coefficients, all precise)
  if (nh3_on && lp.use_sjs) {
    const LineTable& t = a.tab[FAM_NH3_SJS];
    const LayerFam& LF = lp.fam[FAM_NH3_SJS];
    // coefficient set for this frequency (nh3_sjs.py:95-111)
    double cc[5];
    const double fLower = 26.0, fHigher = 34.0;
    if (f <= fLower) {
      for (int k = 0; k < 5; ++k) cc[k] = lp.sjs[1][k];
    } else if (f >= fHigher) {
      for (int k = 0; k < 5; ++k) cc[k] = lp.sjs[0][k];
    } else {
      const double flfh = (fLower - fHigher) / (f - fLower);
      for (int k = 0; k < 5; ++k) cc[k] = lp.sjs[1][k] + (lp.sjs[1][k] - lp.sjs[0][k]) / flfh;
    }
    const float A = (float)cc[0], B = (float)cc[1], C = (float)cc[2], D = (float)cc[3];
    const double delta = lp.sjs[0][4];   // D is -0.45 in every set
    for (int c0 = 0; c0 < t.n; c0 += nthr) {
      const int c1 = min(t.n, c0 + nthr);
      const int li = c0 + tid;
      if (li < c1) {
        const float S = line_strength(t, LF, li);
        const float fo = t.ch[li];
        const float dl = (float)delta;
        float KH, e;
        two_sum(t.c2h[li], fmaf(2.f * fo + dl, dl, 0.f), KH, e);
        s_rec[0][tid] = make_float4(KH, e + t.c2l[li], t.w1[li], S);
      }
      __syncthreads();
      const int n = c1 - c0;
      int cnt = 0;
      for (int l = 0; l < n; ++l) {
        const float4 r = s_rec[0][l];
        const float g = fmaf(B, r.z, A);
        const float z = fmaf(D, r.z, C);
        const float gm = g - z, gp = g + z;
        const float g2z2 = gm * gp;
        const float d1 = ((FH - r.x) + (FL - r.y)) - g2z2;
        const float den = fmaf(d1, d1, 4.f * FH * g * g);
        const float num = fmaf(gm, FH, gp * (r.x + g2z2));
        acc_sjs.part = fmaf(r.w * num, rcp_approx(den), acc_sjs.part);
        if (++cnt == 32) {
          acc_sjs.flush();
          cnt = 0;
        }
      }
      acc_sjs.flush();
      __syncthreads();
    }
  }
  // ---------------- H2O (VVW)
  if (a.cfg.use_h2o) {
    const LineTable& t = a.tab[FAM_H2O];
    const LayerFam& LF = lp.fam[FAM_H2O];
    const int2 nr = nearw[FAM_H2O];
    const float l2T = LF.c[0][0];
    for (int c0 = 0; c0 < t.n; c0 += nthr) {
      const int c1 = min(t.n, c0 + nthr);
      const int li = c0 + tid;
      if (li < c1) {
        const float S = line_strength(t, LF, li);
        const float df = LF.c[0][1] * t.w1[li] * exp2f(t.x1[li] * l2T) +
                         LF.c[0][2] * t.w2[li] * exp2f(t.x2[li] * l2T) +
                         LF.c[0][3] * t.w3[li] * exp2f(t.x3[li] * l2T);
        const float df2 = df * df;
        const float Sd = S * df;
        s_rec[0][tid] = make_float4(t.ch[li], t.cl[li], df2, Sd);
        base_h2o += 2.f * Sd / (562500.f + df2);
      }
      __syncthreads();
      const int n = c1 - c0;
      const int2 rr = clamp_range(nr, c0, c1);
      vvw_sweep<false>(s_rec[0], 0, rr.x - c0, fh, fl, acc_h2o);
      vvw_sweep<true>(s_rec[0], rr.x - c0, rr.y - c0, fh, fl, acc_h2o);
      vvw_sweep<false>(s_rec[0], rr.y - c0, n, fh, fl, acc_h2o);
      __syncthreads();
    }
    // block sum of the frequency-independent base term
    float v = base_h2o;
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((tid & 31) == 0) s_red[warp] = v;
    __syncthreads();
    float tot = 0.f;
    for (int w = 0; w < (nthr >> 5); ++w) tot += s_red[w];
    base_h2o = tot;
  }
  if (!valid) return;
  // ---------------- assemble in float64
  const double U = a.cfg.units_db ? DB_PER_INVCM : 1.0;
  double g[NGAS] = {0.0, 0.0, 0.0, 0.0, 0.0};
  if (a.cfg.use_h2) g[GAS_H2] = lp.h2_cia * F64 * U;
  if (a.cfg.use_h2o) {
    const double line = lp.fam[FAM_H2O].fac * F64 * ((double)acc_h2o.value() - (double)base_h2o);
    g[GAS_H2O] = (line + lp.h2o_cont * F64) * U;
  }
  if (a.cfg.use_h2s) g[GAS_H2S] = lp.fam[FAM_H2S].fac * F64 * (double)acc_h2s.value() * U;
  if (a.cfg.use_ph3) g[GAS_PH3] = lp.fam[FAM_PH3].fac * F64 * (double)acc_ph3.value() * U;
  if (nh3_on) {
    double hs = 0.0, sjs = 0.0;
    if (lp.use_hs) {
      const int set = fhs > 30.0 ? 1 : 0;
      hs = Fhs64 * (lp.fam[FAM_NH3_INV].fac * INV_CON[set] * (double)acc_inv.value() +
                    lp.fam[FAM_NH3_ROT].fac * (double)acc_rot.value() +
                    lp.fam[FAM_NH3_V2].fac * (double)acc_v2.value());
      hs *= U;
      if (hs < 0.0) hs = 1.0E-8;           // nh3_hs.py:311-312
    }
    if (lp.use_sjs) sjs = lp.fam[FAM_NH3_SJS].fac * F64 * (double)acc_sjs.value() * U;
    const double W = lp.blendW;
    if (lp.use_hs && lp.use_sjs)
      g[GAS_NH3] = W * sjs + (1.0 - W) * hs;
    else
      g[GAS_NH3] = lp.use_hs ? hs : sjs;
  }
  double tot = 0.0;
  const double* sc = a.scale ? a.scale + (size_t)L * NGAS : nullptr;
  for (int k = 0; k < NGAS; ++k) {
    const double v = sc ? g[k] * sc[k] : g[k];
    if (a.gas64) a.gas64[((size_t)L * a.nf + j) * NGAS + k] = v;
    tot += v;
  }
  a.alpha32[(size_t)L * a.nf + j] = (float)(a.cfg.units_db ? tot / DB_PER_INVCM : tot);
  if (a.layers64) a.layers64[(size_t)j * a.nL + L] = tot;
}

// ------------------------------------------------------------------ launch
cudaError_t launch_prep(const PrepArgs& pa, cudaStream_t st) {
  rb_layer_prep_kernel<<<pa.nL, 32, 0, st>>>(pa);
  return cudaGetLastError();
}

cudaError_t launch_alpha_lines(const AlphaArgs& aa, int block, int ntile, cudaStream_t st) {
  dim3 grid(aa.nL, ntile);
  rb_alpha_kernel<<<grid, block, 0, st>>>(aa);
  return cudaGetLastError();
}

}  // namespace rb
