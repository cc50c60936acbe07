// Absorption coefficient of every (layer, frequency): the per-gas line sums
// of radioBEAR's Jupiter formalisms, restated for sm_103a.
//
//   rb_layer_prep_kernel  one thread per layer: partial pressures, width /
//                         shift / coupling coefficients and strength
//                         prefactors (float32 with float64 only for the
//                         temperature coefficient of the strengths).
//   rb_alpha_kernel       one CTA per (layer, frequency tile), two frequency
//                         slots per thread evaluated with packed f32x2
//                         arithmetic.  Lines are staged in shared-memory
//                         chunks: each thread builds one line's layer-
//                         dependent record (duplicated into both halves of
//                         a 64-bit pair, so the sweep loads operands ready
//                         for f32x2), then every thread sweeps the chunk.
//                         Sums are float32 with compensated (Kahan)
//                         accumulation every 16 lines; the prefactor
//                         (mantissa x 2^exponent), unit conversion, clamp,
//                         blend and scaling are applied per slot at the end.
//
// Numerics (per line l, frequency f, F = f^2):
//   Ben-Reuven  S_l [(g-z) F + (g+z) K_l] / [(F - K_l)^2 + 4 F g^2],
//               K_l = (fo+d)^2 + g^2 - z^2      (nh3_hs.py:216-225, h2s_ddb.py:270-272)
//   Gross       S_l g / [(F - fo^2)^2 + 4 F g^2]          (nh3_hs.py:260-263)
//   VVW         S_l df [1/((f-fo)^2+df^2) + 1/((f+fo)^2+df^2) - 2/(750^2+df^2)]
//                                                         (h2o_bk.py:174-187)
// with the common factor f^2 (and the 1/fo^2 of (f/fo)^2, folded into S_l)
// taken out of the sum.  F - K is a double-float difference for lines whose
// centre lies within [0.75 fmin, 1.3 fmax] of the warp's frequencies (there
// float32 would cancel); elsewhere plain float32 is exact to a few ulp.
// Pairs of lines share one reciprocal: n1/d1 + n2/d2 = (n1 d2 + n2 d1)/(d1 d2).
// Strengths: S'_l = 2^(l2I_l + cE E_l - M2) with the exponent formed as a
// double-float and split into integer and fractional parts before exp2.
#include "rb_args.cuh"
#include <math_constants.h>

namespace rb {

// ------------------------------------------------------------------ f32x2
typedef unsigned long long f2;

__device__ __forceinline__ f2 pk(float a, float b) {
  f2 r;
  asm("mov.b64 %0, {%1,%2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ float lo2(f2 v) {
  float a, b;
  asm("mov.b64 {%0,%1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
  return a;
}
__device__ __forceinline__ float hi2(f2 v) {
  float a, b;
  asm("mov.b64 {%0,%1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
  return b;
}
__device__ __forceinline__ f2 add2(f2 a, f2 b) {
  f2 d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f2 mul2(f2 a, f2 b) {
  f2 d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f2 fma2(f2 a, f2 b, f2 c) {
  f2 d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}
__device__ __forceinline__ f2 rcp2(f2 v) { return pk(rcp_approx(lo2(v)), rcp_approx(hi2(v))); }
__device__ __forceinline__ f2 dup(float a) { return pk(a, a); }

// Kahan-compensated pair of sums; `part` collects a block of terms.
struct Acc2 {
  f2 s, c, part;
  __device__ __forceinline__ void init() { s = c = part = 0ull; }
  __device__ __forceinline__ void flush() {
    const f2 mone = dup(-1.f);
    const f2 y = fma2(c, mone, part);     // part - c
    const f2 t = add2(s, y);
    c = fma2(y, mone, fma2(s, mone, t));  // (t - s) - y
    s = t;
    part = 0ull;
  }
  __device__ __forceinline__ float v0() const { return lo2(s) - lo2(c); }
  __device__ __forceinline__ float v1() const { return hi2(s) - hi2(c); }
};

// ------------------------------------------------------------------ constants
constexpr float GHZ_INVCM = 29.9792458f;
constexpr float TWO_OVER_PI = 0.63661977236758134f;
constexpr float FOUR_OVER_PI = 1.2732395447351627f;
constexpr float DB_PER_INVCM = 434294.5f;
__device__ constexpr float INV_CON[2] = {0.9301f, 0.9862f};
constexpr double LOG2E = 1.4426950408889634;
constexpr float HS_COEF = (float)(1.0E6 * 6.02297E23 / 8.31432E7);   // nh3_hs.py:49-55

// Inversion coefficient sets (nh3_hs.py:139-168): gnu_H2, gnu_He, gnu_NH3,
// GAMMA_H2, GAMMA_He, GAMMA_NH3, zeta_H2, zeta_He, zeta_NH3, Z_H2, Z_He,
// Z_NH3, d
__device__ constexpr float INV_SET[2][13] = {
    {1.640f, 0.75f, 0.852f, 0.7756f, 0.666f, 1.0f, 1.262f, 0.3f, 0.5296f, 0.7964f, 0.667f, 1.554f,
     -0.0498f},
    {1.7465f, 0.9779f, 0.7298f, 0.8202f, 1.0f, 1.0f, 1.2163f, 0.0291f, 0.5152f, 0.8873f, 0.8994f,
     0.66666667f, -0.0627f}};

__device__ __forceinline__ float pw(float lg2x, float e) { return exp2f(e * lg2x); }

// prefactor value v (> 0) -> mantissa, exponent (+ M2)
__device__ __forceinline__ void set_fac(LayerFam& F, float v, float M2) {
  int e = 0;
  F.fm = frexpf(v, &e);
  F.fe = e + (int)M2;
  F.M2 = M2;
}

// strength scale: integer upper bound of l2I + cE*E over the family
__device__ __forceinline__ float scale_bound(const PrepArgs& a, int fam, float cE) {
  if (a.nlines[fam] == 0) return 0.f;
  const float m = a.l2Imax[fam] + fmaxf(cE * a.Emin[fam], cE * a.Emax[fam]);
  return isfinite(m) ? ceilf(m) + 1.f : 0.f;
}

__device__ __forceinline__ void set_cE(LayerFam& F, double cE2) {
  F.cEh = (float)cE2;
  F.cEl = (float)(cE2 - (double)F.cEh);
}

__global__ void __launch_bounds__(64) rb_layer_prep_kernel(PrepArgs a) {
  const int L = blockIdx.x * blockDim.x + threadIdx.x;
  if (L >= a.nL) return;
  const int nL = a.nL;
  const double Pd = a.P[L], Td = a.T[L];
  const float P = (float)Pd, T = (float)Td;
  const double* X = a.X;
  const float Ph2 = (float)(Pd * X[X_H2 * nL + L]), Phe = (float)(Pd * X[X_HE * nL + L]);
  const float Pch4 = (float)(Pd * X[X_CH4 * nL + L]), Pnh3 = (float)(Pd * X[X_NH3 * nL + L]);
  const float Ph2o = (float)(Pd * X[X_H2O * nL + L]), Ph2s = (float)(Pd * X[X_H2S * nL + L]);
  const float Pph3 = (float)(Pd * X[X_PH3 * nL + L]);
  LayerParams o;
  o.P = P;
  o.T = T;
  for (int f = 0; f < NFAM; ++f) {
    o.fam[f].fm = 0.f;
    o.fam[f].fe = 0;
    o.fam[f].cEh = o.fam[f].cEl = 0.f;
    o.fam[f].M2 = 0.f;
    for (int s = 0; s < 2; ++s)
      for (int k = 0; k < 8; ++k) o.fam[f].c[s][k] = 0.f;
  }
  // strength temperature coefficients, log2 units, float64 (the only
  // float64 of the absorption path: 1/T - 1/T0 cancels near T0)
  const double invT = 1.0 / Td;
  const double cE300 = -(invT - 1.0 / 300.0) * (19.858252418E-24 / 1.38E-23) * LOG2E;  // nh3_hs
  const double cE296g = -(invT - 1.0 / 296.0) * 1.438396 * LOG2E;                      // sjs, h2s
  const double cE300g = -(invT - 1.0 / 300.0) * 1.438396 * LOG2E;                      // ph3
  const double cEh2o = (1.0 - 300.0 * invT) * LOG2E;                                   // h2o
  // NH3 formalism choice (nh3_hs_sjs.py:6-26)
  o.use_hs = 0;
  o.use_sjs = 0;
  o.blendW = 0.f;
  const int mode = a.cfg.nh3_mode;
  if (mode == NH3_HS) {
    o.use_hs = 1;
  } else if (mode == NH3_SJS) {
    o.use_sjs = 1;
    o.blendW = 1.f;
  } else if (mode == NH3_HS_SJS) {
    if (Pd < 400.0) {
      o.use_hs = 1;
    } else if (Pd > 2000.0) {
      o.use_sjs = 1;
      o.blendW = 1.f;
    } else {
      o.use_hs = 1;
      o.use_sjs = 1;
      o.blendW = (float)((Pd - 400.0) / (2000.0 - 400.0));
    }
  }
  const float Tdiv = 300.f / T;
  const float lTdiv = log2f(Tdiv);
  const float l295 = log2f(295.f / T);
  const float hs_base = HS_COEF * (Pnh3 / 300.f) * pw(lTdiv, 3.5f) * GHZ_INVCM;
  {  // NH3 inversion (nh3_hs.py:137-229)
    LayerFam& F = o.fam[FAM_NH3_INV];
    for (int s = 0; s < 2; ++s) {
      const float* c = INV_SET[s];
      F.c[s][0] = c[0] * Ph2 * pw(lTdiv, c[3]) + c[1] * Phe * pw(lTdiv, c[4]);
      F.c[s][1] = c[2] * Pnh3 * pw(l295, c[5]);
      F.c[s][3] = c[6] * Ph2 * pw(lTdiv, c[9]) + c[7] * Phe * pw(lTdiv, c[10]);
      F.c[s][4] = c[8] * Pnh3 * pw(l295, c[11]);
      F.c[s][6] = c[12];
    }
    set_cE(F, cE300);
    set_fac(F, hs_base * TWO_OVER_PI, scale_bound(a, FAM_NH3_INV, (float)cE300));
  }
  {  // NH3 rotational (nh3_hs.py:232-265)
    LayerFam& F = o.fam[FAM_NH3_ROT];
    F.c[0][1] = 0.2984f * Ph2 * pw(lTdiv, 0.8730f);
    F.c[0][2] = 0.75f * Phe * pw(lTdiv, 0.66666667f);
    F.c[0][3] = 3.1789f * Pnh3 * Tdiv;
    set_cE(F, cE300);
    set_fac(F, 2.4268f * hs_base * FOUR_OVER_PI, scale_bound(a, FAM_NH3_ROT, (float)cE300));
  }
  {  // NH3 nu2 (nh3_hs.py:269-302); per-line widths 1.4 / 0.68 / 9.5
    LayerFam& F = o.fam[FAM_NH3_V2];
    F.c[0][1] = Ph2 * pw(lTdiv, 0.73f);
    F.c[0][2] = Phe * pw(lTdiv, 0.5716f);
    F.c[0][3] = Pnh3 * Tdiv;
    set_cE(F, cE300);
    set_fac(F, 1.1206f * hs_base * FOUR_OVER_PI, scale_bound(a, FAM_NH3_V2, (float)cE300));
  }
  if (o.use_sjs) {  // NH3 sjs (nh3_sjs.py:37-124)
    LayerFam& F = o.fam[FAM_NH3_SJS];
    const float rexp = 8.79f * expf(-T / 83.0f);
    const float GH2a = powf(expf(9.024f - T / 20.3f) - 0.9918f + Ph2, rexp);
    float J[7] = {1.690f, 0.750f, 0.6f, 1.350f, 0.300f, 0.200f, -0.45f};
    float S[7];
    if (GH2a < 1e-12f) {
      for (int k = 0; k < 7; ++k) S[k] = J[k];
    } else {
      const float g = 2.34f * (1.0f - 2.122f * expf(-T / 116.8f) / GH2a);
      const double gd = g;   // the ZH2 polynomial cancels: evaluate in float64
      S[0] = g;
      S[1] = 0.46f + T / 3000.0f;
      S[2] = 0.74f;
      S[3] = (float)(5.7465 + gd * (-7.7644 + gd * (9.1931 + gd * (-5.6816 + gd * 1.2307))));
      S[4] = 0.28f - T / 1750.0f;
      S[5] = 0.50f;
      S[6] = -0.45f;
    }
    const float tt = pw(log2f(296.f / T), 2.f / 3.f);
    for (int s = 0; s < 2; ++s) {
      const float* c = s == 0 ? J : S;
      o.sjs[s][0] = tt * (c[0] * Ph2 + c[1] * Phe);
      o.sjs[s][1] = tt * (c[2] * Pnh3);
      o.sjs[s][2] = tt * (c[3] * Ph2 + c[4] * Phe);
      o.sjs[s][3] = tt * (c[5] * Pnh3);
      o.sjs[s][4] = c[6] * Pnh3;
    }
    const float Pscale = 1.0f + P / 1.0E5f;
    set_cE(F, cE296g);
    set_fac(F, 7.244E+21f * (Pnh3 / 296.f) * pw(log2f(296.f / T), 3.5f) * Pscale * GHZ_INVCM * TWO_OVER_PI,
            scale_bound(a, FAM_NH3_SJS, (float)cE296g));
  } else {
    for (int s = 0; s < 2; ++s)
      for (int k = 0; k < 5; ++k) o.sjs[s][k] = 0.f;
  }
  {  // H2S (h2s_ddb.py:42-87)
    LayerFam& F = o.fam[FAM_H2S];
    const float l296 = log2f(296.f / T);
    const float t7 = pw(l296, 0.7f);
    F.c[0][0] = t7 * (1.960f * Ph2 + 1.200f * Phe);
    F.c[0][1] = t7 * Ph2s;
    F.c[0][5] = 1.f;                     // zeta = gamma
    F.c[0][7] = 1.28f * Ph2s;            // delta
    set_cE(F, cE296g);
    set_fac(F, 7.244E+21f * (Ph2s / 296.f) * pw(l296, 3.5f) * GHZ_INVCM * TWO_OVER_PI,
            scale_bound(a, FAM_H2S, (float)cE296g));
  }
  {  // PH3 (ph3_jh.py:64-108)
    LayerFam& F = o.fam[FAM_PH3];
    F.c[0][1] = pw(lTdiv, 2.f / 3.f) * (3.2930f * Ph2 + 1.6803f * Phe);
    F.c[0][2] = Tdiv * 4.2157f * Pph3;
    set_cE(F, cE300g);
    set_fac(F, 7.244E+21f * (Pph3 / 300.f) * pw(lTdiv, 3.5f) * GHZ_INVCM * TWO_OVER_PI,
            scale_bound(a, FAM_PH3, (float)cE300g));
  }
  {  // H2O lines (h2o_bk.py:80-99) and continuum (102-121)
    LayerFam& F = o.fam[FAM_H2O];
    const float Theta = Tdiv;
    const float lTh = lTdiv;
    const float density = (Ph2o / (8.314472e-5f * T)) * (0.997317f * 6.0221415e17f);
    F.c[0][0] = lTh;
    F.c[0][1] = Ph2o;
    F.c[0][2] = Ph2;
    F.c[0][3] = Phe;
    set_cE(F, cEh2o);
    set_fac(F, 4.342945e-4f * density * pw(lTh, 2.5f) / DB_PER_INVCM,
            scale_bound(a, FAM_H2O, (float)cEh2o));
    const float Cf_he = 1.0e6f * 1.03562010226e-10f, Cf_h2 = 1.0e6f * 5.07722009423e-11f;
    const float th3 = Theta * Theta * Theta;
    const float foreign = Cf_he * Phe * Ph2o * th3 + Cf_h2 * Ph2 * Ph2o * th3;
    const float selfc = 3.1e-07f * pw(lTh, 12.f) * ((Ph2o * 1000.f) * (Ph2o * 1000.f));
    o.h2o_cont = (4.342945f * foreign + 4.342945f * selfc) / DB_PER_INVCM;
  }
  {  // H2 CIA (h2_jj_ddb.py:7-38)
    const float th = 273.f / T;
    const float lth = log2f(th);
    float pre;
    if (a.cfg.h2state == 'n') {
      pre = fminf(pw(log2f(T / 40.f), 2.5f), 1.f);
    } else {
      pre = fminf(pw(log2f(T / 55.f), 2.7f), 1.f);
      pre = fminf(pre * pw(log2f(T / 120.f), 0.55f), 1.f);
    }
    o.h2_cia = 3.9522E-14f * Ph2 * pre *
               (Ph2 * pw(lth, 3.12f) + 1.382f * Phe * pw(lth, 2.24f) + 9.322f * Pch4 * pw(lth, 3.34f));
  }
  for (int g = 0; g < NGAS; ++g) o.scale[g] = a.scale ? (float)a.scale[(size_t)L * NGAS + g] : 1.f;
  a.out[L] = o;
}

// ------------------------------------------------------------------ records
constexpr int CHUNK = 128;      // lines per shared-memory chunk (= max threads per CTA)

// S' = 2^(l2I + cE E - M2), exponent as a double-float, split before exp2
__device__ __forceinline__ float line_strength(const LineTable& t, const LayerFam& F, int li) {
  const float Eh = t.Eh[li], El = t.El[li];
  const float ph = F.cEh * Eh;
  const float pl = fmaf(F.cEh, Eh, -ph) + fmaf(F.cEh, El, F.cEl * Eh);
  float s, e;
  two_sum(t.l2Ih[li] - F.M2, ph, s, e);
  const float lo = e + pl + t.l2Il[li];
  const float ti = rintf(s);
  const float tf = (s - ti) + lo;
  if (ti < -140.f) return 0.f;
  return ldexpf(exp2f(tf), (int)ti);
}

// Ben-Reuven record: {(-K,-K), (G4,G4)}, {(Na,Na), (Nb,Nb)}, and (-KL,-KL)
__device__ __forceinline__ void br_record(const LineTable& t, const float* c, int li, float S,
                                          ulonglong2* A, ulonglong2* B, f2* KL) {
  const float w1 = t.w1[li];
  const float w2 = t.w2[li];
  const float g = c[0] + c[1] * w1 + c[2] * w2;
  const float z = c[3] + c[4] * w1 + c[5] * g;
  const float d = c[6] * g + c[7];
  const float fo = t.ch[li];
  const float small = fmaf(2.f * fo + d, d, (g - z) * (g + z));   // 2 fo d + d^2 + g^2 - z^2
  float KH, e;
  two_sum(t.c2h[li], small, KH, e);
  const float kl = e + t.c2l[li];
  *A = make_ulonglong2(dup(-KH), dup(4.f * g * g));
  *B = make_ulonglong2(dup(S * (g - z)), dup(S * (g + z) * (KH + kl)));
  *KL = dup(-kl);
}

// ------------------------------------------------------------------ sweeps
template <bool PRECISE>
__device__ __forceinline__ void br_pair(const ulonglong2 a1, const ulonglong2 b1, f2 k1,
                                        const ulonglong2 a2, const ulonglong2 b2, f2 k2, f2 F,
                                        f2 FL, f2& part) {
  f2 d1 = add2(F, a1.x), d2 = add2(F, a2.x);
  if (PRECISE) {
    d1 = add2(d1, add2(FL, k1));
    d2 = add2(d2, add2(FL, k2));
  }
  const f2 den1 = fma2(d1, d1, mul2(a1.y, F));
  const f2 den2 = fma2(d2, d2, mul2(a2.y, F));
  const f2 n1 = fma2(b1.x, F, b1.y);
  const f2 n2 = fma2(b2.x, F, b2.y);
  const f2 N = fma2(n1, den2, mul2(n2, den1));
  part = fma2(N, rcp2(mul2(den1, den2)), part);
}

template <bool PRECISE>
__device__ __forceinline__ void br_sweep(const ulonglong2* __restrict__ A,
                                         const ulonglong2* __restrict__ B,
                                         const f2* __restrict__ KL, int b, int e, f2 F, f2 FL,
                                         Acc2& acc) {
  int l = b;
  for (; l + 16 <= e; l += 16) {
#pragma unroll
    for (int p = 0; p < 16; p += 2)
      br_pair<PRECISE>(A[l + p], B[l + p], PRECISE ? KL[l + p] : 0ull, A[l + p + 1], B[l + p + 1],
                       PRECISE ? KL[l + p + 1] : 0ull, F, FL, acc.part);
    acc.flush();
  }
  for (; l + 1 < e; l += 2)
    br_pair<PRECISE>(A[l], B[l], PRECISE ? KL[l] : 0ull, A[l + 1], B[l + 1],
                     PRECISE ? KL[l + 1] : 0ull, F, FL, acc.part);
  if (l < e) {
    const ulonglong2 a1 = A[l], b1 = B[l];
    f2 d1 = add2(F, a1.x);
    if (PRECISE) d1 = add2(d1, add2(FL, KL[l]));
    const f2 den1 = fma2(d1, d1, mul2(a1.y, F));
    acc.part = fma2(fma2(b1.x, F, b1.y), rcp2(den1), acc.part);
  }
  acc.flush();
}

// Gross record: {(-K,-K), (G4,G4)}, {(Sg,Sg), (-KL,-KL)}
template <bool PRECISE>
__device__ __forceinline__ void gross_pair(const ulonglong2 a1, const ulonglong2 b1,
                                           const ulonglong2 a2, const ulonglong2 b2, f2 F, f2 FL,
                                           f2& part) {
  f2 d1 = add2(F, a1.x), d2 = add2(F, a2.x);
  if (PRECISE) {
    d1 = add2(d1, add2(FL, b1.y));
    d2 = add2(d2, add2(FL, b2.y));
  }
  const f2 den1 = fma2(d1, d1, mul2(a1.y, F));
  const f2 den2 = fma2(d2, d2, mul2(a2.y, F));
  const f2 N = fma2(b1.x, den2, mul2(b2.x, den1));
  part = fma2(N, rcp2(mul2(den1, den2)), part);
}

template <bool PRECISE>
__device__ __forceinline__ void gross_sweep(const ulonglong2* __restrict__ A,
                                            const ulonglong2* __restrict__ B, int b, int e, f2 F,
                                            f2 FL, Acc2& acc) {
  int l = b;
  for (; l + 16 <= e; l += 16) {
#pragma unroll
    for (int p = 0; p < 16; p += 2)
      gross_pair<PRECISE>(A[l + p], B[l + p], A[l + p + 1], B[l + p + 1], F, FL, acc.part);
    acc.flush();
  }
  for (; l + 1 < e; l += 2) gross_pair<PRECISE>(A[l], B[l], A[l + 1], B[l + 1], F, FL, acc.part);
  if (l < e) {
    const ulonglong2 a1 = A[l], b1 = B[l];
    f2 d1 = add2(F, a1.x);
    if (PRECISE) d1 = add2(d1, add2(FL, b1.y));
    acc.part = fma2(b1.x, rcp2(fma2(d1, d1, mul2(a1.y, F))), acc.part);
  }
  acc.flush();
}

// VVW record: {(-ch,-ch), (ch,ch)}, {(df^2,df^2), (S df, S df)}, (-cl,-cl)
__device__ __forceinline__ f2 vvw_term(const ulonglong2 a, const ulonglong2 b, f2 fq, f2 dn,
                                       f2& den) {
  const f2 den1 = fma2(dn, dn, b.x);
  const f2 dp = add2(fq, a.y);
  const f2 den2 = fma2(dp, dp, b.x);
  den = mul2(den1, den2);
  return mul2(b.y, add2(den1, den2));
}

template <bool PRECISE>
__device__ __forceinline__ void vvw_pair(const ulonglong2 a1, const ulonglong2 b1, f2 c1,
                                         const ulonglong2 a2, const ulonglong2 b2, f2 c2, f2 fq,
                                         f2 fl, f2& part) {
  f2 dm1 = add2(fq, a1.x), dm2 = add2(fq, a2.x);
  if (PRECISE) {
    dm1 = add2(dm1, add2(fl, c1));
    dm2 = add2(dm2, add2(fl, c2));
  }
  f2 D1, D2;
  const f2 n1 = vvw_term(a1, b1, fq, dm1, D1);
  const f2 n2 = vvw_term(a2, b2, fq, dm2, D2);
  part = fma2(fma2(n1, D2, mul2(n2, D1)), rcp2(mul2(D1, D2)), part);
}

template <bool PRECISE>
__device__ __forceinline__ void vvw_sweep(const ulonglong2* __restrict__ A,
                                          const ulonglong2* __restrict__ B,
                                          const f2* __restrict__ CL, int b, int e, f2 fq, f2 fl,
                                          Acc2& acc) {
  int l = b;
  for (; l + 16 <= e; l += 16) {
#pragma unroll
    for (int p = 0; p < 16; p += 2)
      vvw_pair<PRECISE>(A[l + p], B[l + p], PRECISE ? CL[l + p] : 0ull, A[l + p + 1], B[l + p + 1],
                        PRECISE ? CL[l + p + 1] : 0ull, fq, fl, acc.part);
    acc.flush();
  }
  for (; l + 1 < e; l += 2)
    vvw_pair<PRECISE>(A[l], B[l], PRECISE ? CL[l] : 0ull, A[l + 1], B[l + 1],
                      PRECISE ? CL[l + 1] : 0ull, fq, fl, acc.part);
  if (l < e) {
    const ulonglong2 a1 = A[l], b1 = B[l];
    f2 dm1 = add2(fq, a1.x);
    if (PRECISE) dm1 = add2(dm1, add2(fl, CL[l]));
    f2 D1;
    const f2 n1 = vvw_term(a1, b1, fq, dm1, D1);
    acc.part = fma2(n1, rcp2(D1), acc.part);
  }
  acc.flush();
}

__device__ __forceinline__ int2 clamp_range(int2 nr, int c0, int c1) {
  return make_int2(max(c0, min(c1, nr.x)), max(c0, min(c1, nr.y)));
}

// Assemble one slot: per-gas absorption (T = float or double), scaled.
template <typename T>
__device__ __forceinline__ void assemble(const LayerParams& lp, const AlphaConfig& cfg, T F, T Fhs,
                                         int set, float inv, float rot, float v2, float sjs,
                                         float h2o, float base_h2o, float h2s, float ph3, T* g) {
  const T U = cfg.units_db ? (T)434294.5 : (T)1;
  for (int k = 0; k < NGAS; ++k) g[k] = (T)0;
  auto sc = [](float m, int e, float v) -> T {
    if (sizeof(T) == 4) return (T)ldexpf(m * v, e);
    return (T)ldexp((double)m * (double)v, e);
  };
  if (cfg.use_h2) g[GAS_H2] = (T)lp.h2_cia * F * U;
  if (cfg.use_h2o) {
    const LayerFam& L = lp.fam[FAM_H2O];
    g[GAS_H2O] = (sc(L.fm, L.fe, h2o - base_h2o) * F + (T)lp.h2o_cont * F) * U;
  }
  if (cfg.use_h2s) g[GAS_H2S] = sc(lp.fam[FAM_H2S].fm, lp.fam[FAM_H2S].fe, h2s) * F * U;
  if (cfg.use_ph3) g[GAS_PH3] = sc(lp.fam[FAM_PH3].fm, lp.fam[FAM_PH3].fe, ph3) * F * U;
  if (cfg.nh3_mode != NH3_OFF) {
    T hs = (T)0, sj = (T)0;
    if (lp.use_hs) {
      hs = Fhs * (sc(lp.fam[FAM_NH3_INV].fm * INV_CON[set], lp.fam[FAM_NH3_INV].fe, inv) +
                  sc(lp.fam[FAM_NH3_ROT].fm, lp.fam[FAM_NH3_ROT].fe, rot) +
                  sc(lp.fam[FAM_NH3_V2].fm, lp.fam[FAM_NH3_V2].fe, v2));
      hs *= U;
      if (hs < (T)0) hs = (T)1.0E-8;           // nh3_hs.py:311-312
    }
    if (lp.use_sjs) sj = sc(lp.fam[FAM_NH3_SJS].fm, lp.fam[FAM_NH3_SJS].fe, sjs) * F * U;
    const T W = (T)lp.blendW;
    if (lp.use_hs && lp.use_sjs)
      g[GAS_NH3] = W * sj + ((T)1 - W) * hs;
    else
      g[GAS_NH3] = lp.use_hs ? hs : sj;
  }
  for (int k = 0; k < NGAS; ++k) g[k] *= (T)lp.scale[k];
}

// ------------------------------------------------------------------ kernel
__global__ void __launch_bounds__(CHUNK) rb_alpha_kernel(AlphaArgs a) {
  const int L = a.nL - 1 - blockIdx.x;           // deep (blend) layers first
  const int tid = threadIdx.x;
  const int nthr = blockDim.x;
  const int warp = tid >> 5;
  const int s0 = blockIdx.y * (2 * nthr) + 2 * tid;   // this thread's slot pair
  __shared__ __align__(16) ulonglong2 sA[2][CHUNK];
  __shared__ __align__(16) ulonglong2 sB[2][CHUNK];
  __shared__ __align__(16) f2 sK[2][CHUNK];
  __shared__ float s_red[CHUNK / 32];
  const LayerParams& lp = a.lp[L];
  const SlotPlan& P = a.sp;
  const bool in0 = s0 < a.nslot;
  const float2 one = make_float2(1.f, 0.f);
  const float2 F0 = in0 ? P.F[s0] : one, F1 = in0 ? P.F[s0 + 1] : one;
  const float2 H0 = in0 ? P.Fhs[s0] : one, H1 = in0 ? P.Fhs[s0 + 1] : one;
  const float2 q0 = in0 ? P.f[s0] : one, q1 = in0 ? P.f[s0 + 1] : one;
  const int set = in0 ? P.set[s0] : 0;           // both slots share the set
  const f2 F = pk(F0.x, F1.x), FL = pk(F0.y, F1.y);
  const f2 Fh = pk(H0.x, H1.x), FLh = pk(H0.y, H1.y);
  const f2 fq = pk(q0.x, q1.x), fl = pk(q0.y, q1.y);
  const int wglobal = blockIdx.y * (nthr >> 5) + warp;
  const int2* nearw = a.near + (size_t)wglobal * NFAM;
  const bool nh3_on = a.cfg.nh3_mode != NH3_OFF;

  Acc2 acc;
  float r_inv[2] = {0.f, 0.f}, r_rot[2] = {0.f, 0.f}, r_v2[2] = {0.f, 0.f}, r_sjs[2] = {0.f, 0.f};
  float r_h2o[2] = {0.f, 0.f}, r_h2s[2] = {0.f, 0.f}, r_ph3[2] = {0.f, 0.f};
  float base_h2o = 0.f;

  // ---------------- Ben-Reuven families with layer-level coefficients
  for (int q = 0; q < 3; ++q) {
    const int fam = q == 0 ? FAM_NH3_INV : (q == 1 ? FAM_H2S : FAM_PH3);
    if (fam == FAM_NH3_INV && !(nh3_on && lp.use_hs)) continue;
    if (fam == FAM_H2S && !a.cfg.use_h2s) continue;
    if (fam == FAM_PH3 && !a.cfg.use_ph3) continue;
    const LineTable& t = a.tab[fam];
    if (t.n == 0) continue;
    const LayerFam& LF = lp.fam[fam];
    const bool two = fam == FAM_NH3_INV;
    const int st = two ? set : 0;
    const f2 Fx = two ? Fh : F, FLx = two ? FLh : FL;
    const int2 nr = nearw[fam];
    acc.init();
    for (int c0 = 0; c0 < t.n; c0 += nthr) {
      const int c1 = min(t.n, c0 + nthr);
      const int li = c0 + tid;
      if (li < c1) {
        const float S = line_strength(t, LF, li);
        br_record(t, LF.c[0], li, S, &sA[0][tid], &sB[0][tid], &sK[0][tid]);
        if (two) br_record(t, LF.c[1], li, S, &sA[1][tid], &sB[1][tid], &sK[1][tid]);
      }
      __syncthreads();
      const int2 rr = clamp_range(nr, c0, c1);
      br_sweep<false>(sA[st], sB[st], sK[st], 0, rr.x - c0, Fx, FLx, acc);
      br_sweep<true>(sA[st], sB[st], sK[st], rr.x - c0, rr.y - c0, Fx, FLx, acc);
      br_sweep<false>(sA[st], sB[st], sK[st], rr.y - c0, c1 - c0, Fx, FLx, acc);
      __syncthreads();
    }
    float* r = fam == FAM_NH3_INV ? r_inv : (fam == FAM_H2S ? r_h2s : r_ph3);
    r[0] = acc.v0();
    r[1] = acc.v1();
  }
  // ---------------- Gross families (nh3_hs rotational, nu2)
  if (nh3_on && lp.use_hs) {
    for (int fam = FAM_NH3_ROT; fam <= FAM_NH3_V2; ++fam) {
      const LineTable& t = a.tab[fam];
      if (t.n == 0) continue;
      const LayerFam& LF = lp.fam[fam];
      const int2 nr = nearw[fam];
      acc.init();
      for (int c0 = 0; c0 < t.n; c0 += nthr) {
        const int c1 = min(t.n, c0 + nthr);
        const int li = c0 + tid;
        if (li < c1) {
          const float S = line_strength(t, LF, li);
          const float g = LF.c[0][1] * t.w1[li] + LF.c[0][2] * t.w2[li] + LF.c[0][3] * t.w3[li];
          sA[0][tid] = make_ulonglong2(dup(-t.c2h[li]), dup(4.f * g * g));
          sB[0][tid] = make_ulonglong2(dup(S * g), dup(-t.c2l[li]));
        }
        __syncthreads();
        const int2 rr = clamp_range(nr, c0, c1);
        gross_sweep<false>(sA[0], sB[0], 0, rr.x - c0, Fh, FLh, acc);
        gross_sweep<true>(sA[0], sB[0], rr.x - c0, rr.y - c0, Fh, FLh, acc);
        gross_sweep<false>(sA[0], sB[0], rr.y - c0, c1 - c0, Fh, FLh, acc);
        __syncthreads();
      }
      float* r = fam == FAM_NH3_ROT ? r_rot : r_v2;
      r[0] = acc.v0();
      r[1] = acc.v1();
    }
  }
  // ---------------- nh3_sjs (frequency-dependent coefficients, all precise)
  if (nh3_on && lp.use_sjs && a.tab[FAM_NH3_SJS].n > 0) {
    const LineTable& t = a.tab[FAM_NH3_SJS];
    const LayerFam& LF = lp.fam[FAM_NH3_SJS];
    // coefficient set per slot (nh3_sjs.py:95-111): Spilker + (Joiner - Spilker) wJ
    const float w0 = in0 ? P.wJ[s0] : 0.f, w1 = in0 ? P.wJ[s0 + 1] : 0.f;
    float cf[2][4];
    for (int k = 0; k < 4; ++k) {
      cf[0][k] = fmaf(lp.sjs[0][k] - lp.sjs[1][k], w0, lp.sjs[1][k]);
      cf[1][k] = fmaf(lp.sjs[0][k] - lp.sjs[1][k], w1, lp.sjs[1][k]);
    }
    const f2 A2 = pk(cf[0][0], cf[1][0]), B2 = pk(cf[0][1], cf[1][1]);
    const f2 C2 = pk(cf[0][2], cf[1][2]), D2 = pk(cf[0][3], cf[1][3]);
    const f2 mone = dup(-1.f), four = dup(4.f);
    const float dl = lp.sjs[0][4];   // D is -0.45 in every set
    acc.init();
    for (int c0 = 0; c0 < t.n; c0 += nthr) {
      const int c1 = min(t.n, c0 + nthr);
      const int li = c0 + tid;
      if (li < c1) {
        const float S = line_strength(t, LF, li);
        const float fo = t.ch[li];
        float KH, e;
        two_sum(t.c2h[li], (2.f * fo + dl) * dl, KH, e);
        sA[0][tid] = make_ulonglong2(dup(KH), dup(e + t.c2l[li]));
        sB[0][tid] = make_ulonglong2(dup(t.w1[li]), dup(S));
      }
      __syncthreads();
      const int n = c1 - c0;
      int cnt = 0;
      for (int l = 0; l < n; ++l) {
        const ulonglong2 ra = sA[0][l], rb = sB[0][l];
        const f2 g = fma2(B2, rb.x, A2);
        const f2 z = fma2(D2, rb.x, C2);
        const f2 gm = fma2(z, mone, g);
        const f2 gp = add2(g, z);
        const f2 g2z2 = mul2(gm, gp);
        const f2 d1 = fma2(g2z2, mone, add2(fma2(ra.x, mone, F), fma2(ra.y, mone, FL)));
        const f2 den = fma2(d1, d1, mul2(mul2(four, F), mul2(g, g)));
        const f2 num = fma2(gm, F, mul2(gp, add2(ra.x, g2z2)));
        acc.part = fma2(mul2(rb.y, num), rcp2(den), acc.part);
        if (++cnt == 16) {
          acc.flush();
          cnt = 0;
        }
      }
      acc.flush();
      __syncthreads();
    }
    r_sjs[0] = acc.v0();
    r_sjs[1] = acc.v1();
  }
  // ---------------- H2O (VVW)
  if (a.cfg.use_h2o && a.tab[FAM_H2O].n > 0) {
    const LineTable& t = a.tab[FAM_H2O];
    const LayerFam& LF = lp.fam[FAM_H2O];
    const int2 nr = nearw[FAM_H2O];
    const float l2T = LF.c[0][0];
    acc.init();
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
        sA[0][tid] = make_ulonglong2(dup(-t.ch[li]), dup(t.ch[li]));
        sB[0][tid] = make_ulonglong2(dup(df2), dup(Sd));
        sK[0][tid] = dup(-t.cl[li]);
        base_h2o += 2.f * Sd / (562500.f + df2);
      }
      __syncthreads();
      const int2 rr = clamp_range(nr, c0, c1);
      vvw_sweep<false>(sA[0], sB[0], sK[0], 0, rr.x - c0, fq, fl, acc);
      vvw_sweep<true>(sA[0], sB[0], sK[0], rr.x - c0, rr.y - c0, fq, fl, acc);
      vvw_sweep<false>(sA[0], sB[0], sK[0], rr.y - c0, c1 - c0, fq, fl, acc);
      __syncthreads();
    }
    r_h2o[0] = acc.v0();
    r_h2o[1] = acc.v1();
    // block sum of the frequency-independent base term
    float v = base_h2o;
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((tid & 31) == 0) s_red[warp] = v;
    __syncthreads();
    float tot = 0.f;
    for (int w = 0; w < (nthr >> 5); ++w) tot += s_red[w];
    base_h2o = tot;
  }
  if (!in0) return;
  // ---------------- assemble both slots
  const bool out64 = a.layers64 || a.gas64;
  for (int h = 0; h < 2; ++h) {
    const int j = P.j[s0 + h];
    if (j < 0) continue;
    const float2 Fs = h ? F1 : F0;
    const float2 Hs = h ? H1 : H0;
    float g32[NGAS];
    assemble<float>(lp, a.cfg, Fs.x + Fs.y, Hs.x + Hs.y, set, r_inv[h], r_rot[h], r_v2[h],
                    r_sjs[h], r_h2o[h], base_h2o, r_h2s[h], r_ph3[h], g32);
    float tot = 0.f;
    for (int k = 0; k < NGAS; ++k) tot += g32[k];
    a.alpha32[(size_t)L * a.nf + j] = a.cfg.units_db ? tot / DB_PER_INVCM : tot;
    if (out64) {
      const double f = a.freqs[j], fh = a.freqs_hs[j];
      double g64[NGAS];
      assemble<double>(lp, a.cfg, f * f, fh * fh, set, r_inv[h], r_rot[h], r_v2[h], r_sjs[h],
                       r_h2o[h], base_h2o, r_h2s[h], r_ph3[h], g64);
      double t64 = 0.0;
      for (int k = 0; k < NGAS; ++k) {
        if (a.gas64) a.gas64[((size_t)L * a.nf + j) * NGAS + k] = g64[k];
        t64 += g64[k];
      }
      if (a.layers64) a.layers64[(size_t)j * a.nL + L] = t64;
    }
  }
}

// ------------------------------------------------------------------ launch
cudaError_t launch_prep(const PrepArgs& pa, cudaStream_t st) {
  rb_layer_prep_kernel<<<(pa.nL + 63) / 64, 64, 0, st>>>(pa);
  return cudaGetLastError();
}

cudaError_t launch_alpha_lines(const AlphaArgs& aa, int block, int ntile, cudaStream_t st) {
  dim3 grid(aa.nL, ntile);
  rb_alpha_kernel<<<grid, block, 0, st>>>(aa);
  return cudaGetLastError();
}

}  // namespace rb
