// Absorption coefficient of every (layer, frequency): the per-gas line sums
// of radioBEAR's Jupiter formalisms, restated for sm_103a.
//
//   rb_layer_prep_kernel     eight threads per layer: partial pressures,
//                            width / shift / coupling coefficients and
//                            strength prefactors (float32 with float64 only
//                            for the temperature coefficient of the
//                            strengths).
//   rb_alpha_lines_kernel<M> persistent line sums.  Work items are (line
//                            range of one family, layer, frequency tile),
//                            taken from a global counter heaviest family
//                            first.  A CTA stages the layer-dependent
//                            records of 128 lines at a time in shared memory
//                            (double-buffered, one barrier per chunk), lines
//                            packed in pairs as f32x2; each thread sweeps
//                            them for M frequency slots ("chains") with
//                            packed f32x2 arithmetic, two line pairs sharing
//                            one reciprocal, Kahan-compensated every 64
//                            lines.  One float per (item, slot) goes to a
//                            scratch table.
//   rb_alpha_assemble_kernel one thread per (layer, slot): family sums,
//                            prefactors (mantissa x 2^exponent), units,
//                            clamp, blend and scaling; float32 total for the
//                            brightness scan, optional float64 outputs.
//
// Numerics (per line l, frequency f, F = f^2):
//   Ben-Reuven  S_l [(g-z) F + (g+z) K_l] / [(F - K_l)^2 + 4 F g^2],
//               K_l = (fo+d)^2 + g^2 - z^2      (nh3_hs.py:216-225, h2s_ddb.py:77-78)
//   Gross       S_l g / [(F - fo^2)^2 + 4 F g^2]          (nh3_hs.py:260-263)
//   VVW         S_l df [1/((f-fo)^2+df^2) + 1/((f+fo)^2+df^2) - 2/(750^2+df^2)]
//                                                         (h2o_bk.py:174-187)
// with the common factor f^2 (and the 1/fo^2 of (f/fo)^2, folded into S_l)
// taken out of the sum.  For lines whose centre lies within [0.75 fmin,
// 1.3 fmax] of a chain's 32 frequencies the denominator is formed from the
// double-float difference F - K (float32 would cancel there); elsewhere it is
// expanded as F (F + G4 - 2K) + K^2 (VVW: den1 den2 = F (F + 2(df^2 - fo^2))
// + (fo^2 + df^2)^2), whose rounding error is at most ~18 ulp outside that
// window, in two operations instead of five.
// Strengths: S'_l = 2^(l2I_l + cE E_l - M2) with the exponent formed as a
// double-float and split into integer and fractional parts before exp2.
#include "rb_args.cuh"
#include "rb_f32x2.cuh"
#include "rb_assemble.cuh"
#include <math_constants.h>

#include <algorithm>

namespace rb {

// Kahan-compensated pair of sums; `part` collects a block of terms.
// The running block sum is kept as two scalars (p0, p1) so the reciprocal
// and the final multiply-add of each term need no repacking.
struct Acc2 {
  f2 s, c;
  float p0, p1;
  __device__ __forceinline__ void init() {
    s = c = 0ull;
    p0 = p1 = 0.f;
  }
  __device__ __forceinline__ void flush() {
    const f2 mone = dup(-1.f);
    const f2 y = fma2(c, mone, pk(p0, p1));   // part - c
    const f2 t = add2(s, y);
    c = fma2(y, mone, fma2(s, mone, t));     // (t - s) - y
    s = t;
    p0 = p1 = 0.f;
  }
  // p += N / D, both halves
  __device__ __forceinline__ void add_div(f2 N, f2 D) {
    p0 = fmaf(lo2(N), rcp_approx(lo2(D)), p0);
    p1 = fmaf(hi2(N), rcp_approx(hi2(D)), p1);
  }
  __device__ __forceinline__ float value() const { return (lo2(s) - lo2(c)) + (hi2(s) - hi2(c)); }
};

// ------------------------------------------------------------------ constants
constexpr float GHZ_INVCM = 29.9792458f;
constexpr float TWO_OVER_PI = 0.63661977236758134f;
constexpr float FOUR_OVER_PI = 1.2732395447351627f;
constexpr float DB_PER_INVCM = 434294.5f;
constexpr double LOG2E = 1.4426950408889634;
constexpr float HS_COEF = (float)(1.0E6 * 6.02297E23 / 8.31432E7);   // nh3_hs.py:49-55

// Inversion coefficient tables [inv_table][set]: gnu_H2, gnu_He, gnu_NH3,
// GAMMA_H2, GAMMA_He, GAMMA_NH3, zeta_H2, zeta_He, zeta_NH3, Z_H2, Z_He,
// Z_NH3, d; set 0 for f <= 30 GHz, set 1 above.  Table 0 nh3_hs
// (nh3_hs.py:139-168), table 1 nh3_dbs (nh3_dbs.py:133-162: its own set 0,
// set 1 equal to nh3_hs's).  Each set's Con is INV_CON (rb_assemble.cuh).
__device__ constexpr float INV_SET[2][2][13] = {
    {{1.640f, 0.75f, 0.852f, 0.7756f, 0.666f, 1.0f, 1.262f, 0.3f, 0.5296f, 0.7964f, 0.667f, 1.554f,
      -0.0498f},
     {1.7465f, 0.9779f, 0.7298f, 0.8202f, 1.0f, 1.0f, 1.2163f, 0.0291f, 0.5152f, 0.8873f, 0.8994f,
      0.66666667f, -0.0627f}},
    {{1.6937f, 0.6997f, 0.7523f, 0.8085f, 1.0f, 1.0f, 1.3263f, 0.1607f, 0.6162f, 0.8199f, 0.0f,
      1.3832f, -0.0139f},
     {1.7465f, 0.9779f, 0.7298f, 0.8202f, 1.0f, 1.0f, 1.2163f, 0.0291f, 0.5152f, 0.8873f, 0.8994f,
      0.66666667f, -0.0627f}}};

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

__device__ __forceinline__ void zero_fam(LayerFam& F) {
  F.fm = 0.f;
  F.fe = 0;
  F.cEh = F.cEl = 0.f;
  F.M2 = 0.f;
  for (int s = 0; s < 2; ++s)
    for (int k = 0; k < 8; ++k) F.c[s][k] = 0.f;
  F.wide = 0;
}

// Ben-Reuven width floor (gamma >= c[s][0], the line-independent part) at
// least 0.32 of the largest shifted centre in every coefficient set.
__device__ __forceinline__ int wide_br(const LayerFam& F, int nsets, float cmax) {
  int w = cmax > 0.f;
  for (int s = 0; s < nsets; ++s) w &= F.c[s][0] >= 0.32f * (cmax + fabsf(F.c[s][7]));
  return w;
}

// Eight threads per layer, one per part of the layer's parameters:
//   0 shared scalars (P, T, NH3 formalism choice, scales, H2 CIA),
//   1 NH3 inversion, 2 rotational, 3 nu2, 4 nh3_sjs, 5 H2S, 6 PH3, 7 H2O.
constexpr int PREP_PARTS = 8;

__global__ void __launch_bounds__(256) rb_layer_prep_kernel(PrepArgs a) {
  const int gid = blockIdx.x * blockDim.x + threadIdx.x;
  const int L = gid / PREP_PARTS, part = gid % PREP_PARTS;
  if (gid == 0 && a.counter) *a.counter = 0;
  if (L >= a.nL) return;
  const int nL = a.nL;
  const double Pd = a.P[L], Td = a.T[L];
  const float P = (float)Pd, T = (float)Td;
  const double* X = a.X;
  // partial pressures in float32 (they are float32 from here on; float64
  // products cost ~64 cycles of GB300's FP64 pipe per warp instruction)
  const float Ph2 = P * (float)X[X_H2 * nL + L], Phe = P * (float)X[X_HE * nL + L];
  const float Pch4 = P * (float)X[X_CH4 * nL + L], Pnh3 = P * (float)X[X_NH3 * nL + L];
  const float Ph2o = P * (float)X[X_H2O * nL + L], Ph2s = P * (float)X[X_H2S * nL + L];
  const float Pph3 = P * (float)X[X_PH3 * nL + L];
  LayerParams& o = a.out[L];
  // strength temperature coefficients, log2 units, float64 (the only
  // float64 of the absorption path: 1/T - 1/T0 cancels near T0)
  // (a float reciprocal refined by one float64 Newton step, ~1e-14 relative,
  // instead of a float64 division)
  const double r0 = (double)__frcp_rn((float)Td);
  const double invT = fma(r0, fma(-Td, r0, 1.0), r0);
  // NH3 formalism choice (nh3_hs_sjs.py:6-26)
  int use_hs = 0, use_sjs = 0;
  float blendW = 0.f;
  const int mode = a.cfg.nh3_mode;
  if (mode == NH3_HS) {
    use_hs = 1;
  } else if (mode == NH3_SJS) {
    use_sjs = 1;
    blendW = 1.f;
  } else if (mode == NH3_HS_SJS) {
    if (Pd < 400.0) {
      use_hs = 1;
    } else if (Pd > 2000.0) {
      use_sjs = 1;
      blendW = 1.f;
    } else {
      use_hs = 1;
      use_sjs = 1;
      blendW = (float)(Pd - 400.0) * (1.f / (2000.f - 400.f));
    }
  }
  const float Tdiv = 300.f / T;
  const float lTdiv = log2f(Tdiv);
  const float l295 = log2f(295.f / T);
  const float hs_base = HS_COEF * (Pnh3 / 300.f) * pw(lTdiv, 3.5f) * GHZ_INVCM;
  const double cE300 = -(invT - 1.0 / 300.0) * (19.858252418E-24 / 1.38E-23) * LOG2E;  // nh3_hs
  LayerFam F;
  zero_fam(F);
  switch (part) {
    case 0: {
      o.P = P;
      o.T = T;
      o.use_hs = use_hs;
      o.use_sjs = use_sjs;
      o.blendW = blendW;
      for (int g = 0; g < NGAS; ++g) o.scale[g] = a.scale ? (float)a.scale[(size_t)L * NGAS + g] : 1.f;
      // H2 CIA (h2_jj_ddb.py:7-38)
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
      return;
    }
    case 1: {  // NH3 inversion (nh3_hs.py:137-229, nh3_dbs.py:131-213)
      for (int s = 0; s < 2; ++s) {
        const float* c = INV_SET[a.cfg.inv_table][s];
        F.c[s][0] = c[0] * Ph2 * pw(lTdiv, c[3]) + c[1] * Phe * pw(lTdiv, c[4]);
        F.c[s][1] = c[2] * Pnh3 * pw(l295, c[5]);
        F.c[s][3] = c[6] * Ph2 * pw(lTdiv, c[9]) + c[7] * Phe * pw(lTdiv, c[10]);
        F.c[s][4] = c[8] * Pnh3 * pw(l295, c[11]);
        F.c[s][6] = c[12];
      }
      set_cE(F, cE300);
      set_fac(F, hs_base * TWO_OVER_PI, scale_bound(a, FAM_NH3_INV, (float)cE300));
      F.wide = wide_br(F, 2, a.cmax[FAM_NH3_INV]);
      o.fam[FAM_NH3_INV] = F;
      return;
    }
    case 2: {  // NH3 rotational (nh3_hs.py:232-265)
      F.c[0][1] = 0.2984f * Ph2 * pw(lTdiv, 0.8730f);
      F.c[0][2] = 0.75f * Phe * pw(lTdiv, 0.66666667f);
      F.c[0][3] = 3.1789f * Pnh3 * Tdiv;
      set_cE(F, cE300);
      set_fac(F, 2.4268f * hs_base * FOUR_OVER_PI, scale_bound(a, FAM_NH3_ROT, (float)cE300));
      o.fam[FAM_NH3_ROT] = F;
      return;
    }
    case 3: {  // NH3 nu2 (nh3_hs.py:269-302); per-line widths 1.4 / 0.68 / 9.5
      F.c[0][1] = Ph2 * pw(lTdiv, 0.73f);
      F.c[0][2] = Phe * pw(lTdiv, 0.5716f);
      F.c[0][3] = Pnh3 * Tdiv;
      set_cE(F, cE300);
      set_fac(F, 1.1206f * hs_base * FOUR_OVER_PI, scale_bound(a, FAM_NH3_V2, (float)cE300));
      o.fam[FAM_NH3_V2] = F;
      return;
    }
    case 4: {  // NH3 sjs (nh3_sjs.py:37-124)
      float sj[2][5] = {{0.f, 0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f, 0.f}};
      if (use_sjs) {
        const double cE296g = -(invT - 1.0 / 296.0) * 1.438396 * LOG2E;
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
          sj[s][0] = tt * (c[0] * Ph2 + c[1] * Phe);
          sj[s][1] = tt * (c[2] * Pnh3);
          sj[s][2] = tt * (c[3] * Ph2 + c[4] * Phe);
          sj[s][3] = tt * (c[5] * Pnh3);
          sj[s][4] = c[6] * Pnh3;
        }
        const float Pscale = 1.0f + P / 1.0E5f;
        set_cE(F, cE296g);
        set_fac(F, 7.244E+21f * (Pnh3 / 296.f) * pw(log2f(296.f / T), 3.5f) * Pscale * GHZ_INVCM * TWO_OVER_PI,
                scale_bound(a, FAM_NH3_SJS, (float)cE296g));
      }
      for (int s = 0; s < 2; ++s)
        for (int k = 0; k < 5; ++k) o.sjs[s][k] = sj[s][k];
      o.fam[FAM_NH3_SJS] = F;
      return;
    }
    case 5: {  // H2S (h2s_ddb.py:42-87)
      const double cE296g = -(invT - 1.0 / 296.0) * 1.438396 * LOG2E;
      const float l296 = log2f(296.f / T);
      const float t7 = pw(l296, 0.7f);
      F.c[0][0] = t7 * (1.960f * Ph2 + 1.200f * Phe);
      F.c[0][1] = t7 * Ph2s;
      F.c[0][5] = 1.f;                     // zeta = gamma
      F.c[0][7] = 1.28f * Ph2s;            // delta
      set_cE(F, cE296g);
      set_fac(F, 7.244E+21f * (Ph2s / 296.f) * pw(l296, 3.5f) * GHZ_INVCM * TWO_OVER_PI,
              scale_bound(a, FAM_H2S, (float)cE296g));
      F.wide = wide_br(F, 1, a.cmax[FAM_H2S]);
      o.fam[FAM_H2S] = F;
      return;
    }
    case 6: {  // PH3 (ph3_jh.py:64-108)
      const double cE300g = -(invT - 1.0 / 300.0) * 1.438396 * LOG2E;
      F.c[0][1] = pw(lTdiv, 2.f / 3.f) * (3.2930f * Ph2 + 1.6803f * Phe);
      F.c[0][2] = Tdiv * 4.2157f * Pph3;
      set_cE(F, cE300g);
      set_fac(F, 7.244E+21f * (Pph3 / 300.f) * pw(lTdiv, 3.5f) * GHZ_INVCM * TWO_OVER_PI,
              scale_bound(a, FAM_PH3, (float)cE300g));
      o.fam[FAM_PH3] = F;
      return;
    }
    default: {  // H2O lines (h2o_bk.py:80-99) and continuum (102-121)
      const double cEh2o = (1.0 - 300.0 * invT) * LOG2E;
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
      o.fam[FAM_H2O] = F;
      const float Cf_he = 1.0e6f * 1.03562010226e-10f, Cf_h2 = 1.0e6f * 5.07722009423e-11f;
      const float th3 = Theta * Theta * Theta;
      const float foreign = Cf_he * Phe * Ph2o * th3 + Cf_h2 * Ph2 * Ph2o * th3;
      const float selfc = 3.1e-07f * pw(lTh, 12.f) * ((Ph2o * 1000.f) * (Ph2o * 1000.f));
      o.h2o_cont = (4.342945f * foreign + 4.342945f * selfc) / DB_PER_INVCM;
      return;
    }
  }
}

// ------------------------------------------------------------------ records
// A chunk holds the records of CH_LINES consecutive lines of one family for
// one layer, as CH_QUADS quads of four lines.  Field f of quad q is a
// ulonglong2 {P, Q}: P packs lines (4q, 4q+1) and Q lines (4q+2, 4q+3) as
// f32x2, so one 16-byte broadcast load feeds every chain of a thread.
//
// Fields        0        1     2      3        4       5      6     7
//   Ben-Reuven  G4-2K    K^2   S(g-z) S(g+z)K  -K_hi   -K_lo  G4    -
//   Gross       G4-2K    K^2   S g    -        -K_hi   -K_lo  G4    -
//   VVW         2(d2-c2) C^2   2h     2h C     -fo_hi  -fo_lo d2    h
//   nh3_sjs     -K_hi    -K_lo G0     S
// (G4 = 4 gamma^2; VVW: c2 = fo^2, d2 = df^2, C = c2 + d2, h = S df.)
constexpr int CH_LINES = 128;
constexpr int CH_QUADS = CH_LINES / 4;
constexpr int NFIELD = 8;

struct Chunk {
  ulonglong2 f[NFIELD][CH_QUADS];
};

enum Kind : int { K_BR = 0, K_GROSS = 1, K_VVW = 2, K_SJS = 3 };

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

// Record of one line (fields above).  Padding lines get zero strength and a
// denominator >= 3/4 for every F >= 0 (K = 1, G4 = 1), so they add exactly 0.
template <int KIND>
__device__ __forceinline__ void line_fields(const LineTable& t, const LayerFam& LF, int set, int li,
                                            bool valid, float S, float sjs_shift, float* v,
                                            float& base_part) {
  if (!valid) {
    if (KIND == K_SJS) {
      v[0] = -1e18f; v[1] = 0.f; v[2] = 0.f; v[3] = 0.f;
    } else if (KIND == K_VVW) {
      v[0] = 0.f; v[1] = 1.f; v[2] = 0.f; v[3] = 0.f; v[4] = 0.f; v[5] = 0.f; v[6] = 1.f; v[7] = 0.f;
    } else {
      v[0] = -1.f; v[1] = 1.f; v[2] = 0.f; v[3] = 0.f; v[4] = -1.f; v[5] = 0.f; v[6] = 1.f; v[7] = 0.f;
    }
    return;
  }
  if (KIND == K_BR) {
    const float* c = LF.c[set];
    const float w1 = t.w1[li], w2 = t.w2[li];
    const float g = c[0] + c[1] * w1 + c[2] * w2;
    const float z = c[3] + c[4] * w1 + c[5] * g;
    const float d = c[6] * g + c[7];
    const float fo = t.ch[li];
    const float small = fmaf(2.f * fo + d, d, (g - z) * (g + z));   // 2 fo d + d^2 + g^2 - z^2
    float KH, e;
    two_sum(t.c2h[li], small, KH, e);
    const float kl = e + t.c2l[li];
    const float G4 = 4.f * g * g;
    v[0] = fmaf(-2.f, KH, G4) - 2.f * kl;
    v[1] = fmaf(KH, KH, 2.f * KH * kl);
    v[2] = S * (g - z);
    v[3] = S * (g + z) * (KH + kl);
    v[4] = -KH;
    v[5] = -kl;
    v[6] = G4;
    v[7] = 0.f;
  } else if (KIND == K_GROSS) {
    const float g = LF.c[0][1] * t.w1[li] + LF.c[0][2] * t.w2[li] + LF.c[0][3] * t.w3[li];
    const float KH = t.c2h[li], kl = t.c2l[li];
    const float G4 = 4.f * g * g;
    v[0] = fmaf(-2.f, KH, G4) - 2.f * kl;
    v[1] = fmaf(KH, KH, 2.f * KH * kl);
    v[2] = S * g;
    v[3] = 0.f;
    v[4] = -KH;
    v[5] = -kl;
    v[6] = G4;
    v[7] = 0.f;
  } else if (KIND == K_VVW) {
    const float l2T = LF.c[0][0];
    const float df = LF.c[0][1] * t.w1[li] * exp2f(t.x1[li] * l2T) +
                     LF.c[0][2] * t.w2[li] * exp2f(t.x2[li] * l2T) +
                     LF.c[0][3] * t.w3[li] * exp2f(t.x3[li] * l2T);
    const float d2 = df * df;
    const float h = S * df;
    const float ch = t.ch[li], cl = t.cl[li];
    const float c2 = fmaf(ch, ch, 2.f * ch * cl);
    const float C = c2 + d2;
    v[0] = 2.f * (d2 - c2);
    v[1] = C * C;
    v[2] = 2.f * h;
    v[3] = 2.f * h * C;
    v[4] = -ch;
    v[5] = -cl;
    v[6] = d2;
    v[7] = h;
    base_part += 2.f * h / (562500.f + d2);     // the -2 df / (750^2 + df^2) term (h2o_bk.py:174-176,184)
  } else {  // K_SJS
    const float fo = t.ch[li];
    float KH, e;
    two_sum(t.c2h[li], (2.f * fo + sjs_shift) * sjs_shift, KH, e);
    v[0] = -KH;
    v[1] = -(e + t.c2l[li]);
    v[2] = t.w1[li];
    v[3] = S;
  }
}

// Build the records of lines [c0, c1), padded to whole quads, into ck0
// (coefficient set 0) and ck1 (set 1), either may be null.  One line per
// thread: the strength is formed once for both sets, and every thread of
// the CTA takes an equal share.  In a chunk, field f of line l is float
// f * CH_LINES + l (quad q packs lines 4q .. 4q+3).
template <int KIND>
__device__ __forceinline__ void build_chunk(Chunk* ck0, Chunk* ck1, const LineTable& t,
                                            const LayerFam& LF, int c0, int c1, float sjs_shift,
                                            float& base_part) {
  constexpr int NF = KIND == K_SJS ? 4 : NFIELD;
  const int nl = 4 * ((c1 - c0 + 3) >> 2);
  float* o0 = reinterpret_cast<float*>(ck0);
  float* o1 = reinterpret_cast<float*>(ck1);
  for (int l = threadIdx.x; l < nl; l += blockDim.x) {
    const int li = c0 + l;
    const bool valid = li < c1;
    const float S = valid ? line_strength(t, LF, li) : 0.f;
    float v[NFIELD];
    if (o0) {
      line_fields<KIND>(t, LF, 0, li, valid, S, sjs_shift, v, base_part);
#pragma unroll
      for (int f = 0; f < NF; ++f) o0[f * CH_LINES + l] = v[f];
    }
    if (KIND == K_BR && o1) {
      float u = 0.f;   // the VVW base term is counted once (set 0 only)
      line_fields<KIND>(t, LF, 1, li, valid, S, sjs_shift, v, u);
#pragma unroll
      for (int f = 0; f < NF; ++f) o1[f * CH_LINES + l] = v[f];
    }
  }
}

// ------------------------------------------------------------------ sweeps
// Two line pairs P, Q (packed halves) share one reciprocal per chain:
// nP/dP + nQ/dQ = (nP dQ + nQ dP) / (dP dQ).
//
// Fast form, lines whose centre is outside [0.75 fmin, 1.3 fmax] of the
// chain: den = F (F + (G4 - 2K)) + K^2, error <= ~18 ulp there.
template <int KIND>
__device__ __forceinline__ void eval_fast(f2 F, const ulonglong2& c1, const ulonglong2& c2,
                                          const ulonglong2& a, const ulonglong2& b, Acc2& acc) {
  const f2 dP = fma2(F, add2(F, c1.x), c2.x);
  const f2 dQ = fma2(F, add2(F, c1.y), c2.y);
  f2 N;
  if (KIND == K_GROSS) {
    N = fma2(a.x, dQ, mul2(a.y, dP));
  } else {
    const f2 nP = fma2(a.x, F, b.x);
    const f2 nQ = fma2(a.y, F, b.y);
    N = fma2(nP, dQ, mul2(nQ, dP));
  }
  acc.add_div(N, mul2(dP, dQ));
}

// Precise Ben-Reuven / Gross: den = ((F - K_hi) + (FL - K_lo))^2 + G4 F.
template <int KIND>
__device__ __forceinline__ void eval_precise(f2 F, f2 FL, const ulonglong2& a,
                                             const ulonglong2& b, const ulonglong2& mKH,
                                             const ulonglong2& mKL, const ulonglong2& G4,
                                             Acc2& acc) {
  const f2 eP = add2(add2(F, mKH.x), add2(FL, mKL.x));
  const f2 eQ = add2(add2(F, mKH.y), add2(FL, mKL.y));
  const f2 dP = fma2(eP, eP, mul2(G4.x, F));
  const f2 dQ = fma2(eQ, eQ, mul2(G4.y, F));
  f2 N;
  if (KIND == K_GROSS) {
    N = fma2(a.x, dQ, mul2(a.y, dP));
  } else {
    const f2 nP = fma2(a.x, F, b.x);
    const f2 nQ = fma2(a.y, F, b.y);
    N = fma2(nP, dQ, mul2(nQ, dP));
  }
  acc.add_div(N, mul2(dP, dQ));
}

// Precise VVW: den1 = ((f - fo_hi) + (fl - fo_lo))^2 + df^2, den2 = (f + fo)^2 + df^2,
// line term h (den1 + den2) / (den1 den2).
__device__ __forceinline__ void vvw_half(f2 fq, f2 fl, f2 mch, f2 mcl, f2 d2, f2 h, f2& n, f2& D) {
  const f2 dm = add2(add2(fq, mch), add2(fl, mcl));
  const f2 den1 = fma2(dm, dm, d2);
  const f2 dp = fma2(mch, dup(-1.f), fq);
  const f2 den2 = fma2(dp, dp, d2);
  n = mul2(h, add2(den1, den2));
  D = mul2(den1, den2);
}

__device__ __forceinline__ void eval_precise_vvw(f2 fq, f2 fl, const ulonglong2& mch,
                                                 const ulonglong2& mcl, const ulonglong2& d2,
                                                 const ulonglong2& h, Acc2& acc) {
  f2 nP, DP, nQ, DQ;
  vvw_half(fq, fl, mch.x, mcl.x, d2.x, h.x, nP, DP);
  vvw_half(fq, fl, mch.y, mcl.y, d2.y, h.y, nQ, DQ);
  acc.add_div(fma2(nP, DQ, mul2(nQ, DP)), mul2(DP, DQ));
}

// Per-thread frequency registers of one chain.
struct ChainF {
  f2 F, FL;     // f^2 as (hi, lo), both halves duplicated
  f2 fq, fl;    // f as (hi, lo) (VVW precise path only)
};

// Records of one quad held in registers.
struct QuadRec {
  ulonglong2 c1, c2, a, b;          // fast fields 0..3
  ulonglong2 mKH, mKL, G4, h;       // precise fields 4..7
};

// Fields for the chains of one record set: FAST if some chain takes the
// expanded form, PREC if some chain takes the double-float form.
template <int KIND, bool FAST, bool PREC>
__device__ __forceinline__ void load_quad(const Chunk& ck, int q, QuadRec& r) {
  if (FAST) {
    r.c1 = ck.f[0][q];
    r.c2 = ck.f[1][q];
  }
  if (FAST || KIND != K_VVW) {   // the precise VVW path needs no a, b
    r.a = ck.f[2][q];
    r.b = KIND == K_GROSS ? r.a : ck.f[3][q];
  }
  if (PREC) {
    r.mKH = ck.f[4][q];
    r.mKL = ck.f[5][q];
    r.G4 = ck.f[6][q];
    r.h = KIND == K_VVW ? ck.f[7][q] : r.G4;
  }
}

template <int KIND, bool PREC>
__device__ __forceinline__ void eval_tier(const QuadRec& r, const ChainF& c, Acc2& acc) {
  if (!PREC) {
    eval_fast<KIND>(c.F, r.c1, r.c2, r.a, r.b, acc);
  } else if (KIND == K_VVW) {
    eval_precise_vvw(c.fq, c.fl, r.mKH, r.mKL, r.G4, r.h, acc);
  } else {
    eval_precise<KIND>(c.F, c.FL, r.a, r.b, r.mKH, r.mKL, r.G4, acc);
  }
}

// Chains [lo, hi) at precision mask PM: any of them fast / precise.
template <int PM>
__host__ __device__ constexpr bool any_fast(int lo, int hi) {
  return lo >= hi ? false : (((PM >> lo) & 1) == 0 || any_fast<PM>(lo + 1, hi));
}
template <int PM>
__host__ __device__ constexpr bool any_prec(int lo, int hi) {
  return lo >= hi ? false : (((PM >> lo) & 1) != 0 || any_prec<PM>(lo + 1, hi));
}

// Quads [q0, q1) for all M chains, chain k at the double-float tier when
// bit k of PM is set.  Chains [0, KS) read set-0 records (ck0), chains past
// the split read set-1 records (ck1); with MIX, chain KS reads per lane
// from the set of its own slot.  Every record load is shared by the chains
// of its set; Kahan flush every 64 lines (all terms are positive, so a
// 16-term float32 block sum per lane is good to ~1e-6 before compensation).
template <int M, int KIND, int PM, int KS, bool MIX>
__device__ __forceinline__ void run_tier(const Chunk& ck0, const Chunk& ck1, const Chunk& ckl,
                                         int q0, int q1, const ChainF (&cf)[M], Acc2 (&acc)[M]) {
  constexpr bool USE0 = KS > 0;
  constexpr bool USE1 = KS + (MIX ? 1 : 0) < M;
  constexpr int K1 = KS + (MIX ? 1 : 0);
  int q = q0;
  for (; q < q1;) {
    const int qe = min(q1, q + 16);
#pragma unroll 1
    for (; q < qe; ++q) {
      QuadRec r0, r1, rl;
      if (USE0) load_quad<KIND, any_fast<PM>(0, KS), any_prec<PM>(0, KS)>(ck0, q, r0);
      if (USE1) load_quad<KIND, any_fast<PM>(K1, M), any_prec<PM>(K1, M)>(ck1, q, r1);
      if (MIX) load_quad<KIND, any_fast<PM>(KS, KS + 1), any_prec<PM>(KS, KS + 1)>(ckl, q, rl);
#pragma unroll
      for (int k = 0; k < M; ++k) {
        const QuadRec& r = k < KS ? r0 : ((MIX && k == KS) ? rl : r1);
        if ((PM >> k) & 1)
          eval_tier<KIND, true>(r, cf[k], acc[k]);
        else
          eval_tier<KIND, false>(r, cf[k], acc[k]);
      }
    }
#pragma unroll
    for (int k = 0; k < M; ++k) acc[k].flush();
  }
}

// Set split of one warp -> one compiled variant (M = 2 or 4).
template <int M, int KIND, int PM>
__device__ __forceinline__ void run_split(int ks, bool mix, const Chunk& ck0, const Chunk& ck1,
                                          const Chunk& ckl, int q0, int q1,
                                          const ChainF (&cf)[M], Acc2 (&acc)[M]) {
  if (KIND != K_BR || ks >= M) {
    run_tier<M, KIND, PM, M, false>(ck0, ck1, ckl, q0, q1, cf, acc);
    return;
  }
  // inversion lines with set-1 chains in this warp
  if (!mix) {
    switch (ks) {
      case 0: run_tier<M, KIND, PM, 0, false>(ck0, ck1, ckl, q0, q1, cf, acc); break;
      case 1: run_tier<M, KIND, PM, 1, false>(ck0, ck1, ckl, q0, q1, cf, acc); break;
      case 2: run_tier<M, KIND, PM, (M > 2 ? 2 : 0), false>(ck0, ck1, ckl, q0, q1, cf, acc); break;
      default: run_tier<M, KIND, PM, (M > 3 ? 3 : 0), false>(ck0, ck1, ckl, q0, q1, cf, acc); break;
    }
  } else {
    switch (ks) {
      case 0: run_tier<M, KIND, PM, 0, true>(ck0, ck1, ckl, q0, q1, cf, acc); break;
      case 1: run_tier<M, KIND, PM, 1, true>(ck0, ck1, ckl, q0, q1, cf, acc); break;
      case 2: run_tier<M, KIND, PM, (M > 2 ? 2 : 0), true>(ck0, ck1, ckl, q0, q1, cf, acc); break;
      default: run_tier<M, KIND, PM, (M > 3 ? 3 : 0), true>(ck0, ck1, ckl, q0, q1, cf, acc); break;
    }
  }
}

// One chunk.  M = 2: the quads are cut where a chain's double-float window
// starts or ends, and each chain takes the double-float form only inside
// its own window (the other chain of the warp stays on the expanded form).
// M = 4: the hull of the chains' windows runs at the double-float tier for
// every chain.
template <int M, int KIND>
__device__ __forceinline__ void sweep_chunk(const Chunk& ck0, const Chunk& ck1, const Chunk& ckl,
                                            int c0, int c1, int ks, bool mix, const int (&na)[M],
                                            const int (&nb)[M], const ChainF (&cf)[M],
                                            Acc2 (&acc)[M]) {
  const int nq = (c1 - c0 + 3) >> 2;
  int qa[M], qb[M];   // each chain's window, in quads of this chunk
#pragma unroll
  for (int k = 0; k < M; ++k) {
    qa[k] = nq;
    qb[k] = 0;
    if (na[k] < nb[k]) {
      qa[k] = max((na[k] - c0) >> 2, 0);
      qb[k] = min((nb[k] - c0 + 3) >> 2, nq);
    }
  }
  if (M == 2) {
    int q = 0;
    while (q < nq) {
      int e = nq, pm = 0;
#pragma unroll
      for (int k = 0; k < M; ++k) {
        const bool in = qa[k] < qb[k] && q >= qa[k] && q < qb[k];
        pm |= in ? (1 << k) : 0;
        e = min(e, in ? qb[k] : (qa[k] > q && qa[k] < qb[k] ? qa[k] : nq));
      }
      switch (pm) {
        case 0: run_split<M, KIND, 0>(ks, mix, ck0, ck1, ckl, q, e, cf, acc); break;
        case 1: run_split<M, KIND, 1>(ks, mix, ck0, ck1, ckl, q, e, cf, acc); break;
        case 2: run_split<M, KIND, 2>(ks, mix, ck0, ck1, ckl, q, e, cf, acc); break;
        default: run_split<M, KIND, 3>(ks, mix, ck0, ck1, ckl, q, e, cf, acc); break;
      }
      q = e;
    }
    return;
  }
  int ha = nq, hb = 0;   // hull
#pragma unroll
  for (int k = 0; k < M; ++k) {
    if (qa[k] < qb[k]) {
      ha = min(ha, qa[k]);
      hb = max(hb, qb[k]);
    }
  }
  constexpr int ALL = (1 << M) - 1;
  if (ha >= hb) {
    run_split<M, KIND, 0>(ks, mix, ck0, ck1, ckl, 0, nq, cf, acc);
    return;
  }
  if (ha > 0) run_split<M, KIND, 0>(ks, mix, ck0, ck1, ckl, 0, ha, cf, acc);
  run_split<M, KIND, ALL>(ks, mix, ck0, ck1, ckl, ha, hb, cf, acc);
  if (hb < nq) run_split<M, KIND, 0>(ks, mix, ck0, ck1, ckl, hb, nq, cf, acc);
}

__device__ __forceinline__ bool fam_is_hs(int fam) {
  return fam == FAM_NH3_INV || fam == FAM_NH3_ROT || fam == FAM_NH3_V2;
}

// Whether a family contributes to a layer (the assembly kernel reads
// exactly these).
__device__ __forceinline__ bool fam_enabled(const AlphaArgs& a, const LayerParams& lp, int fam) {
  const bool nh3 = a.cfg.nh3_mode != NH3_OFF;
  switch (fam) {
    case FAM_NH3_INV:
    case FAM_NH3_ROT:
    case FAM_NH3_V2: return nh3 && lp.use_hs;
    case FAM_NH3_SJS: return nh3 && lp.use_sjs;
    case FAM_H2O: return a.cfg.use_h2o;
    case FAM_H2S: return a.cfg.use_h2s;
    default: return a.cfg.use_ph3;
  }
}

__device__ __forceinline__ size_t res_index(const AlphaArgs& a, int L, int tile, int t) {
  return (((size_t)L * a.ntile + tile) * a.ntmpl + t) * a.spt;
}

// One item of a Ben-Reuven / Gross / VVW family: lines [l0, l1) of one
// layer for all slots of one tile.  Records are double-buffered: chunk c+1
// is built while chunk c is swept, one barrier per chunk.  Inversion items
// build the records of each coefficient set the tile uses.
template <int M, int KIND>
__device__ __forceinline__ void lines_item(const AlphaArgs& a, Chunk (&buf)[2][2], float* s_red,
                                           int L, int tile, int t, int fam, int l0, int l1) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const bool hsf = fam_is_hs(fam);
  const LineTable& tab = a.tab[fam];
  const LayerFam& LF = a.lp[L].fam[fam];
  const ChainPlan* cp = a.chains + ((size_t)tile * a.W + warp) * M;
  const int tflags = a.tile_flags[tile];
  const bool inv = fam == FAM_NH3_INV;
  const bool b0 = !inv || (tflags & CH_SET0), b1 = inv && (tflags & CH_SET1);
  const int wsets = a.warp_sets[tile * a.W + warp];
  const int ks = inv ? (wsets & 255) : M;
  const bool mix = inv && (wsets & 256);
  ChainF cf[M];
  int na[M], nb[M], ls[M];
  int lane_set = 0;
#pragma unroll
  for (int k = 0; k < M; ++k) {
    ls[k] = 32 * cp[k].block + lane;
    const int s = tile * a.spt + ls[k];
    const float2 Fv = hsf ? a.sp.Fhs[s] : a.sp.F[s];
    cf[k].F = dup(Fv.x);
    cf[k].FL = dup(Fv.y);
    if (KIND == K_VVW) {
      const float2 fv = a.sp.f[s];
      cf[k].fq = dup(fv.x);
      cf[k].fl = dup(fv.y);
    } else {
      cf[k].fq = cf[k].fl = 0ull;
    }
    if (mix && k == ks) lane_set = a.sp.set[s];
    const int2 nr = cp[k].near[fam];
    na[k] = LF.wide ? 0 : nr.x;
    nb[k] = LF.wide ? 0 : nr.y;
  }
  Acc2 acc[M];
#pragma unroll
  for (int k = 0; k < M; ++k) acc[k].init();
  float base_part = 0.f;
  const int nch = (l1 - l0 + CH_LINES - 1) / CH_LINES;
  build_chunk<KIND>(b0 ? &buf[0][0] : nullptr, b1 ? &buf[0][1] : nullptr, tab, LF, l0,
                    min(l1, l0 + CH_LINES), 0.f, base_part);
  __syncthreads();
  for (int c = 0; c < nch; ++c) {
    const int c0 = l0 + c * CH_LINES, c1 = min(l1, c0 + CH_LINES);
    const int nbuf = (c + 1) & 1;
    if (c + 1 < nch)
      build_chunk<KIND>(b0 ? &buf[nbuf][0] : nullptr, b1 ? &buf[nbuf][1] : nullptr, tab, LF, c1,
                        min(l1, c1 + CH_LINES), 0.f, base_part);
    const Chunk& ck0 = buf[c & 1][0];
    const Chunk& ck1 = buf[c & 1][1];
    sweep_chunk<M, KIND>(ck0, ck1, lane_set ? ck1 : ck0, c0, c1, ks, mix, na, nb, cf, acc);
    __syncthreads();
  }
  float* out = a.res + res_index(a, L, tile, t);
#pragma unroll
  for (int k = 0; k < M; ++k)
    if (cp[k].flags & CH_VALID) out[ls[k]] = acc[k].value();
  if (KIND == K_VVW) {
    float v = base_part;
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) s_red[warp] = v;
    __syncthreads();
    if (tid == 0) {
      float tot = 0.f;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += s_red[w];
      a.base[((size_t)L * a.ntile + tile) * a.ntmpl + t] = tot;
    }
  }
}

// One nh3_sjs item (nh3_sjs.py:37-124): coefficients depend on frequency
// (Spilker / Joiner blend per slot), every line takes the double-float path
// and its own reciprocal; chains are swept one after another.
template <int M>
__device__ __forceinline__ void sjs_item(const AlphaArgs& a, Chunk (&buf)[2][2], int L, int tile,
                                         int t, int l0, int l1) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const LineTable& tab = a.tab[FAM_NH3_SJS];
  const LayerParams& lp = a.lp[L];
  const LayerFam& LF = lp.fam[FAM_NH3_SJS];
  const ChainPlan* cp = a.chains + ((size_t)tile * a.W + warp) * M;
  const float shift = lp.sjs[0][4];   // delta = -0.45 P_NH3 in every set
  float c0s[4], dcs[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    c0s[q] = lp.sjs[1][q];
    dcs[q] = lp.sjs[0][q] - lp.sjs[1][q];
  }
  int ls[M];
  unsigned am = 0;
#pragma unroll
  for (int k = 0; k < M; ++k) {
    ls[k] = 32 * cp[k].block + lane;
    if (cp[k].flags & CH_VALID) am |= 1u << k;
  }
  Acc2 acc[M];
#pragma unroll
  for (int k = 0; k < M; ++k) acc[k].init();
  float unused = 0.f;
  const f2 mone = dup(-1.f);
  const int nch = (l1 - l0 + CH_LINES - 1) / CH_LINES;
  build_chunk<K_SJS>(&buf[0][0], nullptr, tab, LF, l0, min(l1, l0 + CH_LINES), shift, unused);
  __syncthreads();
  for (int c = 0; c < nch; ++c) {
    const int c0 = l0 + c * CH_LINES, c1 = min(l1, c0 + CH_LINES);
    if (c + 1 < nch)
      build_chunk<K_SJS>(&buf[(c + 1) & 1][0], nullptr, tab, LF, c1, min(l1, c1 + CH_LINES), shift,
                         unused);
    const Chunk& ck = buf[c & 1][0];
    const int nq = (c1 - c0 + 3) >> 2;
#pragma unroll
    for (int k = 0; k < M; ++k) {
      if (!((am >> k) & 1u)) continue;
      const int s = tile * a.spt + ls[k];
      const float wJ = a.sp.wJ[s];
      const f2 A = dup(fmaf(dcs[0], wJ, c0s[0])), B = dup(fmaf(dcs[1], wJ, c0s[1]));
      const f2 C = dup(fmaf(dcs[2], wJ, c0s[2])), D = dup(fmaf(dcs[3], wJ, c0s[3]));
      const float2 Fv = a.sp.F[s];
      const f2 F = dup(Fv.x), FL = dup(Fv.y), F4 = dup(4.f * Fv.x);
      int cnt = 0;
      for (int q = 0; q < nq; ++q) {
        const ulonglong2 mKH = ck.f[0][q], mKL = ck.f[1][q], G0 = ck.f[2][q], S = ck.f[3][q];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const f2 kh = h ? mKH.y : mKH.x, kl = h ? mKL.y : mKL.x;
          const f2 w = h ? G0.y : G0.x, st = h ? S.y : S.x;
          const f2 g = fma2(B, w, A);
          const f2 z = fma2(D, w, C);
          const f2 gm = fma2(z, mone, g);
          const f2 gp = add2(g, z);
          const f2 g2z2 = mul2(gm, gp);
          const f2 d1 = fma2(g2z2, mone, add2(add2(F, kh), add2(FL, kl)));
          const f2 den = fma2(d1, d1, mul2(F4, mul2(g, g)));
          const f2 num = fma2(gm, F, mul2(gp, fma2(kh, mone, g2z2)));
          acc[k].add_div(mul2(st, num), den);
        }
        if (++cnt == 8) {
          cnt = 0;
          acc[k].flush();
        }
      }
      acc[k].flush();
    }
    __syncthreads();
  }
  float* out = a.res + res_index(a, L, tile, t);
#pragma unroll
  for (int k = 0; k < M; ++k)
    if ((am >> k) & 1u) out[ls[k]] = acc[k].value();
}

// ------------------------------------------------------------------ assembly
constexpr int ASM_TMAX = 16;   // templates summed from registers by the assembly (= tfam size)

// Sum of the items of one family for one slot, in template order (the
// items were written by the line-sum kernel launched before).
__device__ __forceinline__ float fam_sum(const AlphaArgs& a, const float* r, int fam) {
  float v = 0.f;
#pragma unroll 4
  for (int t = a.vbeg[fam]; t < a.vend[fam]; ++t) v += __ldcg(r + (size_t)t * a.spt);
  return v;
}

// One slot of one layer: family sums -> per-gas absorption, scaled, float32
// total for the brightness scan and the optional float64 outputs.
__device__ __forceinline__ void assemble_slot(const AlphaArgs& a, int L, int tile, int ls,
                                              const LayerParams& lp) {
  const int s = tile * a.spt + ls;
  if (s >= a.nslot) return;
  const int j = s < a.nf ? s : -1;   // the frequency plan's slot -> frequency map (padding -1)
  if (j < 0) return;
  const float* r = a.res + res_index(a, L, tile, 0) + ls;
  const int set = a.sp.set[s];
  // Family sums in template order.  Up to ASM_TMAX templates every item's
  // value is loaded first (independent loads, one round trip to L2) and
  // added to its template's family; items of a family that is off in this
  // layer were not written and their sums are not used.
  float fs[NFAM];
#pragma unroll
  for (int f = 0; f < NFAM; ++f) fs[f] = 0.f;
  if (a.ntmpl <= ASM_TMAX) {
    float v[ASM_TMAX];
#pragma unroll
    for (int t = 0; t < ASM_TMAX; ++t) v[t] = t < a.ntmpl ? __ldcg(r + (size_t)t * a.spt) : 0.f;
#pragma unroll
    for (int t = 0; t < ASM_TMAX; ++t) {
      if (t >= a.ntmpl) break;
      switch (a.tfam[t]) {   // kernel argument, the same for every thread
        case FAM_NH3_INV: fs[FAM_NH3_INV] += v[t]; break;
        case FAM_NH3_ROT: fs[FAM_NH3_ROT] += v[t]; break;
        case FAM_NH3_V2: fs[FAM_NH3_V2] += v[t]; break;
        case FAM_NH3_SJS: fs[FAM_NH3_SJS] += v[t]; break;
        case FAM_H2O: fs[FAM_H2O] += v[t]; break;
        case FAM_H2S: fs[FAM_H2S] += v[t]; break;
        default: fs[FAM_PH3] += v[t]; break;
      }
    }
  } else {
    for (int f = 0; f < NFAM; ++f) fs[f] = fam_sum(a, r, f);
  }
  const bool hs_on = fam_enabled(a, lp, FAM_NH3_INV);
  const float inv = hs_on ? fs[FAM_NH3_INV] : 0.f, rot = hs_on ? fs[FAM_NH3_ROT] : 0.f,
              v2 = hs_on ? fs[FAM_NH3_V2] : 0.f;
  const float sjs = fam_enabled(a, lp, FAM_NH3_SJS) ? fs[FAM_NH3_SJS] : 0.f;
  const float h2o = a.cfg.use_h2o ? fs[FAM_H2O] : 0.f;
  const float h2s = a.cfg.use_h2s ? fs[FAM_H2S] : 0.f, ph3 = a.cfg.use_ph3 ? fs[FAM_PH3] : 0.f;
  float base = 0.f;
  if (a.cfg.use_h2o) {
    const float* bs = a.base + ((size_t)L * a.ntile + tile) * a.ntmpl;
    for (int t = a.vbeg[FAM_H2O]; t < a.vend[FAM_H2O]; ++t) base += __ldcg(bs + t);
  }
  double co = 0.0, cl = 0.0;
  if (a.extra) {
    co = a.extra[(size_t)L * a.nf + j];
    cl = a.extra[((size_t)a.nL + L) * a.nf + j];
  }
  const float2 Fs = a.sp.F[s], Hs = a.sp.Fhs[s];
  float g32[NGAS];
  assemble<float>(lp, a.cfg, Fs.x + Fs.y, Hs.x + Hs.y, set, inv, rot, v2, sjs, h2o, base, h2s, ph3,
                  co, cl, g32);
  float tot = 0.f;
  for (int k = 0; k < NGAS; ++k) tot += g32[k];
  a.alpha32[(size_t)L * a.nf + j] = a.cfg.units_db ? tot / DB_PER_INVCM : tot;
  if (a.layers64 || a.gas64) {
    const double f = a.freqs[j], fh = a.freqs_hs[j];
    double g64[NGAS];
    assemble<double>(lp, a.cfg, f * f, fh * fh, set, inv, rot, v2, sjs, h2o, base, h2s, ph3, co, cl,
                     g64);
    double t64 = 0.0;
    for (int k = 0; k < NGAS; ++k) {
      if (a.gas64) a.gas64[((size_t)L * a.nf + j) * NGAS + k] = g64[k];
      t64 += g64[k];
    }
    if (a.layers64) a.layers64[(size_t)j * a.nL + L] = t64;
  }
}

// ------------------------------------------------------------------ kernels
// Persistent line-sum kernel: every CTA takes items from a.counter until
// none are left.  Item i -> template entry i / (nL ntile), then layers deep
// to shallow, then tiles; template entries come heaviest family first, so
// the queue ends with the smallest items.  Each item writes its per-slot
// sums; rb_alpha_assemble_kernel, launched next, assembles them.
template <int M>
__global__ void __launch_bounds__(128, M >= 4 ? 4 : 6) rb_alpha_lines_kernel(AlphaArgs a) {
  __shared__ __align__(16) Chunk buf[2][2];   // [double buffer][coefficient set]
  __shared__ int s_item[2];
  __shared__ float s_red[4];
  const int per = a.nL * a.ntile;
  for (int it = 0;; ++it) {
    // Thread 0 takes items until one has work (an item whose family is off
    // in its layer, nh3_sjs outside the blend layers say, is skipped).  The
    // previous item's last barrier orders its record reads before the next
    // item's record stores; s_item is double-buffered across iterations.
    if (threadIdx.x == 0) {
      int item;
      for (;;) {
        item = atomicAdd(a.counter, 1);
        if (item >= a.nitems) break;
        const int t = item / per, rem = item - t * per;
        const int L = a.nL - 1 - rem / a.ntile;
        if (fam_enabled(a, a.lp[L], a.tmpl[t].fam)) break;
      }
      s_item[it & 1] = item;
    }
    __syncthreads();
    const int item = s_item[it & 1];
    if (item >= a.nitems) break;
    const int t = item / per, rem = item - t * per;
    const int L = a.nL - 1 - rem / a.ntile, tile = rem % a.ntile;
    const TmplEntry e = a.tmpl[t];
    switch (e.fam) {
      case FAM_NH3_INV:
      case FAM_H2S:
      case FAM_PH3: lines_item<M, K_BR>(a, buf, s_red, L, tile, t, e.fam, e.l0, e.l1); break;
      case FAM_NH3_ROT:
      case FAM_NH3_V2: lines_item<M, K_GROSS>(a, buf, s_red, L, tile, t, e.fam, e.l0, e.l1); break;
      case FAM_H2O: lines_item<M, K_VVW>(a, buf, s_red, L, tile, t, e.fam, e.l0, e.l1); break;
      default: sjs_item<M>(a, buf, L, tile, t, e.l0, e.l1); break;
    }
  }
}

// Assembly: one thread per (layer, slot), layers x nslot threads in a 1-D
// grid (the batched sweeps have millions of layers).  The CTA first copies
// the LayerParams of the layers it spans into shared memory with one
// coalesced read (the slots' coefficient reads then wait on no round trips);
// a CTA spans at most ASM_LMAX layers when a layer has 32 slots or more.
constexpr int ASM_LMAX = 5;
__global__ void __launch_bounds__(128) rb_alpha_assemble_kernel(AlphaArgs a) {
  __shared__ __align__(16) LayerParams s_lp[ASM_LMAX];
  const size_t ntot = (size_t)a.nL * a.nslot;
  const size_t g0 = (size_t)blockIdx.x * blockDim.x;
  const int L0 = (int)(g0 / a.nslot);
  const int nlay = (int)((min(g0 + blockDim.x, ntot) - 1) / a.nslot) - L0 + 1;
  const bool staged = nlay <= ASM_LMAX;
  if (staged) {
    constexpr int WORDS = (int)(sizeof(LayerParams) / sizeof(int));
    const int* src = reinterpret_cast<const int*>(a.lp + L0);
    int* dst = reinterpret_cast<int*>(s_lp);
    for (int i = threadIdx.x; i < nlay * WORDS; i += blockDim.x) dst[i] = __ldg(src + i);
  }
  __syncthreads();
  const size_t g = g0 + threadIdx.x;
  if (g >= ntot) return;
  const int L = (int)(g / a.nslot);
  const int s = (int)(g - (size_t)L * a.nslot);
  assemble_slot(a, L, s / a.spt, s % a.spt, staged ? s_lp[L - L0] : a.lp[L]);
}

// ------------------------------------------------------------------ launch
cudaError_t launch_prep(const PrepArgs& pa, cudaStream_t st) {
  const int n = pa.nL * PREP_PARTS;
  rb_layer_prep_kernel<<<(n + 255) / 256, 256, 0, st>>>(pa);
  return cudaGetLastError();
}

// Resident CTAs per SM of the line-sum kernel for M chains and W warps.
int alpha_lines_occupancy(int M, int W) {
  int n = 0;
  cudaError_t e = cudaSuccess;
  if (M == 4) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, rb_alpha_lines_kernel<4>, 32 * W, 0);
  else e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, rb_alpha_lines_kernel<2>, 32 * W, 0);
  return e == cudaSuccess ? n : 0;
}

cudaError_t launch_alpha_lines(const AlphaArgs& aa, int nblocks, cudaStream_t st) {
  if (aa.nitems > 0) {
    const int nb = std::max(1, std::min(nblocks, aa.nitems));
    const int nthr = 32 * aa.W;
    if (aa.M == 4) rb_alpha_lines_kernel<4><<<nb, nthr, 0, st>>>(aa);
    else rb_alpha_lines_kernel<2><<<nb, nthr, 0, st>>>(aa);
  }
  return cudaGetLastError();
}

cudaError_t launch_alpha_assemble(const AlphaArgs& aa, cudaStream_t st) {
  const size_t n = (size_t)aa.nL * aa.nslot;
  rb_alpha_assemble_kernel<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(aa);
  return cudaGetLastError();
}

}  // namespace rb
