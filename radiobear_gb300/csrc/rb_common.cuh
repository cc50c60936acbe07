// Shared device-side definitions for the radioBEAR GB300 forward model.
//
// Layout conventions (all device buffers owned by an rb_handle):
//   * line catalogues: structure-of-arrays per family, lines sorted by
//     centre frequency, derived columns precomputed on the host in float64;
//   * per-layer scalars (partial pressures, width coefficients, strength
//     prefactors) live in an array of LayerParams, one per layer, computed
//     by rb_layer_prep_kernel in float64;
//   * absorption for the brightness scan is float32 [nL][nf] (frequency
//     contiguous, so a warp reading 32 frequencies of one layer is one
//     128-byte transaction).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace rb {

// Line families.  Values match include/radiobear_gb300.h RB_FAM_*.
enum Family : int {
  FAM_NH3_INV = 0,   // nh3_hs inversion lines, Ben-Reuven (constituents/nh3/nh3_hs.py:172-229)
  FAM_NH3_ROT = 1,   // nh3_hs rotational lines, Gross (nh3_hs.py:232-265)
  FAM_NH3_V2 = 2,    // nh3_hs nu2 lines, Gross with fixed widths (nh3_hs.py:269-302)
  FAM_NH3_SJS = 3,   // nh3_sjs lines, Ben-Reuven with frequency-dependent coefficients
  FAM_H2O = 4,       // h2o_bk lines, modified Van Vleck-Weisskopf (h2o_bk.py:130-189)
  FAM_H2S = 5,       // h2s_ddb lines, Ben-Reuven zeta = gamma (h2s_ddb.py:42-87)
  FAM_PH3 = 6,       // ph3_jh lines, Ben-Reuven zeta = delta = 0 (ph3_jh.py:64-108)
  NFAM = 7
};

// Gas slots of the per-gas output, the reference's sorted constituent order
// (alpha.py:80): h2, h2o, h2s, nh3, ph3.
enum Gas : int { GAS_H2 = 0, GAS_H2O = 1, GAS_H2S = 2, GAS_NH3 = 3, GAS_PH3 = 4, NGAS = 5 };

// Abundance rows of the X input [NX][nL].
enum XRow : int { X_H2 = 0, X_HE = 1, X_CH4 = 2, X_NH3 = 3, X_H2O = 4, X_H2S = 5, X_PH3 = 6, NX = 7 };

// NH3 formalism selector.
enum Nh3Mode : int { NH3_OFF = 0, NH3_HS = 1, NH3_SJS = 2, NH3_HS_SJS = 3 };

// One line family on the device (SoA, sorted by centre).
struct LineTable {
  int n;
  // centre terms (float pairs = exact-ish double-float of a float64 value)
  const float* c2h;    // centre^2 high part   (BR/Gross: fo^2; VVW: unused)
  const float* c2l;    // centre^2 low part
  const float* ch;     // centre high part     (VVW: fo + SR; BR: fo)
  const float* cl;     // centre low part
  const double* lnI;   // log strength incl. line weights and the 1/fo^2 of (f/fo)^2
  const double* E;     // lower-state energy term multiplying LayerFam::cE
  const float* w1;     // per-line width parameters (family specific)
  const float* w2;
  const float* w3;
  const float* x1;     // per-line temperature exponents (VVW only)
  const float* x2;
  const float* x3;
  const float* lnI32;  // float copy of lnI for the scale pre-pass
  const float* E32;    // float copy of E
};

// Per (layer, family) scalars.
struct LayerFam {
  double fac;      // alpha_fam(f) = fac * f^2 * sum_l S'_l shape_l(f)   [cm^-1]
  double M;        // log-strength offset: S'_l = exp(lnI_l + cE*E_l - M)
  double cE;
  // width model (Ben-Reuven, per coefficient set s):
  //   gamma = g0 + g1*w1 + g2*w2, zeta = z0 + z1*w1 + zg*gamma,
  //   delta = dg*gamma + d0
  // Gross: gamma = g1*w1 + g2*w2 + g3*w3 (set 0).
  // VVW:  df = g1*w1*T^x1 + g2*w2*T^x2 + g3*w3*T^x3 with Theta exponents
  //       (g1..g3 = partial pressures), logTheta in g0.
  float c[2][8];
};

// Per-layer parameters.
struct LayerParams {
  double P, T;
  LayerFam fam[NFAM];
  double h2_cia;       // alpha_h2(f) = h2_cia * f^2
  double h2o_cont;     // continuum part of alpha_h2o(f) = h2o_cont * f^2
  double blendW;       // nh3_hs_sjs weight of sjs (0: hs only, 1: sjs only)
  int use_hs, use_sjs; // which NH3 formalisms this layer evaluates
  // nh3_sjs coefficient sets: [0] Joiner, [1] Spilker; each
  // {GH2, GHe, GNH3, ZH2, ZHe, ZNH3, D} already multiplied by the partial
  // pressures and (T0/T)^(2/3) where the formula does so.
  double sjs[2][8];
};

struct AlphaConfig {
  int nh3_mode;        // Nh3Mode
  int use_h2, use_h2o, use_h2s, use_ph3;
  int h2state;         // 'e' or 'n'
  int units_db;        // 0: cm^-1, 1: dB/km (the nh3 clamp applies after units)
};

// ---------------------------------------------------------------- helpers
__host__ __device__ inline void split_double(double v, float& hi, float& lo) {
  hi = (float)v;
  lo = (float)(v - (double)hi);
}

// Error-free transformation a + b = s + e (Knuth TwoSum), float.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// Compensated accumulator: running sum plus a plain partial over a block
// of terms, folded in with Kahan's correction every few dozen terms.
struct KahanAcc {
  float s, c, part;
  __device__ __forceinline__ void init() { s = 0.f; c = 0.f; part = 0.f; }
  __device__ __forceinline__ void flush() {
    float y = part - c;
    float t = s + y;
    c = (t - s) - y;
    s = t;
    part = 0.f;
  }
  __device__ __forceinline__ float value() const { return s - c + part; }
};

}  // namespace rb
