// Shared device-side definitions for the radioBEAR GB300 forward model.
//
// Layout conventions (all device buffers owned by an rb_handle):
//   * line catalogues: structure-of-arrays per family, lines sorted by
//     centre frequency, derived columns precomputed on the host in float64
//     and stored as float pairs (double-float) where float32 would lose
//     digits;
//   * per-layer scalars (width coefficients, strength prefactors as
//     mantissa x 2^exponent) live in an array of LayerParams, one per layer;
//   * frequencies are planned into "slots", tiles of 32 * M * W slots (M
//     slots per thread, W warps per CTA), padded at the end of the last tile;
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

// Gas slots of the per-gas output: the reference's sorted constituent order
// (alpha.py:80) for the line gases h2, h2o, h2s, nh3, ph3, then the
// closed-form absorbers co (co_ddb) and clouds (clouds_idp).
enum Gas : int {
  GAS_H2 = 0, GAS_H2O = 1, GAS_H2S = 2, GAS_NH3 = 3, GAS_PH3 = 4, GAS_CO = 5, GAS_CLOUDS = 6,
  NGAS = 7
};

// Rows of the X input [NX][nL]: gas mole fractions, then the cloud
// densities (g/cm^3) of the reference's cloud table columns H2O (ice),
// SOLN (liquid), NH4SH, NH3, H2S and CH4.
enum XRow : int {
  X_H2 = 0, X_HE = 1, X_CH4 = 2, X_NH3 = 3, X_H2O = 4, X_H2S = 5, X_PH3 = 6, X_CO = 7,
  X_CL_H2O = 8, X_CL_SOLN = 9, X_CL_NH4SH = 10, X_CL_NH3 = 11, X_CL_H2S = 12, X_CL_CH4 = 13,
  NX = 14
};

// NH3 formalism selector (structure of the blend; the inversion
// coefficient table is AlphaConfig::inv_table).
enum Nh3Mode : int { NH3_OFF = 0, NH3_HS = 1, NH3_SJS = 2, NH3_HS_SJS = 3 };

// co_ddb line shape (other_dict['coshape'], co_ddb.py:36-39,86-93).
enum CoShape : int { CO_VOIGT = 0, CO_VVW = 1, CO_DIFF = 2, CO_STD = 3 };

// clouds_idp particle switches (other_dict '<kind>_p' > 0, clouds_idp.py:16-49).
enum CloudBit : int {
  CL_ICE = 1, CL_WATER = 2, CL_NH4SH = 4, CL_NH3ICE = 8, CL_H2SICE = 16, CL_CH4 = 32
};

// One line family on the device (SoA, sorted by centre).
struct LineTable {
  int n;
  const float* c2h;    // centre^2 high part   (Ben-Reuven / Gross / sjs: fo^2)
  const float* c2l;    //          low part
  const float* ch;     // centre high part     (VVW: fo + SR; others: fo)
  const float* cl;     //        low part
  const float* l2Ih;   // log2 strength (incl. line weights and the 1/fo^2 of (f/fo)^2), hi
  const float* l2Il;   //                                                               lo
  const float* Eh;     // energy term multiplying LayerFam::cE, hi
  const float* El;     //                                       lo
  const float* w1;     // per-line width parameters (family specific)
  const float* w2;
  const float* w3;
  const float* x1;     // per-line temperature exponents (VVW only)
  const float* x2;
  const float* x3;
  float l2Imax, Emin, Emax;   // family statistics for the strength scale
};

// Per (layer, family) scalars.
//   alpha_fam(f) = fm * 2^fe * f^2 * sum_l S'_l shape_l(f)   [cm^-1]
//   S'_l = 2^(l2I_l + cE * E_l - M2) <= 1, M2 an integer upper bound of the
//   exponent over the family (from l2Imax, Emin, Emax), so no line pass is
//   needed to scale float32 sums.
struct LayerFam {
  float fm;        // prefactor mantissa
  int fe;          // exponent incl. M2
  float cEh, cEl;  // double-float log2 energy coefficient
  float M2;        // integer-valued strength offset
  // width model (Ben-Reuven, per coefficient set s):
  //   gamma = c0 + c1*w1 + c2*w2, zeta = c3 + c4*w1 + c5*gamma,
  //   delta = c6*gamma + c7
  // Gross: gamma = c1*w1 + c2*w2 + c3*w3 (set 0).
  // VVW:  df = c1*w1*Th^x1 + c2*w2*Th^x2 + c3*w3*Th^x3, c0 = log2(Theta).
  float c[2][8];
  // 1 when the lines are wide enough at this layer for the expanded
  // denominator everywhere: 4 gamma^2 >= 0.27 K for every line (gamma at
  // least 0.32 of the largest centre), which bounds its rounding error by
  // ~18 ulp as outside the near-line windows.  Ben-Reuven families only.
  int wide;
};

// Per-layer parameters.
struct LayerParams {
  float P, T;
  LayerFam fam[NFAM];
  float h2_cia;        // alpha_h2(f) = h2_cia * f^2
  float h2o_cont;      // continuum part of alpha_h2o(f) = h2o_cont * f^2
  float blendW;        // nh3_hs_sjs weight of sjs (0: hs only, 1: sjs only)
  int use_hs, use_sjs; // which NH3 formalisms this layer evaluates
  // nh3_sjs coefficient sets [0] Joiner, [1] Spilker:
  //   gamma = [0] + [1]*G0, zeta = [2] + [3]*G0, delta = [4]
  float sjs[2][5];
  float scale[NGAS];   // per-gas multipliers (1 when no scale is given)
};

struct AlphaConfig {
  int nh3_mode;        // Nh3Mode
  int use_h2, use_h2o, use_h2s, use_ph3;
  int h2state;         // 'e' or 'n'
  int units_db;        // 0: cm^-1, 1: dB/km (the nh3 clamp applies after units)
  int inv_table;       // NH3 inversion coefficients: 0 nh3_hs, 1 nh3_dbs
  int use_co;          // co_ddb
  int coshape;         // CoShape
  int use_clouds;      // clouds_idp
  int cloud_mask;      // CloudBit set
};

// Frequency slot plan (see AlphaArgs for the slot -> thread mapping).
struct SlotPlan {
  const int* j;          // [nslot] frequency index, -1 = padding
  const float2* F;       // [nslot] (hi, lo) of f^2
  const float2* Fhs;     // [nslot] (hi, lo) of the nh3_hs frequency squared
  const float2* f;       // [nslot] (hi, lo) of f
  const float* wJ;       // [nslot] nh3_sjs Joiner weight (0 f<=26, 1 f>=34, linear between)
  const int* set;        // [nslot] nh3_hs coefficient set (0: <=30 GHz, 1: >30 GHz)
};

// ---------------------------------------------------------------- helpers
__host__ __device__ inline void split_double(double v, float& hi, float& lo) {
  hi = (float)v;
  lo = (float)(v - (double)hi);
}

// Error-free transformation a + b = s + e (Knuth TwoSum), float.  The
// _rn intrinsics keep the compiler from contracting a product that feeds
// a or b into the first addition (s would then round the exact product
// while e accounts for the rounded one).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

}  // namespace rb
