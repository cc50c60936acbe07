// Per-gas absorption of one (layer, frequency) from the family line sums:
// prefactors, units, the nh3_hs clamp and the nh3_hs / nh3_sjs pressure
// blend, the per-gas scales.  Shared by the absorption assembly kernel and
// the stored-tangent JVP, which both form the float32 alpha the brightness
// scan reads.
#pragma once
#include "rb_args.cuh"

namespace rb {

// Con of the inversion coefficient sets [inv_table][set] (nh3_hs.py:139-168,
// nh3_dbs.py:133-162).
__device__ constexpr float INV_CON[2][2] = {{0.9301f, 0.9862f}, {0.9619f, 0.9862f}};

// Assemble one slot: per-gas absorption (T = float or double), scaled.
// co / cl are the co_ddb and clouds_idp absorption in cm^-1 (0 when off).
template <typename T>
__device__ __forceinline__ void assemble(const LayerParams& lp, const AlphaConfig& cfg, T F, T Fhs,
                                         int set, float inv, float rot, float v2, float sjs,
                                         float h2o, float base_h2o, float h2s, float ph3, double co,
                                         double cl, T* g) {
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
      hs = Fhs * (sc(lp.fam[FAM_NH3_INV].fm * INV_CON[cfg.inv_table][set], lp.fam[FAM_NH3_INV].fe, inv) +
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
  if (cfg.use_co) g[GAS_CO] = (T)co * U;
  if (cfg.use_clouds) g[GAS_CLOUDS] = (T)cl * U;
  for (int k = 0; k < NGAS; ++k) g[k] *= (T)lp.scale[k];
}

}  // namespace rb
