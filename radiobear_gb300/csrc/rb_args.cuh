// Kernel argument blocks shared by the launch code (rb_api.cu) and the
// kernels.  Passed by value as __grid_constant__-style kernel parameters.
#pragma once
#include "rb_common.cuh"

namespace rb {

// Segments per chunk of the parallel brightness scan; the adjoint's reverse
// sweep runs over the same chunks (it reuses the forward's chunk partials).
constexpr int SCAN_CHUNK = 64;

struct PrepArgs {
  int nL;
  const double* P;
  const double* T;
  const double* X;       // [NX][nL]
  const double* scale;   // [nL][NGAS] or null
  AlphaConfig cfg;
  float l2Imax[NFAM], Emin[NFAM], Emax[NFAM];
  float cmax[NFAM];      // largest line centre of each family (GHz)
  int nlines[NFAM];
  LayerParams* out;
  int* counter;          // line-sum work counter to reset (or null)
};

// Line-sum work decomposition.
//
// Frequencies are planned into slots, tiles of spt = 32 * M * W slots cut
// into blocks of 32 consecutive slots.  In a tile, lane i of warp w holds M
// "chains"; chain k owns slot 32 * block(w, k) + i, so the 32 lanes of one
// chain cover 32 consecutive slots (one precision decision per chain).  The
// planner picks the partition of blocks into warps (ascending within a
// warp) that minimises the double-float work.  Slot order is frequency
// order, so the nh3_hs coefficient set (0 up to 30 GHz, 1 above) is
// monotone in k: per warp, chains [0, KS) take set 0, chain KS may mix both
// sets lane by lane, the rest take set 1.
//
// The lines of every family are cut into items of at most item_lines lines;
// template entry t = (family, l0, l1).  The persistent kernel takes items
// from a global counter in the order (template entry, layer deep to
// shallow, tile); each item writes one float per slot of its tile into
// res[layer][tile][t][slot], and the assembly kernel sums those per family.
struct ChainPlan {
  int flags;              // CH_VALID | CH_SET0 | CH_SET1
  int block;              // 32-slot block of the tile owned by this chain
  int2 near[NFAM];        // line index range taking the double-float path
};
constexpr int CH_VALID = 1, CH_SET0 = 2, CH_SET1 = 4;

struct TmplEntry {
  int fam, l0, l1, pad;
};

struct AlphaArgs {
  int nL, nf, nslot;
  int M, W, spt, ntile;     // chains per thread, warps per CTA, slots per tile, tiles
  SlotPlan sp;
  const ChainPlan* chains;  // [ntile][W][M]
  const int* tile_flags;    // [ntile] OR of the tile's chain flags
  const int* warp_sets;     // [ntile][W] KS | (mixed chain KS ? 256 : 0)
  const TmplEntry* tmpl;    // [ntmpl], grouped by family
  int ntmpl;
  int vbeg[NFAM], vend[NFAM];  // template range of each family
  unsigned char tfam[16];      // family of templates 0..15 (the assembly's sums)
  int nitems;               // ntmpl * nL * ntile
  int* counter;             // work counter, zeroed by rb_layer_prep_kernel
  float* res;               // [nL][ntile][ntmpl][spt] per-item line sums
  float* base;              // [nL][ntile][ntmpl] h2o frequency-independent term per item
  const double* freqs;      // [nf] (float64 outputs only)
  const double* freqs_hs;   // [nf] frequency evaluated by nh3_hs in slot j
  const LayerParams* lp;
  LineTable tab[NFAM];
  AlphaConfig cfg;
  float* alpha32;           // [nL][nf] total, cm^-1 (brightness input)
  double* layers64;         // [nf][nL] total, units of cfg (or null)
  double* gas64;            // [nL][nf][NGAS] per gas, units of cfg (or null)
  const double* extra;      // [2][nL][nf] co_ddb, clouds_idp in cm^-1 (or null)
};

// Atmosphere tables (rb_atm.cu): the reference's column tables [ncol][n]
// with the roles of the Z, T, P and DZ columns and per-column chemistry of
// chemistry.ConstituentProperties (amu g/mol, c_p / R, refractivity
// constant; refr < 0 selects the H2O law 245 + 1.28e6 / T).
constexpr int ATM_MAXCOL = 32;
struct AtmCols {
  int ncol, iz, it, ip, idz;
  double amu[ATM_MAXCOL], cp[ATM_MAXCOL], refr[ATM_MAXCOL];
};

// Property rows of AtmosphereBase.computeProp (config LP order).
enum PropRow : int {
  PROP_Z = 0, PROP_R = 1, PROP_P = 2, PROP_GM = 3, PROP_AMU = 4, PROP_REFR = 5, PROP_N = 6,
  PROP_H = 7, PROP_LAPSE = 8, PROP_LAPSEP = 9, PROP_g = 10, NPROP = 11
};

struct AtmPropArgs {
  AtmCols cols;
  const double* gas;     // [ncol][ld]
  int ld;                // layers of all atmospheres (column stride)
  const int* off;        // [nvar + 1] layer offsets, or null for one table of ld layers
  double Req, p_ref, GM_ref;
  double* prop;          // [NPROP][ld]
};

struct AtmRegridArgs {
  AtmCols cols, cloud_cols;
  const double* gas_in;    // [ncol][ld_in]
  const double* cloud_in;  // [ncol_cloud][ld_in] (same layers as gas) or null
  int ld_in;
  const int* in_off;       // [nvar + 1]
  int nout;                // grid points per atmosphere
  const double* pgrid;     // [nvar][pgrid_stride] increasing pressures (stride 0: shared)
  int pgrid_stride;
  int ld_out;              // nvar * nout
  double Req, p_ref, GM_ref;
  double* gas_out;         // [ncol][ld_out], atmosphere v at v * nout
  double* cloud_out;       // [ncol_cloud][ld_out] or null
};

// Closed-form absorbers co_ddb (constituents/co/co_ddb.py) and clouds_idp
// (constituents/clouds/clouds_idp.py), float64, one thread per (layer,
// frequency).  The forward writes out; the adjoint contracts d loss / d
// alpha with their temperature and pressure derivatives.
struct ExtraArgs {
  int nL, nf;
  const double* P;          // [nL] bar
  const double* T;          // [nL] K
  const double* X;          // [NX][nL]
  const double* freqs;      // [nf] GHz
  int nco;                  // co.npz lines: f0 (GHz), I0, E (cm^-1)
  const double* co_f0;
  const double* co_I0;
  const double* co_E;
  AlphaConfig cfg;
  double* out;              // [2][nL][nf] cm^-1
  const float* galpha;      // [nL][nf] d loss / d alpha (cm^-1)
  const double* scale;      // [nL][NGAS] or null
  double* grad;             // [nL][2] d loss / dT, d loss / dP
};

// Batches of atmospheres: variant v owns global layers [var_off[v],
// var_off[v+1]) and rays [v * rays_per_var, (v+1) * rays_per_var); all
// variants share the impact parameters b[rays_per_var][2].  var_off == null
// is a single atmosphere (one variant, every ray its own b).
// Where a ray enters the atmosphere and its direction after the one
// refraction at the top shell (raypath.py:60-160), written by
// rb_ray_setup_kernel for the walk.
struct RayStart {
  double r0[3];     // edge point on the top shell [km]
  double s[3];      // direction after the refraction
  double u0;        // r0 . s
  double ll0[2];    // latitude, longitude of the edge point [deg] (latlng output only)
  float em1;        // E^2 - 1 at the edge point
  float em1_eq;     // E^2 - 1 on the equator (the lat == 0 rule)
  float mu;         // sqrt(1 - b^2)
  int hit;          // 0: the ray misses the planet
};

struct RayArgs {
  int nL;
  const int* var_off;   // [nvar + 1] or null
  int rays_per_var;
  const double* R;      // equatorial radius of each layer [km], layer 0 on top
  const double* N;      // refractive index of each layer
  const float2* dR2;    // [nL] R[(c+1)%nL]^2 - R[c]^2 as (hi, lo)   (rb_geom_prep_kernel)
  const float* dR;      // [nL] R[(c+1)%nL] - R[c]
  const float* R32;     // [nL] R as float
  double k;             // b/a of the shell ellipse (Rpol/Req, or 1 for a sphere)
  double rot[9];        // rotate2planet matrix, row-major
  int limb_sec;
  int nb;
  const double* b;      // [nb][2]
  int max_seg;
  int* nseg;            // [nb]
  double* ds;           // [nb][max_seg] km (or null)
  int* layer;           // [nb][max_seg]
  float* hds;           // [nb][max_seg] ds/2 in cm, float (brightness input) or null
  double* r4ds;         // [nb][max_seg] or null
  double* latlng;       // [nb][max_seg+1][2] degrees or null
  int* end_code;        // [nb] or null: 1 index exit, 2 break, 3 capacity
  RayStart* start;      // [nb] rb_ray_setup_kernel -> rb_raypath_kernel
};

struct TbArgs {
  int nL, nf, nb, max_seg;
  const int* var_off;     // [nvar + 1] or null (see RayArgs)
  int rays_per_var;
  const float* alpha32;   // [nL][nf] cm^-1
  const float* T32;       // [nL] K
  const int* nseg;        // [nb]
  const float* hds;       // [nb][max_seg] ds/2 in cm
  const int* layer;       // [nb][max_seg] (Python semantics: negatives wrap)
  int disc;               // 2 E2(tau) weighting (sequential kernel only)
  double* Tb;             // [nb][nf]
  float* Tb32;            // [nb][nf] float copy (disc average input) or null
  double* intW;           // [nb][nf] or null
  double* tau;            // [nb][nf][max_seg] or null (profiles, index 0 = 0)
  double* W;
  double* TbL;
  // chunked scan
  int chunk, nchunk;      // segments per chunk, chunks per ray
  int lanes;              // frequency-pair lanes per (ray, chunk) item of the packed scan (0: automatic)
  float4* part;           // [nb][nchunk][nf] {dtau_hi, dtau_lo, intW, TbL} per chunk
  // adjoint state (null for a forward-only call): the combine writes intW
  // per (ray, frequency) (0 where Tb is clamped to T_cmb) and replaces each
  // chunk's {intW, TbL} by its starting optical depth {tau_hi, tau_lo}
  float* iw32;            // [nb][nf]
};

// ---------------------------------------------------------------- adjoint
// Tangent directions of one layer's parameters.
constexpr int NTH = 5;
enum Tangent : int { TH_T = 0, TH_P = 1, TH_XNH3 = 2, TH_XH2O = 3, TH_XH2S = 4 };

// Derivatives of one family's layer coefficients (LayerFam) along the five
// tangents: dc for c[s][k], dlnpref for the log of the strength prefactor
// fm 2^fe, dcE = d cE / dT (log2 units per K).
struct FamTan {
  float dc[2][8][NTH];
  float dlnpref[NTH];
  float dcE;
};

struct LayerTan {
  FamTan fam[NFAM];
  float dsjs[2][5][NTH];   // nh3_sjs coefficient sets
  float dh2_cia[NTH];
  float dh2o_cont[NTH];
  float dblendW_dP;        // nh3_hs_sjs blend weight, per bar
};

struct TanArgs {
  int nL;
  const double* P;
  const double* T;
  const double* X;
  int nh3_mode, h2state;
  int inv_table;          // AlphaConfig::inv_table
  LayerTan* out;
};

struct TbAdjArgs {
  int nL, nf, nb, max_seg;
  const int* var_off;     // [nvar + 1] or null (see RayArgs)
  int rays_per_var;
  const float* alpha32;   // [nL][nf] cm^-1 (forward absorption)
  const double* T;        // [nL]
  const int* nseg;        // [nb]
  const float* hds;       // [nb][max_seg] ds/2 in cm
  const int* layer;       // [nb][max_seg]
  const double* weights;  // [nb] or null
  const double* grad;     // [nf] (with weights: d loss / d Tb_avg) or [nb][nf]
  float* ga;              // [nL][nf] d loss / d alpha (atomic sums over rays and visits)
  double* gs;             // [nL] d loss / d T through the source term
  const float4* part;     // forward scan partials [nb][nchunk][nf]: {dtau_hi, dtau_lo, tau0_hi, tau0_lo}
  const float* Tb32;      // [nb][nf] forward Tb
  const float* iw32;      // [nb][nf] forward intW, 0 where Tb is clamped (no gradient)
  int nchunk;
  float* S;               // [nb][nchunk][nf] per-chunk sums of dTb/dtau
  // b = 'disc' (E2 weighting): sequential reverse sweep, no chunk partials
  int disc;
  double2* tauE;          // [nb][max_seg][nf] {tau, 2 E2(tau)} per path node
};

// Frequency of one thread of the absorption JVP, precomputed per frequency
// with the plan (float pairs, so the kernel does no float64 arithmetic).
struct JvFreq {
  float F, FL;     // f^2 (hi, lo)
  float Fh, FhL;   // f^2 of the frequency nh3_hs evaluates in this slot
  float fq, fql;   // f (hi, lo)
  float wJ;        // nh3_sjs Spilker / Joiner weight
  int set;         // inversion coefficient set
};

struct JvpArgs {
  int nL, nf;
  const JvFreq* fplan;    // [nf]
  int ft;                 // frequencies per CTA
  int ctas;               // resident CTAs per SM the kernel is compiled for (3 or 4)
  int threads;            // threads per CTA (128 or 256; 0: automatic)
  const LayerParams* lp;
  const LayerTan* lt;
  LineTable tab[NFAM];
  AlphaConfig cfg;
  const float* galpha;    // [nL][nf] d loss / d alpha
  float2* part;           // [nL][ntile][NTH] double-float sums over the tile's frequencies
  // Stored-tangent mode (alpha_out set): before the scan, the kernel writes
  // the layer's float32 alpha and d alpha / d theta per frequency instead of
  // contracting with galpha after the reverse sweep.
  float* alpha_out;       // [nL][nf] cm^-1 (the scan's alpha)
  float* dal_out;         // [nL][NTH][nf] d alpha / d (T, P, ln X_NH3, ln X_H2O, ln X_H2S)
  const double* extra;    // co_ddb / clouds_idp alpha [2][nL][nf] in cm^-1, or null
};

}  // namespace rb
