// Kernel argument blocks shared by the launch code (rb_api.cu) and the
// kernels.  Passed by value as __grid_constant__-style kernel parameters.
#pragma once
#include "rb_common.cuh"

namespace rb {

struct PrepArgs {
  int nL;
  const double* P;
  const double* T;
  const double* X;       // [NX][nL]
  const double* scale;   // [nL][NGAS] or null
  AlphaConfig cfg;
  float l2Imax[NFAM], Emin[NFAM], Emax[NFAM];
  int nlines[NFAM];
  LayerParams* out;
};

struct AlphaArgs {
  int nL, nf, nslot;
  SlotPlan sp;
  const double* freqs;      // [nf] (float64 outputs only)
  const double* freqs_hs;   // [nf] frequency evaluated by nh3_hs in slot j
  const LayerParams* lp;
  LineTable tab[NFAM];
  const int2* near;         // [nwarps total][NFAM] line index ranges
  AlphaConfig cfg;
  float* alpha32;           // [nL][nf] total, cm^-1 (brightness input)
  double* layers64;         // [nf][nL] total, units of cfg (or null)
  double* gas64;            // [nL][nf][NGAS] per gas, units of cfg (or null)
};

struct RayArgs {
  int nL;
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
};

struct TbArgs {
  int nL, nf, nb, max_seg;
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
  float4* part;           // [nb][nchunk][nf] {dtau_hi, dtau_lo, intW, TbL} per chunk
};

}  // namespace rb
