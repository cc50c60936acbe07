// Kernel argument blocks shared by the launch code (rb_api.cu) and the
// kernels.  Passed by value as __grid_constant__-style kernel parameters.
#pragma once
#include "rb_common.cuh"

namespace rb {

struct PrepArgs {
  int nL;
  const double* P;
  const double* T;
  const double* X;     // [NX][nL]
  AlphaConfig cfg;
  LineTable tab[NFAM];
  LayerParams* out;
};

struct AlphaArgs {
  int nL, nf, nwarps_tile;
  const double* freqs;      // [nf]
  const double* freqs_hs;   // [nf] frequency evaluated by nh3_hs in slot j
  const LayerParams* lp;
  LineTable tab[NFAM];
  const int2* near;         // [ntile][nwarps][NFAM] line index ranges
  AlphaConfig cfg;
  const double* scale;      // [nL][NGAS] or null
  float* alpha32;           // [nL][nf] total, cm^-1 (brightness input)
  double* layers64;         // [nf][nL] total, units of cfg (or null)
  double* gas64;            // [nL][nf][NGAS] per gas, units of cfg (or null)
};

struct RayArgs {
  int nL;
  const double* R;      // equatorial radius of each layer [km], layer 0 on top
  const double* N;      // refractive index of each layer
  double k;             // b/a of the shell ellipse (Rpol/Req, or 1 for a sphere)
  double rot[9];        // rotate2planet matrix, row-major
  int limb_sec;
  int nb;
  const double* b;      // [nb][2]
  int max_seg;
  int* nseg;            // [nb]
  double* ds;           // [nb][max_seg] km
  int* layer;           // [nb][max_seg]
  double* r4ds;         // [nb][max_seg] or null
  double* latlng;       // [nb][max_seg+1][2] degrees or null
  int* end_code;        // [nb] or null: 1 index exit, 2 break, 3 capacity
};

struct TbArgs {
  int nL, nf, nb, max_seg;
  const float* alpha32;   // [nL][nf] cm^-1
  const double* T;        // [nL]
  const int* nseg;        // [nb]
  const double* ds;       // [nb][max_seg] km
  const int* layer;       // [nb][max_seg]
  int disc;
  double* Tb;             // [nb][nf]
  double* intW;           // [nb][nf] or null
  double* tau;            // [nb][nf][max_seg] or null (profiles, index 0 = 0)
  double* W;
  double* TbL;
};

}  // namespace rb
