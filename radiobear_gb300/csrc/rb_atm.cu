// Atmosphere producer on the device: the derived properties of
// AtmosphereBase.computeProp (radiobear/atm_base.py:120-194) and the
// pressure regrid of regrid.regrid (radiobear/regrid.py:11-176), for one
// atmosphere or a batch (one CTA per atmosphere), float64.
//
// Tables are the reference's column tables [ncol][n] with a caller-given
// column role map (Z, T, P, DZ) and per-column chemistry (amu, c_p / R,
// refractivity constant; a negative refractivity selects the H2O law
// 245 + 1.28e6 / T, chemistry.py:32-40).
//
//   rb_atm_prop_kernel    per layer: mean amu, refractivity, N, radius
//                         about the layer nearest p_ref; the enclosed mass
//                         G dM as a block prefix sum; GM normalised at
//                         p_ref, g, scale height, lapse rates.
//   rb_atm_regrid_kernel  linear-in-P interpolation onto the grid; points
//                         deeper than the table: constituents at their
//                         deepest value, T and z along a dry adiabat in
//                         hydrostatic equilibrium (serial recurrence);
//                         points above it: T and z along the last slope;
//                         z renormalised to 0 at the deepest point, DZ in
//                         cm; the cloud table interpolated with 0 outside.
#include "rb_args.cuh"
#include <math_constants.h>

namespace rb {

constexpr double ATM_GRAV = 6.6738e-20;   // km3/kg/s2, chemistry.py:7
constexpr double ATM_RGAS = 8.314462;     // J/K/mol, chemistry.py:8
constexpr double ATM_FILL = -999.9;       // regrid.py:63
constexpr int ATM_THREADS = 256;

__device__ __forceinline__ double refr_col(const AtmCols& c, int k, double T) {
  return c.refr[k] < 0.0 ? 245.0 + 1.28E6 / T : c.refr[k];
}

__device__ __forceinline__ bool is_chem(const AtmCols& c, int k) {
  return k != c.iz && k != c.it && k != c.ip && k != c.idz;
}

// Block-wide inclusive prefix sum of one double per thread.
__device__ double block_scan(double v, double* sh) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int o = 1; o < 32; o <<= 1) {
    const double u = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += u;
  }
  if (lane == 31) sh[warp] = v;
  __syncthreads();
  if (warp == 0) {
    double w = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0.0;
    for (int o = 1; o < 32; o <<= 1) {
      const double u = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += u;
    }
    sh[lane] = w;
  }
  __syncthreads();
  const double add = warp > 0 ? sh[warp - 1] : 0.0;
  __syncthreads();
  return v + add;
}

// Index of the layer nearest p_ref (first of equals, as the reference's
// strict-less scan).
__device__ int nearest_pref(const double* P, int n, double p_ref, double* shv, int* shi) {
  double best = 1.0E6;
  int bi = 0x7fffffff;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double d = fabs(P[i] - p_ref);
    if (d < best) {
      best = d;
      bi = i;
    }
  }
  for (int o = 16; o; o >>= 1) {
    const double ob = __shfl_xor_sync(0xffffffffu, best, o);
    const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
    if (ob < best || (ob == best && oi < bi)) {
      best = ob;
      bi = oi;
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    shv[warp] = best;
    shi[warp] = bi;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
      if (shv[w] < shv[0] || (shv[w] == shv[0] && shi[w] < shi[0])) {
        shv[0] = shv[w];
        shi[0] = shi[w];
      }
    if (shi[0] == 0x7fffffff) shi[0] = 0;   // no layer within 1e6 bar: the reference keeps 0
  }
  __syncthreads();
  const int r = shi[0];
  __syncthreads();
  return r;
}

__device__ __forceinline__ double col_amu(const AtmCols& c, const double* g, size_t ld, int i) {
  double s = 0.0;
  for (int k = 0; k < c.ncol; ++k)
    if (is_chem(c, k)) s += c.amu[k] * g[(size_t)k * ld + i];
  return s;
}

// computeProp of one table (columns strided by ld) into prop rows (strided
// by pld).  The whole CTA takes part.
__device__ void atm_props(const AtmCols& c, const double* g, size_t ld, int n, double Req,
                          double p_ref, double GM_ref, double* prop, size_t pld) {
  __shared__ double shv[32];
  __shared__ int shi[32];
  __shared__ double scan_sh[32];
  const double* P = g + (size_t)c.ip * ld;
  const double* T = g + (size_t)c.it * ld;
  const double* Z = g + (size_t)c.iz * ld;
  const int io = nearest_pref(P, n, p_ref, shv, shi);
  const double zOff = Z[io];
  double carry = 0.0;
  for (int base = 0; base < n; base += blockDim.x) {
    const int i = base + threadIdx.x;
    double gdm = 0.0;
    if (i < n) {
      const double rr = Req + Z[i] - zOff;
      const double amu = col_amu(c, g, ld, i);
      double refr = 0.0;
      for (int k = 0; k < c.ncol; ++k)
        if (is_chem(c, k)) refr += refr_col(c, k, T[i]) * g[(size_t)k * ld + i];
      refr = refr * P[i] * (293.0 / T[i]);
      prop[PROP_Z * pld + i] = Z[i];
      prop[PROP_R * pld + i] = rr;
      prop[PROP_P * pld + i] = P[i];
      prop[PROP_AMU * pld + i] = amu;
      prop[PROP_REFR * pld + i] = refr;
      prop[PROP_N * pld + i] = refr / 1.0E6 + 1.0;
      double lapse = 0.0, lapsep = 0.0;
      if (i > 0) {
        const double rho = (amu * P[i]) / (ATM_RGAS * T[i]);
        const double dr = fabs(Z[i] - Z[i - 1]);
        const double dM = 1.0e11 * rho * (4.0 * CUDART_PI * (rr * rr) * dr);
        gdm = ATM_GRAV * dM;
        const double dT = fabs(T[i] - T[i - 1]);
        lapse = dT / dr;
        lapsep = dT / fabs(P[i] - P[i - 1]);
      }
      prop[PROP_LAPSE * pld + i] = lapse;
      prop[PROP_LAPSEP * pld + i] = lapsep;
    }
    const double cum = block_scan(gdm, scan_sh) + carry;
    if (i < n) prop[PROP_GM * pld + i] = cum;
    // carry: the last thread's inclusive sum
    __shared__ double s_carry;
    if (threadIdx.x == blockDim.x - 1) s_carry = cum;
    __syncthreads();
    carry = s_carry;
    __syncthreads();
  }
  const double GMnorm = prop[PROP_GM * pld + io];
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double gm = GM_ref - (prop[PROP_GM * pld + i] - GMnorm);
    const double rr = prop[PROP_R * pld + i];
    const double little_g = gm / (rr * rr);
    prop[PROP_GM * pld + i] = gm;
    prop[PROP_g * pld + i] = little_g;
    prop[PROP_H * pld + i] = (ATM_RGAS * T[i]) / (little_g * prop[PROP_AMU * pld + i]) / 1000.0;
  }
  __syncthreads();
}

__global__ void __launch_bounds__(ATM_THREADS) rb_atm_prop_kernel(AtmPropArgs a) {
  const int v = blockIdx.x;
  const int o = a.off ? a.off[v] : 0;
  const int n = a.off ? a.off[v + 1] - o : a.ld;
  atm_props(a.cols, a.gas + o, a.ld, n, a.Req, a.p_ref, a.GM_ref, a.prop + o, a.ld);
}

// Interval of pressure p in the increasing table Pin, as scipy's linear
// interp1d takes it: hi = the first index with Pin[hi] >= p, clipped to
// [1, n-1], lo = hi - 1; false outside [P0, Pn-1] (bounds_error=False).
__device__ __forceinline__ bool interp_at(const double* Pin, int n, double p, int& lo) {
  if (!(p >= Pin[0] && p <= Pin[n - 1])) return false;
  int a = 0, b = n;   // lower bound
  while (a < b) {
    const int mid = (a + b) >> 1;
    if (Pin[mid] < p) a = mid + 1;
    else b = mid;
  }
  const int hi = a < 1 ? 1 : (a > n - 1 ? n - 1 : a);
  lo = hi - 1;
  return true;
}

// slope (y_hi - y_lo) / (x_hi - x_lo) times (p - x_lo) plus y_lo
__device__ __forceinline__ double lerp_col(const double* x, const double* y, int lo, double p) {
  const double slope = (y[lo + 1] - y[lo]) / (x[lo + 1] - x[lo]);
  return slope * (p - x[lo]) + y[lo];
}

__device__ void renorm_z(double* tab, size_t ld, int iz, int idz, int n) {
  const double zDeep = tab[(size_t)iz * ld + n - 1];
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) tab[(size_t)iz * ld + i] -= zDeep;
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x)
    tab[(size_t)idz * ld + i] =
        i == 0 ? 0.0 : fabs(tab[(size_t)iz * ld + i] - tab[(size_t)iz * ld + i - 1]) * 1.0E5;
  __syncthreads();
}

__global__ void __launch_bounds__(ATM_THREADS) rb_atm_regrid_kernel(AtmRegridArgs a) {
  const int v = blockIdx.x;
  const AtmCols& c = a.cols;
  const int oi = a.in_off[v];
  const int n = a.in_off[v + 1] - oi;
  const int m = a.nout;
  const size_t ldi = a.ld_in, ldo = a.ld_out;
  const double* gin = a.gas_in + oi;
  double* go = a.gas_out + (size_t)v * m;
  const double* grid = a.pgrid + (size_t)v * a.pgrid_stride;
  const double* Pin = gin + (size_t)c.ip * ldi;
  __shared__ int s_any_fill, s_any_deep;
  if (threadIdx.x == 0) {
    s_any_fill = 0;
    s_any_deep = 0;
  }
  __syncthreads();
  // interpolation (regrid.py:103-124); P is the grid, DZ is left for renorm
  for (int i = threadIdx.x; i < m; i += blockDim.x) {
    const double p = grid[i];
    int lo = 0;
    const bool in = n > 1 && interp_at(Pin, n, p, lo);
    if (!in) s_any_fill = 1;
    for (int k = 0; k < c.ncol; ++k) {
      double val;
      if (k == c.ip) val = p;
      else if (k == c.idz) val = 0.0;
      else val = in ? lerp_col(Pin, gin + (size_t)k * ldi, lo, p) : ATM_FILL;
      go[(size_t)k * ldo + i] = val;
    }
  }
  __syncthreads();
  if (s_any_fill) {
    // g and r at the table's deepest layer (computeProp of the input)
    __shared__ double shv[32];
    __shared__ int shi[32];
    __shared__ double s_red[32];
    const int io = nearest_pref(Pin, n, a.p_ref, shv, shi);
    const double* T = gin + (size_t)c.it * ldi;
    const double* Z = gin + (size_t)c.iz * ldi;
    const double zOff = Z[io];
    // sum of G dM over layers (io, n-1]: GM(n-1) - GM(io) before normalisation
    double part = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      if (i <= io) continue;
      const double rr = a.Req + Z[i] - zOff;
      const double amu = col_amu(c, gin, ldi, i);
      const double rho = (amu * Pin[i]) / (ATM_RGAS * T[i]);
      const double dr = fabs(Z[i] - Z[i - 1]);
      part += ATM_GRAV * (1.0e11 * rho * (4.0 * CUDART_PI * (rr * rr) * dr));
    }
    for (int o = 16; o; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = part;
    __syncthreads();
    // constituents outside the table: their deepest value (regrid.py:130-137)
    for (int i = threadIdx.x; i < m; i += blockDim.x) {
      for (int k = 0; k < c.ncol; ++k) {
        if (!is_chem(c, k)) continue;
        double& y = go[(size_t)k * ldo + i];
        if (y == ATM_FILL) y = gin[(size_t)k * ldi + n - 1];
      }
      if (grid[i] >= Pin[n - 1]) s_any_deep = 1;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double gm_rel = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) gm_rel += s_red[w];
      const double rDeep = a.Req + Z[n - 1] - zOff;
      double gg = (a.GM_ref - gm_rel) / (rDeep * rDeep);
      double r = rDeep;
      const double pDeep = Pin[n - 1];
      double* Pg = go + (size_t)c.ip * ldo;
      double* Tg = go + (size_t)c.it * ldo;
      double* Zg = go + (size_t)c.iz * ldo;
      // dry adiabat in hydrostatic equilibrium (regrid.py:138-157)
      for (int i = 0; i < m; ++i) {
        const double p = Pg[i];
        if (p < pDeep) continue;
        const int im = i > 0 ? i - 1 : m - 1;
        const double prev = Pg[im];
        const double dP = p - prev;
        const double Tp = Tg[im];
        const double z = Zg[im];
        double amu = 0.0, cp = 0.0;
        for (int k = 0; k < c.ncol; ++k) {
          if (!is_chem(c, k)) continue;
          cp += c.cp[k] * go[(size_t)k * ldo + i];
          amu += c.amu[k] * go[(size_t)k * ldo + i];
        }
        Tg[i] = Tp + Tp / (cp * p) * dP;
        gg = gg + 2.0 * ATM_RGAS * Tp * log(p / prev) / (r * amu) / 1000.0;
        const double H = ATM_RGAS * Tp / (amu * gg) / 1000.0;
        const double dz = H * dP / p;
        r = r - dz;
        Zg[i] = z - dz;
      }
    }
    __syncthreads();
    // above the table: every column but P and DZ along its last slope
    // (regrid.py:159-176), one thread per column
    const double* Pg = go + (size_t)c.ip * ldo;
    for (int k = threadIdx.x; k < c.ncol; k += blockDim.x) {
      if (k == c.ip || k == c.idz) continue;
      double* y = go + (size_t)k * ldo;
      int i0 = 0;
      while (i0 < m && y[i0] == ATM_FILL) ++i0;
      if (i0 == 0 || i0 + 1 >= m) continue;
      const double slope = (y[i0 + 1] - y[i0]) / (Pg[i0 + 1] - Pg[i0]);
      for (int jj = i0 - 1; jj >= 0; --jj) {
        y[jj] = y[jj + 1] + slope * (Pg[jj + 1] - Pg[jj]);
        if (y[jj] <= 0.0) y[jj] = 1e-20;
      }
    }
    __syncthreads();
  }
  renorm_z(go, ldo, c.iz, c.idz, m);
  // clouds: interpolated, 0 outside, z renormalised
  if (a.cloud_in) {
    const AtmCols& cl = a.cloud_cols;
    const double* cin = a.cloud_in + oi;
    double* co = a.cloud_out + (size_t)v * m;
    const double* Pc = cin + (size_t)cl.ip * ldi;
    for (int i = threadIdx.x; i < m; i += blockDim.x) {
      const double p = grid[i];
      int lo = 0;
      const bool in = n > 1 && interp_at(Pc, n, p, lo);
      for (int k = 0; k < cl.ncol; ++k) {
        double val;
        if (k == cl.ip) val = p;
        else if (k == cl.idz) val = 0.0;
        else val = in ? lerp_col(Pc, cin + (size_t)k * ldi, lo, p) : 0.0;
        co[(size_t)k * ldo + i] = val;
      }
    }
    __syncthreads();
    renorm_z(co, ldo, cl.iz, cl.idz, m);
  }
}

cudaError_t launch_atm_props(const AtmPropArgs& a, int nvar, cudaStream_t st) {
  if (nvar <= 0) return cudaSuccess;
  rb_atm_prop_kernel<<<nvar, ATM_THREADS, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_atm_regrid(const AtmRegridArgs& a, int nvar, cudaStream_t st) {
  if (nvar <= 0) return cudaSuccess;
  rb_atm_regrid_kernel<<<nvar, ATM_THREADS, 0, st>>>(a);
  return cudaGetLastError();
}

}  // namespace rb
