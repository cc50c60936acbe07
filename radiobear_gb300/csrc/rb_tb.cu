// Brightness temperature along each ray: the trapezoidal optical-depth scan
// of Brightness.single (brightness.py:53-117) for sm_103a.
//
// Per segment i (layers ii = layer4ds[i], ii1 = layer4ds[i+1], ds in cm):
//   tau_{i+1} = tau_i + (a0 + a1) ds / 2                   double-float
//   W_{i+1}   = a1 exp(-tau_{i+1})      or 2 a1 E2(tau_{i+1}) for 'disc'
//   intW     += (W_{i+1} + W_i) ds / 2                      compensated fp32
//   TbL      += (T1 W_{i+1} + T0 W_i) ds / 2                compensated fp32
// with W_0 = 0, and Tb = T_cmb if TbL < T_cmb else TbL / intW
// (brightness.py:107-117).  The last ds of the path is not used, as in the
// reference loop.
//
// Fast path (exp weighting): every ray's segments are cut into chunks that
// are scanned in parallel with a local optical depth starting at 0; since
// exp(-(tau_a + t)) = exp(-tau_a) exp(-t), chunk sums combine exactly as
//   intW = sum_c exp(-tau_c) intW_c,  TbL = sum_c exp(-tau_c) TbL_c,
// tau_c being the optical depth at the chunk's first point.  One CTA covers
// (128 frequencies, one chunk, one ray); the chunk's ds / layer / T are
// staged in shared memory so the loop's only global loads are the
// alpha[layer][f0..f127] rows (coalesced, L2 resident).  With an even
// number of frequencies the packed variant takes two per thread.
// Sequential path: one thread per (ray, frequency) over the whole path; used
// for the E2 weighting of b = 'disc' and when per-segment profiles
// (tau, W, TbL) are requested.
#include "rb_args.cuh"
#include "rb_f32x2.cuh"
#include "rb_expint.cuh"
#include <math_constants.h>

namespace rb {

constexpr double T_CMB = 2.725;   // utils.py:77

__device__ __forceinline__ void kahan_add(float& s, float& c, float v) {
  const float y = v - c;
  const float t = s + y;
  c = (t - s) - y;
  s = t;
}

__device__ __forceinline__ int wrap_layer(int l, int nL) { return l < 0 ? l + nL : l; }

// Layer offset and count of a ray's atmosphere (batches: see RayArgs).
__device__ __forceinline__ void ray_layers(const TbArgs& a, int ray, int& off, int& nL) {
  off = 0;
  nL = a.nL;
  if (a.var_off) {
    const int v = ray / a.rays_per_var;
    off = a.var_off[v];
    nL = a.var_off[v + 1] - off;
  }
}

// ------------------------------------------------------------ sequential
__global__ void __launch_bounds__(128) rb_tb_seq_kernel(TbArgs a) {
  const int ray = blockIdx.x;
  const int f = blockIdx.y * blockDim.x + threadIdx.x;
  if (ray >= a.nb) return;
  const bool valid = f < a.nf;
  const int fi = valid ? f : 0;
  const int nseg = a.nseg[ray];
  const float* hds = a.hds + (size_t)ray * a.max_seg;
  const int* lay = a.layer + (size_t)ray * a.max_seg;
  const size_t pbase = ((size_t)ray * a.nf + fi) * a.max_seg;
  float th = 0.f, tl = 0.f;          // tau (double-float)
  float W0 = 0.f;
  float iw = 0.f, iwc = 0.f, tb = 0.f, tbc = 0.f;
  if (valid && a.tau) {
    a.tau[pbase] = 0.0;
    a.W[pbase] = 0.0;
    a.TbL[pbase] = 0.0;
  }
  int off, nLr;
  ray_layers(a, ray, off, nLr);
  int ii = nseg > 0 ? off + wrap_layer(lay[0], nLr) : 0;
  float T0 = nseg > 0 ? a.T32[ii] : 0.f;
  float a0 = nseg > 0 ? a.alpha32[(size_t)ii * a.nf + fi] : 0.f;
  for (int i = 0; i + 1 < nseg; ++i) {
    const int ii1 = off + wrap_layer(lay[i + 1], nLr);
    const float hd = hds[i];
    const float a1 = a.alpha32[(size_t)ii1 * a.nf + fi];
    const float T1 = a.T32[ii1];
    const float dtau = (a0 + a1) * hd;
    float s, e;
    two_sum(th, dtau, s, e);
    e += tl;
    th = s + e;
    tl = e - (th - s);
    float W1;
    if (a.disc)
      W1 = (float)(2.0 * (double)a1 * expint2((double)th + (double)tl));
    else
      W1 = a1 * __expf(-th) * (1.f - tl);
    kahan_add(iw, iwc, (W1 + W0) * hd);
    kahan_add(tb, tbc, fmaf(T1, W1, T0 * W0) * hd);
    if (valid && a.tau) {
      const size_t p = pbase + i + 1;
      a.tau[p] = (double)th + (double)tl;
      a.W[p] = (double)W1;
      a.TbL[p] = (double)tb - (double)tbc;
    }
    W0 = W1;
    T0 = T1;
    a0 = a1;
  }
  if (!valid) return;
  const double TbL = (double)tb - (double)tbc;
  const double IW = (double)iw - (double)iwc;
  const double out = (TbL < T_CMB) ? T_CMB : TbL / IW;
  a.Tb[(size_t)ray * a.nf + f] = out;
  if (a.Tb32) a.Tb32[(size_t)ray * a.nf + f] = (float)out;
  if (a.intW) a.intW[(size_t)ray * a.nf + f] = IW;
}

// ------------------------------------------------------------ chunked
constexpr int TB_CHUNK = SCAN_CHUNK;

__global__ void __launch_bounds__(128) rb_tb_chunk_kernel(TbArgs a) {
  const int ray = blockIdx.x;   // rays in x: batches have more than 65535
  const int ch = blockIdx.y;
  const int f = blockIdx.z * blockDim.x + threadIdx.x;
  const int nseg = a.nseg[ray];
  const int nsteps = nseg - 1;                 // segments used by the scan
  const int i0 = ch * TB_CHUNK;
  float4* part = a.part + ((size_t)ray * a.nchunk + ch) * a.nf;
  if (i0 >= nsteps) return;                    // chunk past the end of this ray (never read)
  const int n = min(TB_CHUNK, nsteps - i0);
  __shared__ int s_off[TB_CHUNK + 1];
  __shared__ float s_T[TB_CHUNK + 1];
  __shared__ float s_hd[TB_CHUNK];
  const float* hds = a.hds + (size_t)ray * a.max_seg + i0;
  const int* lay = a.layer + (size_t)ray * a.max_seg + i0;
  int off, nLr;
  ray_layers(a, ray, off, nLr);
  for (int t = threadIdx.x; t <= n; t += blockDim.x) {
    const int l = off + wrap_layer(lay[t], nLr);
    s_off[t] = l * a.nf;
    s_T[t] = a.T32[l];
    if (t < n) s_hd[t] = hds[t];
  }
  __syncthreads();
  if (f >= a.nf) return;
  const float* al = a.alpha32 + f;
  float th = 0.f, tl = 0.f;
  float a0 = al[s_off[0]];
  // W at the chunk's first point relative to exp(-tau_start); W_0 = 0 on a path
  float W0 = (i0 == 0) ? 0.f : a0;
  float T0 = s_T[0];
  float iw = 0.f, iwc = 0.f, tb = 0.f, tbc = 0.f;
  int i = 0;
  for (; i + 4 <= n; i += 4) {
    float an[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) an[k] = al[s_off[i + 1 + k]];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const float hd = s_hd[i + k];
      const float a1 = an[k];
      const float T1 = s_T[i + 1 + k];
      float s, e;
      two_sum(th, (a0 + a1) * hd, s, e);
      e += tl;
      th = s + e;
      tl = e - (th - s);
      const float W1 = a1 * __expf(-th) * (1.f - tl);
      kahan_add(iw, iwc, (W1 + W0) * hd);
      kahan_add(tb, tbc, fmaf(T1, W1, T0 * W0) * hd);
      W0 = W1;
      T0 = T1;
      a0 = a1;
    }
  }
  for (; i < n; ++i) {
    const float hd = s_hd[i];
    const float a1 = al[s_off[i + 1]];
    const float T1 = s_T[i + 1];
    float s, e;
    two_sum(th, (a0 + a1) * hd, s, e);
    e += tl;
    th = s + e;
    tl = e - (th - s);
    const float W1 = a1 * __expf(-th) * (1.f - tl);
    kahan_add(iw, iwc, (W1 + W0) * hd);
    kahan_add(tb, tbc, fmaf(T1, W1, T0 * W0) * hd);
    W0 = W1;
    T0 = T1;
    a0 = a1;
  }
  part[f] = make_float4(th, tl, iw - iwc, tb - tbc);
}

// Packed scan: the same arithmetic for two adjacent frequencies per thread
// in f32x2 (double-float optical depth and the two compensated sums lane by
// lane, one exp per lane); alpha rows are read as float2.  Needs an even
// frequency count (8-byte aligned pairs).  One CTA covers (256 frequencies,
// one chunk, one ray); the partials are the scalar kernel's.
__device__ __forceinline__ void two_sum2(f2 a, f2 b, f2& s, f2& e) {
  s = add2(a, b);
  const f2 bb = sub2(s, a);
  e = add2(sub2(a, sub2(s, bb)), sub2(b, bb));
}

__device__ __forceinline__ void kahan_add2(f2& s, f2& c, f2 v) {
  const f2 y = sub2(v, c);
  const f2 t = add2(s, y);
  c = sub2(sub2(t, s), y);
  s = t;
}

// Lanes per item of the packed scan: frequency pairs (a power of two in
// [4, 128]); a CTA of 128 threads takes 128 / lanes (ray, chunk) items so
// that few frequencies still fill it.
__host__ __device__ __forceinline__ int scan_lanes(int npair) {
  int l = 4;
  while (l < npair && l < 128) l <<= 1;
  return l;
}
// Staged float4 per item: entry 0 {T_0, w_0, T_0 w_0, row offset of node 0},
// entry k + 1 {hd_k, w_{k+1}, T_{k+1} w_{k+1}, row offset of node k + 1} for
// step k (node k -> k + 1), with the trapezoid weight of node j inside the
// chunk w_j = hd_{j-1} + hd_j (hd_{-1} = hd_n = 0 at the chunk's ends).
constexpr int SCAN_ITEM_F4 = TB_CHUNK + 1;
constexpr int SCAN_FLUSH = 16;   // steps per float32 block sum

// exp(-x) of both halves as 2^(-x log2(e)): one packed multiply and the
// PTX base-2 exponential approximation with flush to zero (a result below
// 2^-126, an optical depth above ~87, is 0: its weight in every sum is far
// below the float32 rounding of the sum).
__device__ __forceinline__ f2 exp_neg2(f2 x) {
  const f2 y = mul2(x, dup(-1.4426950408889634f));
  float lo = lo2(y), hi = hi2(y);
  asm("ex2.approx.ftz.f32 %0, %0;" : "+f"(lo));
  asm("ex2.approx.ftz.f32 %0, %0;" : "+f"(hi));
  return pk(lo, hi);
}

// Running state of one thread's frequency pair in the packed scan.
struct ScanPair {
  f2 a0;                    // alpha at the previous node
  f2 th, ntl;               // optical depth th - ntl
  f2 iwb, tbb;              // current float32 block sums
  f2 iw, iwc, tb, tbc;      // Kahan sums of the blocks
  __device__ __forceinline__ void init(f2 a, f2 iw0, f2 tb0) {
    a0 = a;
    th = ntl = 0ull;
    iwb = iw0;
    tbb = tb0;
    iw = iwc = tb = tbc = 0ull;
  }
  // step k: e = {hd_k, w_{k+1}, T_{k+1} w_{k+1}, -}, a1 = alpha at node k + 1
  __device__ __forceinline__ void step(f2 a1, const float4& e) {
    const f2 x = mul2(add2(a0, a1), dup(e.x));
    const f2 s = add2(th, x);
    ntl = add2(ntl, sub2(sub2(s, th), x));   // -(Fast2Sum error)
    th = s;
    const f2 ax = mul2(a1, exp_neg2(th));
    const f2 W1 = fma2(ax, ntl, ax);
    iwb = fma2(W1, dup(e.y), iwb);
    tbb = fma2(W1, dup(e.z), tbb);
    a0 = a1;
  }
  __device__ __forceinline__ void flush() {
    kahan_add2(iw, iwc, iwb);
    kahan_add2(tb, tbc, tbb);
    iwb = tbb = 0ull;
    const f2 s = sub2(th, ntl);              // renormalise: (th, tl) = Fast2Sum(th, tl)
    ntl = add2(ntl, sub2(s, th));
    th = s;
  }
};

// Pass 1 of the packed scan's staging: the item's lanes load node t's
// layer and hd_t, SU nodes per lane at a time (independent loads), then
// T of each node's layer, into entry t {-, -, T_t, offset} and entry t + 1
// {hd_t, ...}.
template <int SU>
__device__ __forceinline__ void stage_nodes(const TbArgs& a, float4* sp, const float* hds,
                                            const int* lay, int off, int nLr, int fl, int FP,
                                            int n) {
  for (int t0 = fl; t0 <= n; t0 += SU * FP) {
    int lv[SU];
    float hv[SU];
#pragma unroll
    for (int u = 0; u < SU; ++u) {
      const int t = t0 + u * FP;
      lv[u] = t <= n ? lay[t] : 0;
      hv[u] = t < n ? hds[t] : 0.f;
    }
#pragma unroll
    for (int u = 0; u < SU; ++u) {
      const int t = t0 + u * FP;
      if (t > n) break;
      const int l = off + wrap_layer(lv[u], nLr);
      sp[t].z = a.T32[l];
      sp[t].w = __int_as_float(l * a.nf);
      if (t < n) sp[t + 1].x = hv[u];
    }
  }
}

// The chunk's sums regrouped by node: sum_k (W_{k+1} + W_k) hd_k =
// sum_j W_j w_j, and likewise for T W, so a step adds W_{k+1} times two
// staged per-node weights.  The node sums run as float32 blocks of
// SCAN_FLUSH terms (all positive: <= 16 ulp each) added into Kahan sums.
// The optical depth is a float32 running sum th with its rounding errors
// collected (Fast2Sum) in tl, renormalised into (th, tl) once per block:
// exp(-tau) = exp(-th) (1 - tl) to O(tl^2).  Fast2Sum is exact while th >=
// the step's increment; a larger step errs by ~ulp of itself and at least
// doubles the sum, so those errors form a geometric series below ~2 ulp of
// the optical depth reached (the exponent's error; the adjoint, which
// subtracts back from a chunk's total, recomputes that total exactly).
//
// The 5-CTA bound (96 registers) lets the compiler keep 32 steps of alpha
// loads in flight without spilling: 64 rays x 256 frequencies through 1000
// layers 0.0292 ms unbounded (46 registers) / 0.0272 ms at 6 CTAs (80
// registers, spills) / 0.0272 ms at 5; a 256 x 256 image (31,405 rays on
// the disc) at 8 frequencies 0.52 / 0.43 / 0.39 ms.
__global__ void __launch_bounds__(128, 5) rb_tb_chunk2_kernel(TbArgs a) {
  const int npair = a.nf / 2;
  const int FP = a.lanes ? a.lanes : scan_lanes(npair);
  const int IPB = 128 / FP;
  const int sub = threadIdx.x / FP, fl = threadIdx.x % FP;
  const long long item = (long long)blockIdx.x * IPB + sub;
  const long long nitem = (long long)a.nb * a.nchunk;
  extern __shared__ __align__(16) float4 s_scan4[];
  int ray = 0, ch = 0, n = 0, i0 = 0;
  bool live = false;
  if (item < nitem) {
    // chunk-major: a CTA's items are one chunk index of consecutive rays, so
    // the chunks past the rays' ends gather in CTAs that exit at once
    ch = (int)(item / a.nb);
    ray = (int)(item % a.nb);
    const int nsteps = a.nseg[ray] - 1;
    i0 = ch * TB_CHUNK;
    live = i0 < nsteps;
    n = live ? min(TB_CHUNK, nsteps - i0) : 0;
  }
  const int f = 2 * (blockIdx.z * FP + fl);   // first of the pair
  // a chunk past the end of its ray writes nothing: the combine and the
  // adjoint read the partials of a ray's live chunks only
  float4* sp = s_scan4 + sub * SCAN_ITEM_F4;
  // Staging in two passes.  1 (stage_nodes): the item's lanes load node
  // t's layer, T and hd_t; with at most 8 lanes per item a lane's up to 17
  // nodes are loaded at once (the 256 x 256 image at 8 frequencies: 0.364
  // -> 0.337 ms), else
  // 4 at a time.  2: the node weights from the staged hd.
  if (live) {
    const float* hds = a.hds + (size_t)ray * a.max_seg + i0;
    const int* lay = a.layer + (size_t)ray * a.max_seg + i0;
    int off, nLr;
    ray_layers(a, ray, off, nLr);
    // few lanes per item (few frequencies): a lane's nodes at once
    if (FP <= 8) stage_nodes<17>(a, sp, hds, lay, off, nLr, fl, FP, n);
    else stage_nodes<4>(a, sp, hds, lay, off, nLr, fl, FP, n);
  }
  __syncthreads();
  if (live) {
    for (int t = fl; t <= n; t += FP) {
      const float hp = t > 0 ? sp[t].x : 0.f;
      const float hc = t < n ? sp[t + 1].x : 0.f;
      const float w = hp + hc, T = sp[t].z;
      sp[t].y = w;
      sp[t].z = T * w;
      if (t == 0) sp[0].x = T;
    }
  }
  __syncthreads();
  if (!live || f >= a.nf) return;
  const float* al = a.alpha32 + f;
  auto ld = [&](const float4& e) -> f2 {
    return *reinterpret_cast<const f2*>(al + __float_as_int(e.w));
  };
  // alpha row of node j read ahead: the offset alone, by its own shared
  // load, so the step's record is not kept in registers from the prefetch
  auto ld_ahead = [&](int j) -> f2 {
    int o;
    asm volatile("ld.shared.b32 %0, [%1];"
                 : "=r"(o)
                 : "r"((unsigned)__cvta_generic_to_shared(&sp[j].w)));
    return *reinterpret_cast<const f2*>(al + o);
  };
  const float4 e0 = sp[0];
  f2 a0 = ld(e0);
  // node 0: W_0 = 0 on a path's first chunk, exp(0) a_0 otherwise
  f2 iwb = 0ull, tbb = 0ull;
  if (i0 > 0) {
    iwb = mul2(a0, dup(e0.y));
    tbb = mul2(a0, dup(e0.z));
  }
  ScanPair st;
  st.init(a0, iwb, tbb);
  int i = 0;
  constexpr int BLK = 32;   // steps whose alpha loads are in flight together
  for (; i + BLK <= n; i += BLK) {
    f2 an[BLK];
#pragma unroll
    for (int k = 0; k < BLK; ++k) an[k] = ld_ahead(i + 1 + k);
#pragma unroll
    for (int k = 0; k < BLK; ++k) {
      st.step(an[k], sp[i + 1 + k]);
      if (k % SCAN_FLUSH == SCAN_FLUSH - 1) st.flush();
    }
  }
#pragma unroll 1
  for (int k = 0; i < n; ++i) {
    const float4 e = sp[i + 1];
    st.step(ld(e), e);
    if (++k == SCAN_FLUSH) {
      k = 0;
      st.flush();
    }
  }
  st.flush();
  const f2 IW = sub2(st.iw, st.iwc), TB = sub2(st.tb, st.tbc);
  const f2 tl = sub2(0ull, st.ntl);
  float4* part = a.part + ((size_t)ray * a.nchunk + ch) * a.nf;
  part[f] = make_float4(lo2(st.th), lo2(tl), lo2(IW), lo2(TB));
  part[f + 1] = make_float4(hi2(st.th), hi2(tl), hi2(IW), hi2(TB));
}

// Combine chunk partials of each (ray, frequency) into Tb.
__host__ __device__ __forceinline__ int combine_lanes(int nf) {
  int l = 8;
  while (l < nf && l < 128) l <<= 1;
  return l;
}

__global__ void __launch_bounds__(128) rb_tb_combine_kernel(TbArgs a) {
  const int FT = combine_lanes(a.nf);
  const int ray = blockIdx.x * (128 / FT) + threadIdx.x / FT;
  const int f = blockIdx.y * FT + threadIdx.x % FT;
  if (ray >= a.nb || f >= a.nf) return;
  float4* part = a.part + (size_t)ray * a.nchunk * a.nf + f;
  const int nsteps = a.nseg[ray] - 1;
  const int nc = nsteps > 0 ? (nsteps + TB_CHUNK - 1) / TB_CHUNK : 0;
  float ph = 0.f, pl = 0.f;          // optical depth at the chunk start
  float iw = 0.f, iwc = 0.f, tb = 0.f, tbc = 0.f;
  constexpr int CB = 8;              // partials loaded together
  for (int c0 = 0; c0 < nc; c0 += CB) {
    float4 pb[CB];
#pragma unroll
    for (int k = 0; k < CB; ++k)
      pb[k] = c0 + k < nc ? part[(size_t)(c0 + k) * a.nf] : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int k = 0; k < CB; ++k) {
      if (c0 + k >= nc) break;
      const float4 p = pb[k];
      if (a.iw32)   // the chunk's starting optical depth for the adjoint
        *reinterpret_cast<float2*>(&part[(size_t)(c0 + k) * a.nf].z) = make_float2(ph, pl);
      const float sc = __expf(-ph) * (1.f - pl);
      kahan_add(iw, iwc, sc * p.z);
      kahan_add(tb, tbc, sc * p.w);
      float s, e;
      two_sum(ph, p.x, s, e);
      e += pl + p.y;
      ph = s + e;
      pl = e - (ph - s);
    }
  }
  const float TbL = tb - tbc, IW = iw - iwc;
  const bool clamped = TbL < (float)T_CMB;   // off the planet or no emission: T_cmb exactly
  const float out = clamped ? (float)T_CMB : TbL / IW;
  a.Tb[(size_t)ray * a.nf + f] = clamped ? T_CMB : (double)out;
  if (a.Tb32) a.Tb32[(size_t)ray * a.nf + f] = out;
  if (a.intW) a.intW[(size_t)ray * a.nf + f] = (double)IW;
  if (a.iw32) a.iw32[(size_t)ray * a.nf + f] = clamped || !(IW > 0.f) ? 0.f : IW;
}

// Weighted sum over rays (disc quadrature): one warp per frequency, lane i
// takes rays i, i + 32, ... in float64 and the warp adds the lanes' sums.
// blockIdx.y = variant of a batch: rays [v nb, (v+1) nb), out[v][f].
__global__ void __launch_bounds__(128) rb_disc_avg_kernel(int nb, int nf, const float* Tb32,
                                                          const double* w, double* out) {
  const int f = blockIdx.x * 4 + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (f >= nf) return;
  Tb32 += (size_t)blockIdx.y * nb * nf;
  out += (size_t)blockIdx.y * nf;
  double s = 0.0;
  for (int r = lane; r < nb; r += 32) s += w[r] * (double)Tb32[(size_t)r * nf + f];
  for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) out[f] = s;
}

// Test hook: E1 (order 1) or E2 (order 2) of n arguments.
__global__ void rb_e2_kernel(int order, int n, const double* x, double* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = order == 1 ? expint1(x[i]) : expint2(x[i]);
}

int tb_nchunk(int max_seg) { return (max_seg + TB_CHUNK - 1) / TB_CHUNK; }

cudaError_t launch_tb_seq(const TbArgs& a, cudaStream_t st) {
  if (a.nb <= 0 || a.nf <= 0) return cudaSuccess;
  dim3 grid(a.nb, (a.nf + 127) / 128);
  rb_tb_seq_kernel<<<grid, 128, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_tb_chunked(const TbArgs& a, cudaStream_t st) {
  if (a.nb <= 0 || a.nf <= 0) return cudaSuccess;
  if (a.nf % 2 == 0) {
    const int FP = a.lanes ? a.lanes : scan_lanes(a.nf / 2);
    const long long nitem = (long long)a.nb * a.nchunk;
    const long long nblk = (nitem + 128 / FP - 1) / (128 / FP);
    dim3 grid((unsigned)nblk, 1, (a.nf / 2 + FP - 1) / FP);
    const size_t smem = sizeof(float4) * SCAN_ITEM_F4 * (128 / FP);
    rb_tb_chunk2_kernel<<<grid, 128, smem, st>>>(a);
  } else {
    dim3 grid(a.nb, a.nchunk, (a.nf + 127) / 128);
    rb_tb_chunk_kernel<<<grid, 128, 0, st>>>(a);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const int FT = combine_lanes(a.nf);
  dim3 g2((a.nb + 128 / FT - 1) / (128 / FT), (a.nf + FT - 1) / FT);
  rb_tb_combine_kernel<<<g2, 128, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_disc_avg(int nb, int nf, const float* Tb32, const double* w, double* out,
                            cudaStream_t st, int nvar) {
  rb_disc_avg_kernel<<<dim3((nf + 3) / 4, nvar), 128, 0, st>>>(nb, nf, Tb32, w, out);
  return cudaGetLastError();
}

cudaError_t launch_e2(int order, int n, const double* x, double* out, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  rb_e2_kernel<<<(n + 127) / 128, 128, 0, st>>>(order, n, x, out);
  return cudaGetLastError();
}

}  // namespace rb
