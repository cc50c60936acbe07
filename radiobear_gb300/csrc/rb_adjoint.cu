// Adjoint of the forward model: dTb/dT, dTb/dP and dTb/dln X (NH3, H2O,
// H2S) per layer, for the exp-weighted brightness of every ray (or their
// quadrature average).  The ray paths are held fixed (they depend on the
// layer radii and refractive indices, inputs of their own).
//
//   rb_tb_adj_lambda_kernel, rb_tb_adj_grad_kernel
//                           reverse sweep of the scan of Brightness.single
//                           (brightness.py:53-117), chunk-parallel like the
//                           forward scan, with
//                             dTb/dW_i  = c_i (T_i - Tb) / intW,
//                             dTb/da_k  = w_k E_k + d_{k-1}/2 Lam_k + d_k/2 Lam_{k+1},
//                             Lam_k     = sum_{i>=k} dTb/dW_i (-a_i E_i),
//                           (c_i the trapezoid node weight, E = exp(-tau));
//                           adds g dTb/dalpha and g W c / intW (the
//                           source-temperature term) per visited layer.
//   rb_layer_tan_kernel     eight parts per layer: the layer coefficients
//                           of the absorption (widths, couplings, strength
//                           prefactors, continua) in dual numbers, giving
//                           their derivatives with respect to the layer's
//                           T, P, ln X_NH3, ln X_H2O, ln X_H2S.
//   rb_alpha_jvp_kernel     one CTA per (layer, up to 128 frequencies): alpha is
//                           recomputed line by line together with its
//                           derivatives with respect to the five layer
//                           parameters (each family depends on T, P and its
//                           own abundance), contracted with dTb/dalpha of
//                           the layer and reduced over the frequencies.
//   rb_tb_adj_disc_kernel   the same reverse sweep for the b = 'disc'
//                           weighting W_i = 2 a_i E2(tau_i) (brightness.py:96):
//                           E_k -> 2 E2(tau_k) in the direct and source terms and
//                           a_k E_k -> 2 a_k E1(tau_k) in Lam (dE2/dx = -E1(x));
//                           E2 does not factor over chunks, so one thread per
//                           (ray, frequency) walks its whole path (forward pass
//                           storing tau and 2 E2 per node, then the reverse pass).
//   rb_adjoint_final_kernel adds the source-temperature term and writes
//                           dTb/dT, dTb/dP, dTb/dln X.
#include "rb_args.cuh"
#include "rb_assemble.cuh"
#include "rb_expint.cuh"
#include "rb_f32x2.cuh"
#include <math_constants.h>

namespace rb {

constexpr double T_CMB_ADJ = 2.725;   // utils.py:77
constexpr double LN2 = 0.69314718055994531;
constexpr double LOG2E_D = 1.4426950408889634;

__device__ __forceinline__ int wrap_l(int l, int nL) {
  l = l < 0 ? l + nL : l;
  return l < 0 ? 0 : (l >= nL ? nL - 1 : l);
}

// ------------------------------------------------------------------ scan adjoint
// The forward's chunk partials (rb_tb_chunk_kernel: per ray, chunk of
// ADJ_CHUNK segments and frequency, the chunk's optical depth as a
// double-float and its intW / TbL from a local optical depth of 0) give the
// optical depth at every chunk start and Tb; the reverse sweep then runs
// chunk by chunk in parallel:
//   rb_tb_adj_lambda_kernel  S_c = sum over the chunk's nodes of
//                            dTb/dtau_k = -w_k a_k E_k
//   rb_tb_adj_grad_kernel    Lam after the chunk = sum of S over later
//                            chunks, then the chunk's nodes in reverse.
constexpr int ADJ_CHUNK = SCAN_CHUNK;   // the forward scan's chunk

// Double-float running sum (a float pair) and compensated float sum.
__device__ __forceinline__ void dfs_add(float& h, float& l, float v) {
  float s, e;
  two_sum(h, v, s, e);
  e += l;
  h = s + e;
  l = e - (h - s);
}

// d loss / d Tb of ray b at frequency f.
__device__ __forceinline__ double adj_gb(const TbAdjArgs& a, int b, int f) {
  if (!a.weights) return a.grad[(size_t)b * a.nf + f];
  const int v = a.var_off ? b / a.rays_per_var : 0;
  const int bi = a.var_off ? b % a.rays_per_var : b;
  return a.weights[bi] * a.grad[(size_t)v * a.nf + f];
}

struct ChunkState {
  float tch, tcl;  // optical depth at this chunk's first node (double-float)
  float Tb, rIW;
  bool live;       // TbL >= T_cmb (else Tb is clamped and has no gradient)
};

// The state of chunk c of ray b at frequency f, written by the forward's
// combine (rb_tb_combine_kernel with iw32): the optical depth at the chunk's
// first node, Tb and intW of the ray (intW 0 where Tb is clamped to T_cmb,
// which has no gradient).
__device__ __forceinline__ ChunkState adj_state(const TbAdjArgs& a, int b, int c, int f) {
  ChunkState st;
  const float4* p = a.part + ((size_t)b * a.nchunk + c) * a.nf + f;
  const float2 t0 = *reinterpret_cast<const float2*>(&p->z);
  st.tch = t0.x;
  st.tcl = t0.y;
  const float iw = a.iw32[(size_t)b * a.nf + f];
  st.live = iw > 0.f;
  st.Tb = st.live ? a.Tb32[(size_t)b * a.nf + f] : (float)T_CMB_ADJ;
  st.rIW = st.live ? 1.f / iw : 0.f;
  return st;
}

// exp(-x) as 2^(-x log2(e)) with the PTX base-2 exponential approximation,
// flushing results below 2^-126 (optical depths above ~87) to zero.
__device__ __forceinline__ float exp_neg(float x) {
  float y = x * -1.4426950408889634f;
  asm("ex2.approx.ftz.f32 %0, %0;" : "+f"(y));
  return y;
}

// The chunk's path nodes staged in shared memory (layer offsets, T,
// half-lengths), so the loops' only global loads are the coalesced
// alpha[layer][f] rows.
struct AdjStage {
  int off[ADJ_CHUNK + 1];
  int lay[ADJ_CHUNK + 1];
  float T[ADJ_CHUNK + 1];
  float hd[ADJ_CHUNK + 1];
};

__device__ __forceinline__ void adj_stage(const TbAdjArgs& a, AdjStage& sg, int b, int i0, int ns,
                                          int N) {
  const float* hd = a.hds + (size_t)b * a.max_seg;
  const int* lay = a.layer + (size_t)b * a.max_seg;
  int off = 0, nLr = a.nL;
  if (a.var_off) {
    const int v = b / a.rays_per_var;
    off = a.var_off[v];
    nLr = a.var_off[v + 1] - off;
  }
  for (int t = threadIdx.x; t <= ns; t += blockDim.x) {
    const int L = off + wrap_l(lay[i0 + t], nLr);
    sg.lay[t] = L;
    sg.off[t] = L * a.nf;
    sg.T[t] = (float)a.T[L];
    sg.hd[t] = (i0 + t < N) ? hd[i0 + t] : 0.f;
  }
}

__global__ void __launch_bounds__(128) rb_tb_adj_lambda_kernel(TbAdjArgs a) {
  __shared__ AdjStage sg;
  const int f = blockIdx.z * blockDim.x + threadIdx.x;
  const int c = blockIdx.y, b = blockIdx.x;   // rays in x: batches have more than 65535
  const int n = min(max(a.nseg[b], 0), a.max_seg);
  const int N = n - 1;
  const int nc = N > 0 ? (N + ADJ_CHUNK - 1) / ADJ_CHUNK : 0;
  const int i0 = c * ADJ_CHUNK;
  if (c >= nc) {
    if (f < a.nf) a.S[((size_t)b * a.nchunk + c) * a.nf + f] = 0.f;
    return;
  }
  const int ns = min(ADJ_CHUNK, N - i0);
  adj_stage(a, sg, b, i0, ns, N);
  __syncthreads();
  if (f >= a.nf) return;
  float* S = a.S + ((size_t)b * a.nchunk + c) * a.nf + f;
  const ChunkState st = adj_state(a, b, c, f);
  if (!st.live) {
    *S = 0.f;
    return;
  }
  const float* al = a.alpha32 + f;
  float th = 0.f, tlo = 0.f, lam = 0.f, lamc = 0.f;
  float a0 = al[sg.off[0]];
  for (int s = 0; s < ns; ++s) {
    const float ak = al[sg.off[s + 1]];
    const float d = 2.f * sg.hd[s];
    dfs_add(th, tlo, (a0 + ak) * d * 0.5f);
    const float dk = 2.f * sg.hd[s + 1];
    const float ck = 0.5f * (d + dk);
    const float Ek = exp_neg(th) * (1.f - tlo);
    const float wk = ck * (sg.T[s + 1] - st.Tb) * st.rIW;
    const float y = -(wk * ak * Ek) - lamc;
    const float tt = lam + y;
    lamc = (tt - lam) - y;
    lam = tt;
    a0 = ak;
  }
  *S = exp_neg(st.tch) * (1.f - st.tcl) * (lam - lamc);
}

// In place: S[b][c][f] becomes the sum of S over the chunks after c
// (compensated, from the last chunk back), Lam after chunk c's last node.
__global__ void __launch_bounds__(128) rb_tb_adj_suffix_kernel(TbAdjArgs a) {
  const int b = blockIdx.x;
  const int f = blockIdx.y * blockDim.x + threadIdx.x;
  if (f >= a.nf) return;
  const int n = min(max(a.nseg[b], 0), a.max_seg);
  const int N = n - 1;
  const int nc = N > 0 ? (N + ADJ_CHUNK - 1) / ADJ_CHUNK : 0;
  float* S = a.S + (size_t)b * a.nchunk * a.nf + f;
  float ln = 0.f, lc = 0.f;
  for (int k = nc - 1; k >= 0; --k) {
    const float v = S[(size_t)k * a.nf];
    S[(size_t)k * a.nf] = ln - lc;
    const float y = v - lc;
    const float t = ln + y;
    lc = (t - ln) - y;
    ln = t;
  }
}

__global__ void __launch_bounds__(128) rb_tb_adj_grad_kernel(TbAdjArgs a) {
  __shared__ AdjStage sg;
  __shared__ float s_src[ADJ_CHUNK + 1][4];   // source term per node and warp
  const int f = blockIdx.z * blockDim.x + threadIdx.x;
  const int c = blockIdx.y, b = blockIdx.x;   // rays in x: batches have more than 65535
  const int n = min(max(a.nseg[b], 0), a.max_seg);
  const int N = n - 1;
  const int nc = N > 0 ? (N + ADJ_CHUNK - 1) / ADJ_CHUNK : 0;
  if (c >= nc) return;   // the whole CTA
  const int i0 = c * ADJ_CHUNK;
  const int ns = min(ADJ_CHUNK, N - i0);
  adj_stage(a, sg, b, i0, ns, N);
  for (int t = threadIdx.x; t < (ADJ_CHUNK + 1) * 4; t += blockDim.x) (&s_src[0][0])[t] = 0.f;
  __syncthreads();
  // lanes past nf or without a gradient run with g = 0 so the warp's
  // source-term shuffle has every lane
  const bool inf = f < a.nf;
  const int nf = a.nf;
  const int fc = inf ? f : 0;
  const int warp = threadIdx.x >> 5;
  double gb = inf ? adj_gb(a, b, fc) : 0.0;
  const ChunkState st = adj_state(a, b, c, fc);
  if (!st.live) gb = 0.0;
  const float g = (float)gb;
  if (!__all_sync(0xffffffffu, g == 0.f)) {
    // Lam after this chunk's last node: the suffix sum of the later chunks
    float Ln = a.S[((size_t)b * a.nchunk + c) * nf + fc], Lc = 0.f;
    const float* al = a.alpha32 + fc;
    // local optical depth at the chunk's last node, recomputed as an exact
    // double-float sum: the reverse recurrence subtracts from it down to the
    // chunk's first node, so it needs it to ~ulp^2 (the forward partial
    // carries ~ulp(tau) from steps larger than its running sum)
    float th = 0.f, tlo = 0.f;
    {
      float ap = al[sg.off[0]];
      for (int s = 0; s < ns; ++s) {
        const float aq = al[sg.off[s + 1]];
        dfs_add(th, tlo, (ap + aq) * (2.f * sg.hd[s]) * 0.5f);
        ap = aq;
      }
    }
    const float Ec = exp_neg(st.tch) * (1.f - st.tcl);
    // nodes i0+ns .. i0+1 in reverse (node i0 belongs to the previous chunk,
    // except node 0, which chunk 0 handles last); the sums over the rays and
    // the visits of a layer are atomic adds into galpha[layer][f], the
    // source term per node summed over the warp's frequencies, then over
    // the CTA's warps, into gsrc[layer]
    float ak = al[sg.off[ns]];
    for (int t = ns; t > 0; --t) {
      const float dprev = 2.f * sg.hd[t - 1];
      const float dcur = 2.f * sg.hd[t];
      const float ck = 0.5f * (dprev + dcur);
      const float Ek = Ec * exp_neg(th) * (1.f - tlo);
      const float wk = ck * (sg.T[t] - st.Tb) * st.rIW;
      const float Lnext = Ln - Lc;
      // Lam_k = Lam_{k+1} - w_k a_k E_k
      const float y = -(wk * ak * Ek) - Lc;
      const float tt = Ln + y;
      Lc = (tt - Ln) - y;
      Ln = tt;
      const float Lk = Ln - Lc;
      if (g != 0.f) atomicAdd(a.ga + sg.off[t] + f, g * (wk * Ek + 0.5f * dprev * Lk + 0.5f * dcur * Lnext));
      float src = g * ak * Ek * ck * st.rIW;
      for (int o = 16; o; o >>= 1) src += __shfl_xor_sync(0xffffffffu, src, o);
      if ((threadIdx.x & 31) == 0) s_src[t][warp] = src;
      const float am = al[sg.off[t - 1]];
      dfs_add(th, tlo, -(am + ak) * dprev * 0.5f);
      ak = am;
    }
    if (c == 0 && g != 0.f)   // node 0: W_0 = 0, only the segment term
      atomicAdd(a.ga + sg.off[0] + f, g * 0.5f * (2.f * sg.hd[0]) * (Ln - Lc));
  }
  __syncthreads();
  const int nwarp = (blockDim.x + 31) >> 5;
  for (int t = threadIdx.x + 1; t <= ns; t += blockDim.x) {
    float v = 0.f;
    for (int w = 0; w < nwarp; ++w) v += s_src[t][w];
    if (v != 0.f) atomicAdd(a.gs + sg.lay[t], (double)v);
  }
}

// b = 'disc': one thread per (ray, frequency).  The forward pass repeats
// the sequential scan's arithmetic (rb_tb_seq_kernel with the E2 weighting,
// so Tb and intW are the forward's), storing {tau_k, 2 E2(tau_k)} per node;
// the reverse pass accumulates Lam_k = Lam_{k+1} - w_k 2 a_k E1(tau_k) and
// adds g (w_k 2 E2_k + hd_{k-1} Lam_k + hd_k Lam_{k+1}) into galpha and
// g W_k c_k / intW into the source term (hd = ds / 2, the node weight
// c_k = hd_{k-1} + hd_k).  Threads past nf run with g = 0 so the warp's
// source-term shuffle has every lane.
__global__ void __launch_bounds__(128) rb_tb_adj_disc_kernel(TbAdjArgs a) {
  const int b = blockIdx.x;
  const int f = blockIdx.y * blockDim.x + threadIdx.x;
  const bool inf = f < a.nf;
  const int fc = inf ? f : 0;
  const int n = min(max(a.nseg[b], 0), a.max_seg);
  if (n < 2) return;                          // no path: Tb = T_cmb, no gradient (warp-uniform)
  const float* hd = a.hds + (size_t)b * a.max_seg;
  const int* lay = a.layer + (size_t)b * a.max_seg;
  int off = 0, nLr = a.nL;
  if (a.var_off) {
    const int v = b / a.rays_per_var;
    off = a.var_off[v];
    nLr = a.var_off[v + 1] - off;
  }
  double2* tE = a.tauE + (size_t)b * a.max_seg * a.nf + fc;
  const float* al = a.alpha32 + fc;
  // forward pass (rb_tb_seq_kernel's arithmetic)
  float th = 0.f, tl = 0.f, W0 = 0.f;
  float iw = 0.f, iwc = 0.f, tb = 0.f, tbc = 0.f;
  int L0 = off + wrap_l(lay[0], nLr);
  float T0 = (float)a.T[L0];
  float a0 = al[(size_t)L0 * a.nf];
  if (inf) tE[0] = make_double2(0.0, 0.0);
  for (int i = 0; i + 1 < n; ++i) {
    const int L1 = off + wrap_l(lay[i + 1], nLr);
    const float h = hd[i];
    const float a1 = al[(size_t)L1 * a.nf];
    const float T1 = (float)a.T[L1];
    dfs_add(th, tl, (a0 + a1) * h);
    const double tau = (double)th + (double)tl;
    const double e2 = 2.0 * expint2(tau);
    const float W1 = (float)((double)a1 * e2);
    float y = (W1 + W0) * h - iwc, t = iw + y;
    iwc = (t - iw) - y;
    iw = t;
    y = fmaf(T1, W1, T0 * W0) * h - tbc;
    t = tb + y;
    tbc = (t - tb) - y;
    tb = t;
    if (inf) tE[(size_t)(i + 1) * a.nf] = make_double2(tau, e2);
    W0 = W1;
    T0 = T1;
    a0 = a1;
  }
  const double TbL = (double)tb - (double)tbc, IW = (double)iw - (double)iwc;
  const bool live = !(TbL < T_CMB_ADJ) && IW > 0.0;
  double gb = (inf && live) ? adj_gb(a, b, fc) : 0.0;
  if (__all_sync(0xffffffffu, gb == 0.0)) return;
  const float Tb = live ? (float)(TbL / IW) : 0.f;
  const float rIW = live ? (float)(1.0 / IW) : 0.f;
  const float g = (float)gb;
  // reverse pass: nodes n-1 .. 1, then node 0 (W_0 = 0: segment term only)
  float Ln = 0.f, Lc = 0.f;                   // Lam_{k+1}, compensated
  for (int k = n - 1; k > 0; --k) {
    const int L = off + wrap_l(lay[k], nLr);
    const float hprev = hd[k - 1];
    const float hcur = k + 1 < n ? hd[k] : 0.f;   // the last ds is not used
    const float ck = hprev + hcur;
    const double2 te = inf ? tE[(size_t)k * a.nf] : make_double2(1.0, 0.0);
    const float ak = al[(size_t)L * a.nf];
    const float wk = ck * ((float)a.T[L] - Tb) * rIW;
    const float Lnext = Ln - Lc;
    const float e1 = g != 0.f ? (float)(2.0 * expint1(te.x)) : 0.f;
    const float yv = -(wk * ak * e1) - Lc;
    const float tt = Ln + yv;
    Lc = (tt - Ln) - yv;
    Ln = tt;
    const float Lk = Ln - Lc;
    if (g != 0.f)
      atomicAdd(a.ga + (size_t)L * a.nf + f, g * (wk * (float)te.y + hprev * Lk + hcur * Lnext));
    float src = g * ak * (float)te.y * ck * rIW;
    for (int o = 16; o; o >>= 1) src += __shfl_xor_sync(0xffffffffu, src, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(a.gs + L, (double)src);
  }
  if (g != 0.f) atomicAdd(a.ga + (size_t)L0 * a.nf + f, g * hd[0] * (Ln - Lc));
}

// ------------------------------------------------------------------ dual numbers
// Value and derivatives with respect to the five layer parameters
// (T, P, ln X_NH3, ln X_H2O, ln X_H2S), float32 (the derivatives feed a
// gradient, not the forward values).
struct D5 {
  float v, d[NTH];
};

__device__ __forceinline__ D5 dc(float v) {
  D5 r;
  r.v = v;
  for (int k = 0; k < NTH; ++k) r.d[k] = 0.f;
  return r;
}
__device__ __forceinline__ D5 operator+(const D5& a, const D5& b) {
  D5 r;
  r.v = a.v + b.v;
  for (int k = 0; k < NTH; ++k) r.d[k] = a.d[k] + b.d[k];
  return r;
}
__device__ __forceinline__ D5 operator-(const D5& a, const D5& b) {
  D5 r;
  r.v = a.v - b.v;
  for (int k = 0; k < NTH; ++k) r.d[k] = a.d[k] - b.d[k];
  return r;
}
__device__ __forceinline__ D5 operator*(const D5& a, const D5& b) {
  D5 r;
  r.v = a.v * b.v;
  for (int k = 0; k < NTH; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
  return r;
}
__device__ __forceinline__ D5 operator/(const D5& a, const D5& b) {
  D5 r;
  r.v = a.v / b.v;
  for (int k = 0; k < NTH; ++k) r.d[k] = (a.d[k] - r.v * b.d[k]) / b.v;
  return r;
}
__device__ __forceinline__ D5 operator*(float s, const D5& a) {
  D5 r;
  r.v = s * a.v;
  for (int k = 0; k < NTH; ++k) r.d[k] = s * a.d[k];
  return r;
}
__device__ __forceinline__ D5 operator+(const D5& a, float s) {
  D5 r = a;
  r.v += s;
  return r;
}
__device__ __forceinline__ D5 chain(const D5& a, float fv, float dfdx) {
  D5 r;
  r.v = fv;
  for (int k = 0; k < NTH; ++k) r.d[k] = dfdx * a.d[k];
  return r;
}
__device__ __forceinline__ D5 dlog2(const D5& a) { return chain(a, log2f(a.v), (float)LOG2E_D / a.v); }
__device__ __forceinline__ D5 dexp2(const D5& a) {
  const float e = exp2f(a.v);
  return chain(a, e, (float)LN2 * e);
}
__device__ __forceinline__ D5 dexp(const D5& a) {
  const float e = expf(a.v);
  return chain(a, e, e);
}
// 2^(e lg2x), the prep kernel's pw()
__device__ __forceinline__ D5 dpw(const D5& lg2x, float e) { return dexp2(e * lg2x); }
__device__ __forceinline__ D5 dmin1(const D5& a) { return a.v < 1.f ? a : dc(1.f); }

__device__ __forceinline__ void store_tan(FamTan& o, int s, int k, const D5& v) {
  for (int q = 0; q < NTH; ++q) o.dc[s][k][q] = (float)v.d[q];
}
__device__ __forceinline__ void store_pref(FamTan& o, const D5& pref) {
  for (int q = 0; q < NTH; ++q) o.dlnpref[q] = pref.v != 0.f ? pref.d[q] / pref.v : 0.f;
}
__device__ __forceinline__ void zero_tan(FamTan& o) {
  for (int s = 0; s < 2; ++s)
    for (int k = 0; k < 8; ++k)
      for (int q = 0; q < NTH; ++q) o.dc[s][k][q] = 0.f;
  for (int q = 0; q < NTH; ++q) o.dlnpref[q] = 0.f;
  o.dcE = 0.f;
}

// Inversion coefficient tables [inv_table][set] (nh3_hs.py:139-168,
// nh3_dbs.py:133-162), as in the prep kernel.
__device__ constexpr float INV_SET_D[2][2][13] = {
    {{1.640, 0.75, 0.852, 0.7756, 0.666, 1.0, 1.262, 0.3, 0.5296, 0.7964, 0.667, 1.554, -0.0498},
     {1.7465, 0.9779, 0.7298, 0.8202, 1.0, 1.0, 1.2163, 0.0291, 0.5152, 0.8873, 0.8994, 0.66666667,
      -0.0627}},
    {{1.6937, 0.6997, 0.7523, 0.8085, 1.0, 1.0, 1.3263, 0.1607, 0.6162, 0.8199, 0.0, 1.3832, -0.0139},
     {1.7465, 0.9779, 0.7298, 0.8202, 1.0, 1.0, 1.2163, 0.0291, 0.5152, 0.8873, 0.8994, 0.66666667,
      -0.0627}}};

// Derivatives of the layer coefficients, eight parts per layer (those of
// rb_layer_prep_kernel: 0 shared, 1 inversion, 2 rotational, 3 nu2,
// 4 nh3_sjs, 5 H2S, 6 PH3, 7 H2O), threads numbered part-major over the
// layers padded to a multiple of 32 (one part per warp).
constexpr int FAMTAN_WORDS = (int)(sizeof(FamTan) / sizeof(float));

__global__ void __launch_bounds__(64) rb_layer_tan_kernel(TanArgs a) {
  // a warp's 32 FamTan, written out layer by layer with consecutive lanes
  // (a thread's own 344-byte struct, 2.4 KB from its neighbours', turned
  // every 4-byte store into its own sector request)
  __shared__ float s_tan[2][32][FAMTAN_WORDS];
  const int gid = blockIdx.x * blockDim.x + threadIdx.x;
  const int nLp = (a.nL + 31) & ~31;
  const int part = gid / nLp, Lg = gid - part * nLp;
  if (part >= 8) return;   // whole warps: nLp is a multiple of 32
  const bool valid = Lg < a.nL;
  const int L = valid ? Lg : a.nL - 1;   // lanes past nL evaluate the last layer, store nothing
  const int nL = a.nL;
  const double Pd = a.P[L], Td = a.T[L];
  const double* X = a.X;
  D5 T = dc(Td), P = dc(Pd);
  T.d[0] = 1.0;
  P.d[1] = 1.0;
  auto pp = [&](int row, int th) {   // partial pressure P X, d/dln X on tangent th
    const double x = X[row * nL + L];
    D5 r = x * P;
    if (th >= 0) r.d[th] = Pd * x;
    return r;
  };
  const D5 Ph2 = pp(X_H2, -1), Phe = pp(X_HE, -1), Pch4 = pp(X_CH4, -1);
  const D5 Pnh3 = pp(X_NH3, TH_XNH3), Ph2o = pp(X_H2O, TH_XH2O), Ph2s = pp(X_H2S, TH_XH2S);
  const D5 Pph3 = pp(X_PH3, -1);
  LayerTan& o = a.out[L];
  const D5 Tdiv = dc(300.0) / T;
  const D5 lTdiv = dlog2(Tdiv);
  const D5 l295 = dlog2(dc(295.0) / T);
  const double GHZ = 29.9792458, TWO_PI = 0.63661977236758134, FOUR_PI = 1.2732395447351627;
  const double HS = 1.0E6 * 6.02297E23 / 8.31432E7;
  const D5 hs_base = HS * GHZ * ((1.0 / 300.0) * Pnh3 * dpw(lTdiv, 3.5));
  const double invT2 = 1.0 / (Td * Td);
  FamTan F;
  zero_tan(F);
  int famo = FAM_H2O;
  switch (part) {
    case 0: {
      // blend weight of nh3_hs_sjs (nh3_hs_sjs.py:6-26)
      if (valid)
        o.dblendW_dP = (a.nh3_mode == NH3_HS_SJS && Pd >= 400.0 && Pd <= 2000.0) ? (float)(1.0 / 1600.0) : 0.f;
      const D5 th = dc(273.0) / T;
      const D5 lth = dlog2(th);
      D5 pre;
      if (a.h2state == 'n') {
        pre = dmin1(dpw(dlog2(T / dc(40.0)), 2.5));
      } else {
        pre = dmin1(dpw(dlog2(T / dc(55.0)), 2.7));
        pre = dmin1(pre * dpw(dlog2(T / dc(120.0)), 0.55));
      }
      const D5 cia = 3.9522E-14 * (Ph2 * pre *
                                   (Ph2 * dpw(lth, 3.12) + 1.382 * (Phe * dpw(lth, 2.24)) +
                                    9.322 * (Pch4 * dpw(lth, 3.34))));
      if (valid)
        for (int q = 0; q < NTH; ++q) o.dh2_cia[q] = (float)cia.d[q];
      return;   // the whole warp: no FamTan in part 0
    }
    case 1: {
      for (int s = 0; s < 2; ++s) {
        const float* c = INV_SET_D[a.inv_table][s];
        store_tan(F, s, 0, c[0] * (Ph2 * dpw(lTdiv, c[3])) + c[1] * (Phe * dpw(lTdiv, c[4])));
        store_tan(F, s, 1, c[2] * (Pnh3 * dpw(l295, c[5])));
        store_tan(F, s, 3, c[6] * (Ph2 * dpw(lTdiv, c[9])) + c[7] * (Phe * dpw(lTdiv, c[10])));
        store_tan(F, s, 4, c[8] * (Pnh3 * dpw(l295, c[11])));
      }
      store_pref(F, TWO_PI * hs_base);
      F.dcE = (float)(19.858252418E-24 / 1.38E-23 * LOG2E_D * invT2);
      famo = FAM_NH3_INV;
      break;
    }
    case 2: {
      store_tan(F, 0, 1, 0.2984 * (Ph2 * dpw(lTdiv, 0.8730)));
      store_tan(F, 0, 2, 0.75 * (Phe * dpw(lTdiv, 0.66666667)));
      store_tan(F, 0, 3, 3.1789 * (Pnh3 * Tdiv));
      store_pref(F, (2.4268 * FOUR_PI) * hs_base);
      F.dcE = (float)(19.858252418E-24 / 1.38E-23 * LOG2E_D * invT2);
      famo = FAM_NH3_ROT;
      break;
    }
    case 3: {
      store_tan(F, 0, 1, Ph2 * dpw(lTdiv, 0.73));
      store_tan(F, 0, 2, Phe * dpw(lTdiv, 0.5716));
      store_tan(F, 0, 3, Pnh3 * Tdiv);
      store_pref(F, (1.1206 * FOUR_PI) * hs_base);
      F.dcE = (float)(19.858252418E-24 / 1.38E-23 * LOG2E_D * invT2);
      famo = FAM_NH3_V2;
      break;
    }
    case 4: {
      if (valid)
        for (int s = 0; s < 2; ++s)
          for (int k = 0; k < 5; ++k)
            for (int q = 0; q < NTH; ++q) o.dsjs[s][k][q] = 0.f;
      const bool use_sjs = a.nh3_mode == NH3_SJS || (a.nh3_mode == NH3_HS_SJS && Pd >= 400.0);
      if (use_sjs) {
        const D5 rexp = 8.79 * dexp((-1.0 / 83.0) * T);
        const D5 base = dexp(dc(9.024) - (1.0 / 20.3) * T) + (-0.9918) + Ph2;
        const D5 GH2a = dexp2(rexp * dlog2(base));
        const double J[7] = {1.690, 0.750, 0.6, 1.350, 0.300, 0.200, -0.45};
        D5 S[7];
        if (GH2a.v < 1e-12) {
          for (int k = 0; k < 7; ++k) S[k] = dc(J[k]);
        } else {
          const D5 g = 2.34 * (dc(1.0) - 2.122 * (dexp((-1.0 / 116.8) * T) / GH2a));
          S[0] = g;
          S[1] = dc(0.46) + (1.0 / 3000.0) * T;
          S[2] = dc(0.74);
          S[3] = dc(5.7465) + g * (dc(-7.7644) + g * (dc(9.1931) + g * (dc(-5.6816) + 1.2307 * g)));
          S[4] = dc(0.28) - (1.0 / 1750.0) * T;
          S[5] = dc(0.50);
          S[6] = dc(-0.45);
        }
        const D5 l296 = dlog2(dc(296.0) / T);
        const D5 tt = dpw(l296, 2.0 / 3.0);
        for (int s = 0; s < 2; ++s) {
          D5 c[7];
          for (int k = 0; k < 7; ++k) c[k] = s == 0 ? dc(J[k]) : S[k];
          const D5 v[5] = {tt * (c[0] * Ph2 + c[1] * Phe), tt * (c[2] * Pnh3),
                           tt * (c[3] * Ph2 + c[4] * Phe), tt * (c[5] * Pnh3), c[6] * Pnh3};
          if (valid)
            for (int k = 0; k < 5; ++k)
              for (int q = 0; q < NTH; ++q) o.dsjs[s][k][q] = (float)v[k].d[q];
        }
        const D5 Pscale = dc(1.0) + 1.0E-5 * P;
        store_pref(F, (7.244E+21 * GHZ * TWO_PI / 296.0) * (Pnh3 * dpw(l296, 3.5) * Pscale));
        F.dcE = (float)(1.438396 * LOG2E_D * invT2);
      }
      famo = FAM_NH3_SJS;
      break;
    }
    case 5: {
      const D5 l296 = dlog2(dc(296.0) / T);
      const D5 t7 = dpw(l296, 0.7);
      store_tan(F, 0, 0, t7 * (1.960 * Ph2 + 1.200 * Phe));
      store_tan(F, 0, 1, t7 * Ph2s);
      store_tan(F, 0, 7, 1.28 * Ph2s);
      store_pref(F, (7.244E+21 * GHZ * TWO_PI / 296.0) * (Ph2s * dpw(l296, 3.5)));
      F.dcE = (float)(1.438396 * LOG2E_D * invT2);
      famo = FAM_H2S;
      break;
    }
    case 6: {
      store_tan(F, 0, 1, dpw(lTdiv, 2.0 / 3.0) * (3.2930 * Ph2 + 1.6803 * Phe));
      store_tan(F, 0, 2, 4.2157 * (Tdiv * Pph3));
      store_pref(F, (7.244E+21 * GHZ * TWO_PI / 300.0) * (Pph3 * dpw(lTdiv, 3.5)));
      F.dcE = (float)(1.438396 * LOG2E_D * invT2);
      famo = FAM_PH3;
      break;
    }
    default: {
      store_tan(F, 0, 0, lTdiv);
      store_tan(F, 0, 1, Ph2o);
      store_tan(F, 0, 2, Ph2);
      store_tan(F, 0, 3, Phe);
      const D5 density = (0.997317 * 6.0221415e17 / 8.314472e-5) * (Ph2o / T);
      store_pref(F, (4.342945e-4 / 434294.5) * (density * dpw(lTdiv, 2.5)));
      F.dcE = (float)(300.0 * LOG2E_D * invT2);
      famo = FAM_H2O;
      const double Cf_he = 1.0e6 * 1.03562010226e-10, Cf_h2 = 1.0e6 * 5.07722009423e-11;
      const D5 th3 = Tdiv * Tdiv * Tdiv;
      const D5 foreign = Cf_he * (Phe * Ph2o * th3) + Cf_h2 * (Ph2 * Ph2o * th3);
      const D5 selfc = 3.1e-07 * (dpw(lTdiv, 12.0) * (1.0e6 * (Ph2o * Ph2o)));
      const D5 cont = (4.342945 / 434294.5) * (foreign + selfc);
      if (valid)
        for (int q = 0; q < NTH; ++q) o.dh2o_cont[q] = (float)cont.d[q];
      break;
    }
  }
  // famo is the same on every lane of the warp (one part per warp)
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const float* src = reinterpret_cast<const float*>(&F);
  for (int k = 0; k < FAMTAN_WORDS; ++k) s_tan[w][lane][k] = src[k];
  __syncwarp();
  const int L0 = Lg - lane;
  for (int j = 0; j < 32 && L0 + j < nL; ++j) {
    float* dst = reinterpret_cast<float*>(&a.out[L0 + j].fam[famo]);
    for (int k = lane; k < FAMTAN_WORDS; k += 32) dst[k] = s_tan[w][j][k];
  }
}

// ------------------------------------------------------------------ alpha JVP
// Records of one line, float: value fields and derivatives along the
// family's three tangents (T, P, ln X of its own gas).
// Lines per record chunk: 128 for 256-thread CTAs, 64 for 128-thread CTAs
// (half the shared memory, so 5 CTAs fit per SM; 4096 atmospheres of
// 300-1200 layers at 128 frequencies: 371 -> 358 ms).
constexpr int JV_CHUNK = 128;
constexpr int JV_NREC = 16;

constexpr int JV_FTMAX = 128;   // frequencies per CTA at most

// Line pairs: field f of lines (2p, 2p+1) is one f32x2 (first line in the
// low half); two fields per 16-byte word, JV_NU2 words per pair.
constexpr int JV_NU2 = 9;

template <int CH>
struct JvpShared {
  static constexpr int PAIRS = CH / 2;
  ulonglong2 rec[2][2][CH / 2][JV_NU2];     // [buffer][coefficient set][pair][word], 144 B per pair
  float fam[NFAM][JV_FTMAX][4];             // per family and frequency: value, three derivatives
  float2 red[8][NTH + 1];
};

// Line kinds of the JVP sweep.
enum JvKind : int { JK_BR = 0, JK_GROSS = 1, JK_VVW = 2, JK_SJS = 3 };

// Compensated float sum.
struct KSum {
  float s, c;
  __device__ __forceinline__ void init() { s = c = 0.f; }
  __device__ __forceinline__ void add(float v) {
    const float y = v - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
  }
  __device__ __forceinline__ float val() const { return s - c; }
};

// Family tangent slots: T, P and the family's own abundance.
__device__ __forceinline__ int fam_xtan(int fam) {
  switch (fam) {
    case FAM_H2O: return TH_XH2O;
    case FAM_H2S: return TH_XH2S;
    case FAM_PH3: return -1;
    default: return TH_XNH3;
  }
}

__device__ __forceinline__ float tan3(const float* d5, int q, int xt) {
  return q == 0 ? d5[TH_T] : (q == 1 ? d5[TH_P] : (xt >= 0 ? d5[xt] : 0.f));
}

__device__ __forceinline__ float strength(const LineTable& t, const LayerFam& F, int li) {
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

// Ben-Reuven record, fields: 0 g, 1 z, 2 KH, 3 KL, 4 S, 5 dlnS/dT,
// 6..8 dg, 9..11 dz, 12..14 dK.
__device__ __forceinline__ void jv_br_record(const LineTable& t, const LayerFam& LF, const FamTan& FT, int set,
                             int li, int xt, float* r, int stride) {
  const float* c = LF.c[set];
  const float w1 = t.w1[li], w2 = t.w2[li];
  const float g = c[0] + c[1] * w1 + c[2] * w2;
  const float z = c[3] + c[4] * w1 + c[5] * g;
  const float d = c[6] * g + c[7];
  const float fo = t.ch[li];
  float KH, e;
  two_sum(t.c2h[li], fmaf(2.f * fo + d, d, (g - z) * (g + z)), KH, e);
  const float KL = e + t.c2l[li];
  r[0 * stride] = g;
  r[1 * stride] = z;
  r[2 * stride] = KH;
  r[3 * stride] = KL;
  r[4 * stride] = strength(t, LF, li);
  r[5 * stride] = (float)LN2 * (t.Eh[li] + t.El[li]) * FT.dcE;
  for (int q = 0; q < 3; ++q) {
    auto dcq = [&](int k) { return tan3(FT.dc[set][k], q, xt); };
    const float dg = dcq(0) + dcq(1) * w1 + dcq(2) * w2;
    const float dz = dcq(3) + dcq(4) * w1 + dcq(5) * g + c[5] * dg;
    const float dd = dcq(6) * g + c[6] * dg + dcq(7);
    r[(6 + q) * stride] = dg;
    r[(9 + q) * stride] = dz;
    r[(12 + q) * stride] = 2.f * (fo + d) * dd + 2.f * g * dg - 2.f * z * dz;
  }
}

// Gross record: 0 g, 2 KH, 3 KL, 4 S, 5 dlnS/dT, 6..8 dg.
__device__ __forceinline__ void jv_gross_record(const LineTable& t, const LayerFam& LF, const FamTan& FT, int li,
                                int xt, float* r, int stride) {
  const float g = LF.c[0][1] * t.w1[li] + LF.c[0][2] * t.w2[li] + LF.c[0][3] * t.w3[li];
  r[0 * stride] = g;
  r[2 * stride] = t.c2h[li];
  r[3 * stride] = t.c2l[li];
  r[4 * stride] = strength(t, LF, li);
  r[5 * stride] = (float)LN2 * (t.Eh[li] + t.El[li]) * FT.dcE;
  for (int q = 0; q < 3; ++q)
    r[(6 + q) * stride] = tan3(FT.dc[0][1], q, xt) * t.w1[li] + tan3(FT.dc[0][2], q, xt) * t.w2[li] +
                          tan3(FT.dc[0][3], q, xt) * t.w3[li];
}

// VVW record: 0 df, 2 fo_hi, 3 fo_lo, 4 S, 5 dlnS/dT, 6..8 d(df).
__device__ __forceinline__ void jv_vvw_record(const LineTable& t, const LayerFam& LF, const FamTan& FT, int li,
                              int xt, float* r, int stride, float* base, float* dbase) {
  const float l2T = LF.c[0][0];
  const float e1 = exp2f(t.x1[li] * l2T), e2 = exp2f(t.x2[li] * l2T), e3 = exp2f(t.x3[li] * l2T);
  const float df = LF.c[0][1] * t.w1[li] * e1 + LF.c[0][2] * t.w2[li] * e2 + LF.c[0][3] * t.w3[li] * e3;
  const float S = strength(t, LF, li);
  const float dlnS = (float)LN2 * (t.Eh[li] + t.El[li]) * FT.dcE;
  r[0 * stride] = df;
  r[2 * stride] = t.ch[li];
  r[3 * stride] = t.cl[li];
  r[4 * stride] = S;
  r[5 * stride] = dlnS;
  const float h = S * df, den = 562500.f + df * df;
  *base += 2.f * h / den;
  for (int q = 0; q < 3; ++q) {
    const float dl2T = tan3(FT.dc[0][0], q, xt);
    const float ddf = tan3(FT.dc[0][1], q, xt) * t.w1[li] * e1 + tan3(FT.dc[0][2], q, xt) * t.w2[li] * e2 +
                      tan3(FT.dc[0][3], q, xt) * t.w3[li] * e3 +
                      (float)LN2 * dl2T *
                          (LF.c[0][1] * t.w1[li] * e1 * t.x1[li] + LF.c[0][2] * t.w2[li] * e2 * t.x2[li] +
                           LF.c[0][3] * t.w3[li] * e3 * t.x3[li]);
    r[(6 + q) * stride] = ddf;
    const float dh = (q == 0 ? h * dlnS : 0.f) + S * ddf;
    dbase[q] += 2.f * dh / den - 2.f * h * 2.f * df * ddf / (den * den);
  }
}

// nh3_sjs record: 2 KH0, 3 KL0 ((fo + shift)^2), 4 S, 5 dlnS/dT, 6 G0, 9..11 dK0.
__device__ __forceinline__ void jv_sjs_record(const LineTable& t, const LayerFam& LF, const FamTan& FT,
                              const LayerTan& LT, float shift, int li, float* r, int stride) {
  const float fo = t.ch[li];
  float KH, e;
  two_sum(t.c2h[li], (2.f * fo + shift) * shift, KH, e);
  r[2 * stride] = KH;
  r[3 * stride] = e + t.c2l[li];
  r[4 * stride] = strength(t, LF, li);
  r[5 * stride] = (float)LN2 * (t.Eh[li] + t.El[li]) * FT.dcE;
  r[6 * stride] = t.w1[li];
  for (int q = 0; q < 3; ++q) r[(9 + q) * stride] = 2.f * (fo + shift) * tan3(LT.dsjs[0][4], q, TH_XNH3);
}

// Fields of one line in the pair records, by line kind (f32x2 packing of
// two lines; the sweep reads words 0..nw-1 of a pair):
//   Ben-Reuven  0 g  1 g+z  2 g-z  3 K  4 -K_hi  5 -K_lo  6 S  7 dlnS/dT  8 4g^2
//               9..11 dg  12..14 dz  15..17 dK                       (9 words)
//   Gross       0 g  1 4g^2  2 S  3 dlnS/dT  4 -K_hi  5 -K_lo  6..8 dg  (5 words)
//   VVW         0 df  1 df^2  2 -fo_hi  3 -fo_lo  4 S  5 dlnS/dT  6..8 d(df)  (5 words)
//   nh3_sjs     0 K0_hi  1 K0_lo  2 S  3 dlnS/dT  4 G0  5..7 dK0      (4 words)
// (K = (fo + delta)^2 + g^2 - z^2, exact as a double-float; nh3_sjs: K0 =
// (fo + shift)^2, g, z and K per frequency in the sweep.)  A padding line
// (odd line count) has S = 0 and zero derivatives, so it adds exactly 0.
constexpr int JV_NF = 18;

// Padding line: zero strength and derivatives, a finite positive denominator.
template <int KIND>
__device__ __forceinline__ void jv_pad_fields(float* v) {
  for (int k = 0; k < JV_NF; ++k) v[k] = 0.f;
  if (KIND == JK_BR) {          // g = g+z = g-z = K = 1, 4g^2 = 4
    v[0] = 1.f; v[1] = 1.f; v[2] = 1.f; v[3] = 1.f; v[4] = -1.f; v[8] = 4.f;
  } else if (KIND == JK_GROSS) {   // g = 1, 4g^2 = 4, K = 1
    v[0] = 1.f; v[1] = 4.f; v[4] = -1.f;
  } else if (KIND == JK_VVW) {  // df = df^2 = 1
    v[0] = 1.f; v[1] = 1.f;
  } else {                      // K0 = 1e18: the denominator ~1e36
    v[0] = 1e18f;
  }
}

__device__ __forceinline__ void jv_br_fields(const LineTable& t, const LayerFam& LF, const FamTan& FT,
                                             int set, int li, int xt, float* v) {
  float r[JV_NREC];
  jv_br_record(t, LF, FT, set, li, xt, r, 1);   // 0 g, 1 z, 2 KH, 3 KL, 4 S, 5 dlnS, 6.. dg dz dK
  const float g = r[0], z = r[1];
  v[0] = g;
  v[1] = g + z;
  v[2] = g - z;
  v[3] = r[2] + r[3];
  v[4] = -r[2];
  v[5] = -r[3];
  v[6] = r[4];
  v[7] = r[5];
  v[8] = 4.f * g * g;
  for (int k = 0; k < 9; ++k) v[9 + k] = r[6 + k];
}

__device__ __forceinline__ void jv_gross_fields(const LineTable& t, const LayerFam& LF, const FamTan& FT,
                                                int li, int xt, float* v) {
  float r[JV_NREC];
  jv_gross_record(t, LF, FT, li, xt, r, 1);     // 0 g, 2 KH, 3 KL, 4 S, 5 dlnS, 6..8 dg
  v[0] = r[0];
  v[1] = 4.f * r[0] * r[0];
  v[2] = r[4];
  v[3] = r[5];
  v[4] = -r[2];
  v[5] = -r[3];
  v[6] = r[6];
  v[7] = r[7];
  v[8] = r[8];
}

__device__ __forceinline__ void jv_vvw_fields(const LineTable& t, const LayerFam& LF, const FamTan& FT,
                                              int li, int xt, float* v, float* base, float* dbase) {
  float r[JV_NREC];
  jv_vvw_record(t, LF, FT, li, xt, r, 1, base, dbase);   // 0 df, 2 fo_hi, 3 fo_lo, 4 S, 5 dlnS, 6..8 ddf
  v[0] = r[0];
  v[1] = r[0] * r[0];
  v[2] = -r[2];
  v[3] = -r[3];
  v[4] = r[4];
  v[5] = r[5];
  v[6] = r[6];
  v[7] = r[7];
  v[8] = r[8];
}

__device__ __forceinline__ void jv_sjs_fields(const LineTable& t, const LayerFam& LF, const FamTan& FT,
                                              const LayerTan& LT, float shift, int li, float* v) {
  float r[JV_NREC];
  jv_sjs_record(t, LF, FT, LT, shift, li, r, 1);   // 2 KH0, 3 KL0, 4 S, 5 dlnS, 6 G0, 9..11 dK0
  v[0] = r[2];
  v[1] = r[3];
  v[2] = r[4];
  v[3] = r[5];
  v[4] = r[6];
  v[5] = r[9];
  v[6] = r[10];
  v[7] = r[11];
}

// Packed two-sum of f32x2 lanes: s + e = a + b exactly, lane by lane.
__device__ __forceinline__ void two_sum2(f2 a, f2 b, f2& s, f2& e) {
  s = add2(a, b);
  const f2 bb = sub2(s, a);
  e = add2(sub2(a, sub2(s, bb)), sub2(b, bb));
}

__device__ __forceinline__ f2 rcp2(f2 x) { return pk(rcp_approx(lo2(x)), rcp_approx(hi2(x))); }

// Ben-Reuven pair: t = S n / den, n = (g - z) F + (g + z) K,
// den = e^2 + 4 g^2 F with e = F - K (double-float); dt along each tangent
// = Ag dg + Az dz + AK dK (+ t dlnS for T), accumulated into d.
__device__ __forceinline__ f2 br_eval2(f2 F, f2 FL, f2 m8F, f2 g, f2 gp, f2 gm, f2 K, f2 mKH,
                                       f2 mKL, f2 S, f2 dlnS, f2 G4, const f2* dg, const f2* dz,
                                       const f2* dK, f2* d) {
  const f2 e = add2(add2(F, mKH), add2(FL, mKL));
  const f2 den = fma2(e, e, mul2(G4, F));
  const f2 r = rcp2(den);
  const f2 n = fma2(gm, F, mul2(gp, K));
  const f2 nr = mul2(n, r);
  const f2 t = mul2(S, nr);
  const f2 Sr = mul2(S, r);
  const f2 Ag = mul2(Sr, fma2(mul2(m8F, g), nr, add2(F, K)));
  const f2 Az = mul2(Sr, sub2(K, F));
  const f2 AK = mul2(Sr, fma2(add2(e, e), nr, gp));
#pragma unroll
  for (int q = 0; q < 3; ++q) d[q] = fma2(Ag, dg[q], fma2(Az, dz[q], fma2(AK, dK[q], d[q])));
  d[0] = fma2(t, dlnS, d[0]);
  return t;
}

// Not inlined: each line kind's sweep gets the kernel's whole register budget
// for its own loop state (inlined into the family switch, the union of the
// four kinds' live values spilled to local memory at 64 registers).

// One family of one layer for the CTA's frequencies.  Records of JV_CHUNK
// lines at a time, double-buffered (chunk c+1 is built, one line per
// thread, while chunk c is swept), stored as line pairs so every f32x2
// instruction of the sweep serves two lines; the NG line groups of a
// frequency sweep pairs grp, grp + NG, ...; value terms are added in blocks
// of 16 lines into a compensated sum.  The groups' sums (value and three
// derivatives) go to sh.fam[fam][fi], added in group order.  Called by
// every thread.
template <int KIND, int CH>
__device__ __noinline__ void jv_family(const JvpArgs& a, JvpShared<CH>& sh, int L, int fam,
                                        const JvFreq& fr, bool on, float& base, float* dbase) {
  const int tid = threadIdx.x;
  const int FTL = a.ft, NG = blockDim.x / a.ft;
  const int fi = tid % FTL, grp = tid / FTL;
  const LayerParams& lp = a.lp[L];
  const LayerTan& LT = a.lt[L];
  const LineTable& t = a.tab[fam];
  const LayerFam& LF = lp.fam[fam];
  const FamTan& FT = LT.fam[fam];
  const int xt = fam_xtan(fam);
  const bool two = fam == FAM_NH3_INV;
  const bool hsf = fam == FAM_NH3_INV || fam == FAM_NH3_ROT || fam == FAM_NH3_V2;
  const float Fx = hsf ? fr.Fh : fr.F, FLx = hsf ? fr.FhL : fr.FL;
  auto put = [&](int bi, int set, int i, const float* v, int nf) {
    float* o = reinterpret_cast<float*>(sh.rec[bi][set][i >> 1]) + (i & 1);
    for (int k = 0; k < nf; ++k) o[2 * k] = v[k];
  };
  auto build = [&](int bi, int c0) {
    const int nc = min(CH, t.n - c0);
    const int ncp = (nc + 1) & ~1;
    for (int i = tid; i < ncp; i += blockDim.x) {
      const int li = c0 + i;
      float v[JV_NF];
      if (i >= nc) {
        jv_pad_fields<KIND>(v);
        put(bi, 0, i, v, JV_NF);
        if (two) put(bi, 1, i, v, JV_NF);
        continue;
      }
      if (KIND == JK_BR) {
        jv_br_fields(t, LF, FT, 0, li, xt, v);
        put(bi, 0, i, v, JV_NF);
        if (two) {
          jv_br_fields(t, LF, FT, 1, li, xt, v);
          put(bi, 1, i, v, JV_NF);
        }
      } else if (KIND == JK_GROSS) {
        jv_gross_fields(t, LF, FT, li, xt, v);
        put(bi, 0, i, v, 10);
      } else if (KIND == JK_VVW) {
        jv_vvw_fields(t, LF, FT, li, xt, v, &base, dbase);
        put(bi, 0, i, v, 10);
      } else {
        jv_sjs_fields(t, LF, FT, LT, lp.sjs[0][4], li, v);
        put(bi, 0, i, v, 8);
      }
    }
  };
  // nh3_sjs per-frequency coefficients and their derivatives
  float A = 0.f, B = 0.f, C = 0.f, D = 0.f, dA[3] = {0, 0, 0}, dB[3] = {0, 0, 0}, dC[3] = {0, 0, 0},
        dD[3] = {0, 0, 0};
  if (KIND == JK_SJS) {
    auto lerp = [&](float j0, float s0) { return fmaf(j0 - s0, fr.wJ, s0); };
    A = lerp(lp.sjs[0][0], lp.sjs[1][0]);
    B = lerp(lp.sjs[0][1], lp.sjs[1][1]);
    C = lerp(lp.sjs[0][2], lp.sjs[1][2]);
    D = lerp(lp.sjs[0][3], lp.sjs[1][3]);
    for (int q = 0; q < 3; ++q) {
      dA[q] = lerp(tan3(LT.dsjs[0][0], q, xt), tan3(LT.dsjs[1][0], q, xt));
      dB[q] = lerp(tan3(LT.dsjs[0][1], q, xt), tan3(LT.dsjs[1][1], q, xt));
      dC[q] = lerp(tan3(LT.dsjs[0][2], q, xt), tan3(LT.dsjs[1][2], q, xt));
      dD[q] = lerp(tan3(LT.dsjs[0][3], q, xt), tan3(LT.dsjs[1][3], q, xt));
    }
  }
  const f2 F2 = dup(Fx), FL2 = dup(FLx), m8F = dup(-8.f * Fx);
  KSum val;
  val.init();
  f2 vp = 0ull, der[3] = {0ull, 0ull, 0ull};
  int nv = 0;
  const int nchunks = (t.n + CH - 1) / CH;
  build(0, 0);
  __syncthreads();
  for (int ci = 0; ci < nchunks; ++ci) {
    const int c0 = ci * CH;
    const int np = (min(CH, t.n - c0) + 1) >> 1;
    if (ci + 1 < nchunks) build((ci + 1) & 1, c0 + CH);
    if (on) {
      const ulonglong2(*Rp)[JV_NU2] = sh.rec[ci & 1][two ? fr.set : 0];
      for (int p = grp; p < np; p += NG) {
        const ulonglong2* w = Rp[p];
        f2 tv;
        if (KIND == JK_BR) {
          const ulonglong2 w0 = w[0], w1 = w[1], w2 = w[2], w3 = w[3], w4 = w[4], w5 = w[5],
                           w6 = w[6], w7 = w[7], w8 = w[8];
          const f2 dg[3] = {w4.y, w5.x, w5.y};
          const f2 dz[3] = {w6.x, w6.y, w7.x};
          const f2 dK[3] = {w7.y, w8.x, w8.y};
          tv = br_eval2(F2, FL2, m8F, w0.x, w0.y, w1.x, w1.y, w2.x, w2.y, w3.x, w3.y, w4.x, dg, dz,
                        dK, der);
        } else if (KIND == JK_GROSS) {
          // t = S g / den, den = e^2 + 4 g^2 F; dt = (t dlnS) + S dg (1 - 8 F g^2 / den) / den
          const ulonglong2 w0 = w[0], w1 = w[1], w2 = w[2], w3 = w[3], w4 = w[4];
          const f2 e = add2(add2(F2, w2.x), add2(FL2, w2.y));
          const f2 r = rcp2(fma2(e, e, mul2(w0.y, F2)));
          const f2 Sr = mul2(w1.x, r);
          tv = mul2(Sr, w0.x);
          const f2 k = mul2(Sr, fma2(mul2(m8F, mul2(w0.x, w0.x)), r, dup(1.f)));
          der[0] = fma2(k, w3.x, fma2(tv, w1.y, der[0]));
          der[1] = fma2(k, w3.y, der[1]);
          der[2] = fma2(k, w4.x, der[2]);
        } else if (KIND == JK_VVW) {
          // t = h (r1 + r2), h = S df, r1 = 1/((f - fo)^2 + df^2), r2 = 1/((f + fo)^2 + df^2);
          // dt = t dlnS (T) + (S u - 2 h df (r1^2 + r2^2)) d(df)
          const ulonglong2 w0 = w[0], w1 = w[1], w2 = w[2], w3 = w[3], w4 = w[4];
          const f2 fq = dup(fr.fq), fql = dup(fr.fql);
          const f2 dm = add2(add2(fq, w1.x), add2(fql, w1.y));
          const f2 dp = sub2(fq, w1.x);
          const f2 r1 = rcp2(fma2(dm, dm, w0.y)), r2 = rcp2(fma2(dp, dp, w0.y));
          const f2 h = mul2(w2.x, w0.x), u = add2(r1, r2);
          tv = mul2(h, u);
          const f2 k2 = mul2(add2(h, h), mul2(w0.x, fma2(r1, r1, mul2(r2, r2))));
          const f2 c = sub2(mul2(w2.x, u), k2);
          der[0] = fma2(c, w3.x, fma2(tv, w2.y, der[0]));
          der[1] = fma2(c, w3.y, der[1]);
          der[2] = fma2(c, w4.x, der[2]);
        } else {
          const ulonglong2 w0 = w[0], w1 = w[1], w2 = w[2], w3 = w[3];
          const f2 G0 = w2.x;
          const f2 g = fma2(dup(B), G0, dup(A)), z = fma2(dup(D), G0, dup(C));
          const f2 gp = add2(g, z), gm = sub2(g, z);
          f2 dg[3], dz[3], dK[3];
          const f2 dK0[3] = {w2.y, w3.x, w3.y};
#pragma unroll
          for (int q = 0; q < 3; ++q) {
            dg[q] = fma2(dup(dB[q]), G0, dup(dA[q]));
            dz[q] = fma2(dup(dD[q]), G0, dup(dC[q]));
            dK[q] = fma2(add2(g, g), dg[q], fma2(mul2(dup(-2.f), z), dz[q], dK0[q]));
          }
          f2 KH, e;
          two_sum2(w0.x, mul2(gm, gp), KH, e);
          const f2 KL = add2(e, w0.y);
          const f2 mone = dup(-1.f);
          tv = br_eval2(F2, FL2, m8F, g, gp, gm, add2(KH, KL), mul2(KH, mone), mul2(KL, mone), w1.x,
                        w1.y, mul2(dup(4.f), mul2(g, g)), dg, dz, dK, der);
        }
        vp = add2(vp, tv);
        if (++nv == 8) {
          val.add(lo2(vp) + hi2(vp));
          vp = 0ull;
          nv = 0;
        }
      }
    }
    __syncthreads();
  }
  val.add(lo2(vp) + hi2(vp));
  if (NG == 1) {   // one line group: the thread's sums are the family's (read back by itself)
    sh.fam[fam][fi][0] = val.val();
    for (int q = 0; q < 3; ++q) sh.fam[fam][fi][1 + q] = lo2(der[q]) + hi2(der[q]);
    return;
  }
  // the line groups' sums, staged in the (now free) record buffer
  float(*s_grp)[4] = reinterpret_cast<float(*)[4]>(&sh.rec[0][0][0][0]);
  s_grp[tid][0] = val.val();
  for (int q = 0; q < 3; ++q) s_grp[tid][1 + q] = lo2(der[q]) + hi2(der[q]);
  __syncthreads();
  if (grp == 0) {
    float v4[4] = {0.f, 0.f, 0.f, 0.f};
    for (int gg = 0; gg < NG; ++gg)
      for (int q = 0; q < 4; ++q) v4[q] += s_grp[gg * FTL + fi][q];
    for (int q = 0; q < 4; ++q) sh.fam[fam][fi][q] = v4[q];
  }
  __syncthreads();
}

// Threads: JV_FT frequencies x (blockDim / JV_FT) line groups; group g
// sweeps lines g, g + NG, ... of every chunk and the groups' sums are added
// per family (with one group, 128 threads for 128 frequencies, each thread
// holds its frequency's family sums itself).  MINB resident CTAs per SM
// (launch_tan_jvp): 128-thread CTAs with 64-line chunks at 5 (96
// registers; 4 or 6 when asked), the 128-frequency tiles' default;
// 256-thread CTAs with 128-line chunks at 3 (80 registers; 4 when asked)
// for smaller tiles (measured: 4096 atmospheres of 300-1200 layers at 128
// frequencies, 290 / 278 / 284 ms at 4 / 5 / 6; one 1000-layer atmosphere
// at 64 frequencies, 0.474 ms per adjoint with 256 threads at 3 against
// 0.533 with 128 threads at 5).
template <int MINB, int NT>
__global__ void __launch_bounds__(NT, MINB) rb_alpha_jvp_kernel(JvpArgs a) {
  constexpr int CH = NT == 128 ? 64 : JV_CHUNK;
  __shared__ __align__(16) JvpShared<CH> sh;
  const int L = blockIdx.x;
  const int tid = threadIdx.x;
  const int FTL = a.ft;
  const int fi = tid % FTL, grp = tid / FTL;
  const int j = blockIdx.y * FTL + fi;
  const bool on = j < a.nf;
  const LayerParams& lp = a.lp[L];
  const LayerTan& LT = a.lt[L];
  // this thread's frequency (lanes past nf take f = 1 GHz and add nothing)
  const JvFreq fr = on ? a.fplan[j] : JvFreq{1.f, 0.f, 1.f, 0.f, 1.f, 0.f, 0.f, 0};
  const int set = fr.set;
  const bool nh3 = a.cfg.nh3_mode != NH3_OFF;
  // families that are off keep zero sums (read back by the same thread)
  if (grp == 0)
    for (int fam = 0; fam < NFAM; ++fam)
      for (int q = 0; q < 4; ++q) sh.fam[fam][fi][q] = 0.f;
  float base = 0.f, dbase[3] = {0.f, 0.f, 0.f};
  for (int fam = 0; fam < NFAM; ++fam) {
    bool en;
    switch (fam) {
      case FAM_NH3_INV:
      case FAM_NH3_ROT:
      case FAM_NH3_V2: en = nh3 && lp.use_hs; break;
      case FAM_NH3_SJS: en = nh3 && lp.use_sjs; break;
      case FAM_H2O: en = a.cfg.use_h2o; break;
      case FAM_H2S: en = a.cfg.use_h2s; break;
      default: en = a.cfg.use_ph3; break;
    }
    if (!en || a.tab[fam].n == 0) continue;
    switch (fam) {
      case FAM_NH3_INV:
      case FAM_H2S:
      case FAM_PH3: jv_family<JK_BR, CH>(a, sh, L, fam, fr, on, base, dbase); break;
      case FAM_NH3_ROT:
      case FAM_NH3_V2: jv_family<JK_GROSS, CH>(a, sh, L, fam, fr, on, base, dbase); break;
      case FAM_H2O: jv_family<JK_VVW, CH>(a, sh, L, fam, fr, on, base, dbase); break;
      default: jv_family<JK_SJS, CH>(a, sh, L, fam, fr, on, base, dbase); break;
    }
  }
  // h2o base term summed over the CTA (every thread built some lines)
  {
    float v[4] = {base, dbase[0], dbase[1], dbase[2]};
    for (int k = 0; k < 4; ++k)
      for (int o = 16; o; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
    __shared__ float s_b[8][4];
    if ((tid & 31) == 0)
      for (int k = 0; k < 4; ++k) s_b[tid >> 5][k] = v[k];
    __syncthreads();
    base = dbase[0] = dbase[1] = dbase[2] = 0.f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      base += s_b[w][0];
      dbase[0] += s_b[w][1];
      dbase[1] += s_b[w][2];
      dbase[2] += s_b[w][3];
    }
  }
  // dalpha/dtheta (cm^-1) of this (layer, frequency), contracted with
  // dTb/dalpha.  The per-frequency combination is float32 (its inputs, the
  // family sums, tangents and coefficients, are float32; GB300's float64
  // rate made it ~10 % of the kernel); the sum over frequencies, where terms
  // of both signs meet, is float64.
  float g5[NTH] = {0.f, 0.f, 0.f, 0.f, 0.f};
  if (on && grp == 0) {
    auto fv = [&](int fam) { return sh.fam[fam][fi][0]; };
    auto fd = [&](int fam) { return &sh.fam[fam][fi][1]; };
    const float gal = a.alpha_out ? 0.f : a.galpha[(size_t)L * a.nf + j];
    const float Fd = fr.F + fr.FL, Fhd = fr.Fh + fr.FhL;
    auto pref = [&](int fam) { return ldexpf(lp.fam[fam].fm, lp.fam[fam].fe); };
    // d(pref * S) / dtheta for a family with tangent triple (T, P, X_own)
    float dal[NTH] = {0.f, 0.f, 0.f, 0.f, 0.f};
    auto add_fam = [&](int fam, float mult, float sv, const float* ds, float* out) {
      const FamTan& FT = LT.fam[fam];
      const float pm = pref(fam) * mult;
      const int xt = fam_xtan(fam);
      out[TH_T] += pm * fmaf(FT.dlnpref[TH_T], sv, ds[0]);
      out[TH_P] += pm * fmaf(FT.dlnpref[TH_P], sv, ds[1]);
#pragma unroll
      for (int q = 2; q < NTH; ++q) out[q] += pm * fmaf(FT.dlnpref[q], sv, q == xt ? ds[2] : 0.f);
    };
    // H2 CIA
    if (a.cfg.use_h2)
      for (int q = 0; q < NTH; ++q) dal[q] += lp.scale[GAS_H2] * LT.dh2_cia[q] * Fd;
    // H2O lines and continuum
    if (a.cfg.use_h2o) {
      float d[NTH] = {0.f, 0.f, 0.f, 0.f, 0.f};
      const float ds[3] = {fd(FAM_H2O)[0] - dbase[0], fd(FAM_H2O)[1] - dbase[1], fd(FAM_H2O)[2] - dbase[2]};
      add_fam(FAM_H2O, 1.f, fv(FAM_H2O) - base, ds, d);
      for (int q = 0; q < NTH; ++q) dal[q] += lp.scale[GAS_H2O] * (d[q] + LT.dh2o_cont[q]) * Fd;
    }
    if (a.cfg.use_h2s) {
      float d[NTH] = {0.f, 0.f, 0.f, 0.f, 0.f};
      add_fam(FAM_H2S, 1.f, fv(FAM_H2S), fd(FAM_H2S), d);
      for (int q = 0; q < NTH; ++q) dal[q] += lp.scale[GAS_H2S] * d[q] * Fd;
    }
    if (a.cfg.use_ph3) {
      float d[NTH] = {0.f, 0.f, 0.f, 0.f, 0.f};
      add_fam(FAM_PH3, 1.f, fv(FAM_PH3), fd(FAM_PH3), d);
      for (int q = 0; q < NTH; ++q) dal[q] += lp.scale[GAS_PH3] * d[q] * Fd;
    }
    if (nh3) {
      float hs = 0.f, dhs[NTH] = {0.f, 0.f, 0.f, 0.f, 0.f}, sj = 0.f, dsj[NTH] = {0.f, 0.f, 0.f, 0.f, 0.f};
      const float INVC[2][2] = {{0.9301f, 0.9862f}, {0.9619f, 0.9862f}};   // Con, per table and set
      if (lp.use_hs) {
        const float con = INVC[a.cfg.inv_table][set];
        hs = Fhd * (pref(FAM_NH3_INV) * con * fv(FAM_NH3_INV) + pref(FAM_NH3_ROT) * fv(FAM_NH3_ROT) +
                    pref(FAM_NH3_V2) * fv(FAM_NH3_V2));
        add_fam(FAM_NH3_INV, con, fv(FAM_NH3_INV), fd(FAM_NH3_INV), dhs);
        add_fam(FAM_NH3_ROT, 1.f, fv(FAM_NH3_ROT), fd(FAM_NH3_ROT), dhs);
        add_fam(FAM_NH3_V2, 1.f, fv(FAM_NH3_V2), fd(FAM_NH3_V2), dhs);
        for (int q = 0; q < NTH; ++q) dhs[q] *= Fhd;
        if (hs < 0.f) {   // clamped to 1e-8 (nh3_hs.py:311-312): no derivative
          hs = 1.0e-8f;
          for (int q = 0; q < NTH; ++q) dhs[q] = 0.f;
        }
      }
      if (lp.use_sjs) {
        sj = Fd * pref(FAM_NH3_SJS) * fv(FAM_NH3_SJS);
        add_fam(FAM_NH3_SJS, 1.f, fv(FAM_NH3_SJS), fd(FAM_NH3_SJS), dsj);
        for (int q = 0; q < NTH; ++q) dsj[q] *= Fd;
      }
      float dn[NTH];
      if (lp.use_hs && lp.use_sjs) {
        const float W = lp.blendW;
        for (int q = 0; q < NTH; ++q) dn[q] = W * dsj[q] + (1.f - W) * dhs[q];
        dn[TH_P] += LT.dblendW_dP * (sj - hs);
      } else {
        for (int q = 0; q < NTH; ++q) dn[q] = lp.use_hs ? dhs[q] : dsj[q];
      }
      for (int q = 0; q < NTH; ++q) dal[q] += lp.scale[GAS_NH3] * dn[q];
    }
    if (a.alpha_out) {
      // stored-tangent mode: the scan's alpha (the assembly kernel's float32
      // arithmetic on the same family sums) and d alpha / d theta
      double co = 0.0, cl = 0.0;
      if (a.extra) {
        co = a.extra[(size_t)L * a.nf + j];
        cl = a.extra[((size_t)a.nL + L) * a.nf + j];
      }
      float g32[NGAS];
      assemble<float>(lp, a.cfg, Fd, Fhd, set, fv(FAM_NH3_INV), fv(FAM_NH3_ROT), fv(FAM_NH3_V2),
                      fv(FAM_NH3_SJS), fv(FAM_H2O), base, fv(FAM_H2S), fv(FAM_PH3), co, cl, g32);
      float tot = 0.f;
      for (int k = 0; k < NGAS; ++k) tot += g32[k];
      a.alpha_out[(size_t)L * a.nf + j] = tot;
      for (int q = 0; q < NTH; ++q) a.dal_out[((size_t)L * NTH + q) * a.nf + j] = dal[q];
    }
    for (int q = 0; q < NTH; ++q) g5[q] = gal * dal[q];
  }
  if (a.alpha_out) return;   // uniform: a kernel argument
  // reduce over the CTA's frequencies as double-floats (terms of both signs
  // meet here; GB300's float64 rate made the float64 shuffles a tenth of the
  // batched kernel); only the warps of line group 0 hold values: FTL is a
  // multiple of 32.  The final kernel adds hi + lo in float64 per layer.
  const int nw0 = FTL >> 5;
  if (grp == 0) {
    for (int q = 0; q < NTH; ++q) {
      float hi = g5[q], lo = 0.f;
      for (int o = 16; o; o >>= 1) {
        const float h2 = __shfl_xor_sync(0xffffffffu, hi, o);
        const float l2 = __shfl_xor_sync(0xffffffffu, lo, o);
        float s, e;
        two_sum(hi, h2, s, e);
        e += lo + l2;
        hi = s + e;
        lo = e - (hi - s);
      }
      if ((tid & 31) == 0) sh.red[tid >> 5][q] = make_float2(hi, lo);
    }
  }
  __syncthreads();
  if (tid < NTH) {
    float hi = 0.f, lo = 0.f;
    for (int w = 0; w < nw0; ++w) {
      const float2 v = sh.red[w][tid];
      float s, e;
      two_sum(hi, v.x, s, e);
      e += lo + v.y;
      hi = s + e;
      lo = e - (hi - s);
    }
    a.part[((size_t)L * gridDim.y + blockIdx.y) * NTH + tid] = make_float2(hi, lo);
  }
}

// dT = sum of tiles + source term (summed over frequencies); dP; dln X
// for NH3, H2O, H2S.
__global__ void rb_adjoint_final_kernel(int nL, int nf, int ntile, const float2* part,
                                        const double* gsrc, const double* gextra, double* dT,
                                        double* dP, double* dlnX) {
  const int L = blockIdx.x * blockDim.x + threadIdx.x;
  if (L >= nL) return;
  double s[NTH] = {0, 0, 0, 0, 0};
  for (int t = 0; t < ntile; ++t)
    for (int q = 0; q < NTH; ++q) {
      const float2 v = part[((size_t)L * ntile + t) * NTH + q];
      s[q] += (double)v.x + (double)v.y;
    }
  if (gextra) {
    s[TH_T] += gextra[2 * L];
    s[TH_P] += gextra[2 * L + 1];
  }
  dT[L] = s[TH_T] + gsrc[L];
  dP[L] = s[TH_P];
  dlnX[L] = s[TH_XNH3];
  dlnX[nL + L] = s[TH_XH2O];
  dlnX[2 * nL + L] = s[TH_XH2S];
}

// Stored-tangent adjoint: d loss / d theta of each layer is the sum over
// frequencies of d loss / d alpha times the stored d alpha / d theta, plus
// the source term (dT) and the co_ddb / clouds_idp terms.  One warp per
// layer, lanes over frequencies: products in float32 as in the contracting
// JVP, sums as double-floats (terms of both signs), hi + lo in float64.
__global__ void __launch_bounds__(128) rb_adjoint_contract_kernel(int nL, int nf, const float* galpha,
                                                                  const float* dal, const double* gsrc,
                                                                  const double* gextra, double* dT,
                                                                  double* dP, double* dlnX) {
  const int L = blockIdx.x * 4 + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (L >= nL) return;   // whole warps: L is uniform in a warp
  const float* g = galpha + (size_t)L * nf;
  const float* d = dal + (size_t)L * NTH * nf;
  float hi[NTH], lo[NTH];
#pragma unroll
  for (int q = 0; q < NTH; ++q) hi[q] = lo[q] = 0.f;
  for (int j = lane; j < nf; j += 32) {
    const float gj = __ldcs(g + j);
#pragma unroll
    for (int q = 0; q < NTH; ++q) dfs_add(hi[q], lo[q], gj * __ldcs(d + (size_t)q * nf + j));
  }
  double s[NTH];
#pragma unroll
  for (int q = 0; q < NTH; ++q) {
    for (int o = 16; o; o >>= 1) {
      const float h2 = __shfl_xor_sync(0xffffffffu, hi[q], o);
      const float l2 = __shfl_xor_sync(0xffffffffu, lo[q], o);
      float t, e;
      two_sum(hi[q], h2, t, e);
      e += lo[q] + l2;
      hi[q] = t + e;
      lo[q] = e - (hi[q] - t);
    }
    s[q] = (double)hi[q] + (double)lo[q];
  }
  if (lane) return;
  if (gextra) {
    s[TH_T] += gextra[2 * L];
    s[TH_P] += gextra[2 * L + 1];
  }
  dT[L] = s[TH_T] + gsrc[L];
  dP[L] = s[TH_P];
  dlnX[L] = s[TH_XNH3];
  dlnX[nL + L] = s[TH_XH2O];
  dlnX[2 * nL + L] = s[TH_XH2S];
}

// ------------------------------------------------------------------ launch
cudaError_t launch_extra_vjp(const ExtraArgs& ea, cudaStream_t st);

// d loss / d alpha and the source term: zeroed, then the reverse sweep.
cudaError_t launch_adjoint_sweep(const TbAdjArgs& ta, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(ta.ga, 0, sizeof(float) * (size_t)ta.nL * ta.nf, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(ta.gs, 0, sizeof(double) * (size_t)ta.nL, st);
  if (e != cudaSuccess) return e;
  if (ta.nb > 0 && ta.disc) {
    const int blk = ta.nf >= 128 ? 128 : ((ta.nf + 31) / 32) * 32;
    rb_tb_adj_disc_kernel<<<dim3(ta.nb, (ta.nf + blk - 1) / blk), blk, 0, st>>>(ta);
  } else if (ta.nb > 0) {
    const int blk = ta.nf >= 128 ? 128 : ((ta.nf + 31) / 32) * 32;
    dim3 grid(ta.nb, ta.nchunk, (ta.nf + blk - 1) / blk);
    rb_tb_adj_lambda_kernel<<<grid, blk, 0, st>>>(ta);
    rb_tb_adj_suffix_kernel<<<dim3(ta.nb, (ta.nf + blk - 1) / blk), blk, 0, st>>>(ta);
    rb_tb_adj_grad_kernel<<<grid, blk, 0, st>>>(ta);
  }
  return cudaGetLastError();
}

// Layer tangents, then the JVP kernel in the launch shape of jv.
static cudaError_t launch_tan_jvp(const TanArgs& tn, const JvpArgs& jv, cudaStream_t st) {
  rb_layer_tan_kernel<<<(((tn.nL + 31) & ~31) * 8 + 63) / 64, 64, 0, st>>>(tn);
  dim3 grid(jv.nL, (jv.nf + jv.ft - 1) / jv.ft);
  const int ctas = jv.ctas ? jv.ctas : 3;   // 256-thread CTAs: 3 per SM unless asked
  // threads per CTA: one line group for 128-frequency tiles (no per-family
  // reduction across groups; 4096 atmospheres at 128 frequencies 412 -> 371
  // ms), two or four otherwise.
  // 128-thread CTAs: 5 per SM (96 registers) unless 4 (120) or 6 (80) are asked.
  const int nt = jv.threads ? jv.threads : (jv.ft >= 128 ? 128 : 256);
  if (nt == 128) {
    if (jv.ctas == 4) rb_alpha_jvp_kernel<4, 128><<<grid, 128, 0, st>>>(jv);
    else if (jv.ctas == 6) rb_alpha_jvp_kernel<6, 128><<<grid, 128, 0, st>>>(jv);
    else rb_alpha_jvp_kernel<5, 128><<<grid, 128, 0, st>>>(jv);
  } else if (ctas >= 4) {
    rb_alpha_jvp_kernel<4, 256><<<grid, 256, 0, st>>>(jv);
  } else {
    rb_alpha_jvp_kernel<3, 256><<<grid, 256, 0, st>>>(jv);
  }
  return cudaGetLastError();
}

// Recomputing adjoint: the reverse sweep, then alpha's JVP contracted with
// d loss / d alpha, then the per-layer sums.
cudaError_t launch_adjoint(const TbAdjArgs& ta, const TanArgs& tn, const JvpArgs& jv,
                           const ExtraArgs* ea, float* galpha, double* gsrc, double* dT, double* dP,
                           double* dlnX, cudaStream_t st) {
  cudaError_t e = launch_adjoint_sweep(ta, st);
  if (e == cudaSuccess) e = launch_tan_jvp(tn, jv, st);
  if (e != cudaSuccess) return e;
  if (ea) {
    cudaError_t x = launch_extra_vjp(*ea, st);
    if (x != cudaSuccess) return x;
  }
  const int ntile = (jv.nf + jv.ft - 1) / jv.ft;
  rb_adjoint_final_kernel<<<(jv.nL + 127) / 128, 128, 0, st>>>(
      jv.nL, jv.nf, ntile, jv.part, gsrc, ea ? ea->grad : nullptr, dT, dP, dlnX);
  return cudaGetLastError();
}

// Stored-tangent adjoint, forward half: layer tangents and the JVP writing
// alpha and d alpha / d theta (jv.alpha_out, jv.dal_out) for the scan.
cudaError_t launch_jvp_store(const TanArgs& tn, const JvpArgs& jv, cudaStream_t st) {
  return launch_tan_jvp(tn, jv, st);
}

// Stored-tangent adjoint, after the reverse sweep: [co / clouds VJP,]
// the contraction with d loss / d alpha.
cudaError_t launch_adjoint_contract(const JvpArgs& jv, const ExtraArgs* ea, const float* galpha,
                                    const double* gsrc, double* dT, double* dP, double* dlnX,
                                    cudaStream_t st) {
  if (ea) {
    cudaError_t x = launch_extra_vjp(*ea, st);
    if (x != cudaSuccess) return x;
  }
  rb_adjoint_contract_kernel<<<(jv.nL + 3) / 4, 128, 0, st>>>(
      jv.nL, jv.nf, galpha, jv.dal_out, gsrc, ea ? ea->grad : nullptr, dT, dP, dlnX);
  return cudaGetLastError();
}

// Frequencies per CTA of rb_alpha_jvp_kernel (threads beyond them split
// the lines).
// (ft_forced: rb_set_tuning's choice, 0 = automatic.)
int adjoint_ft(int nf, int ft_forced) {
  if (ft_forced) return ft_forced;
  return nf >= 128 ? 128 : (nf >= 64 ? 64 : 32);
}
int adjoint_tiles(int nf, int ft_forced) {
  const int ft = adjoint_ft(nf, ft_forced);
  return (nf + ft - 1) / ft;
}

}  // namespace rb
