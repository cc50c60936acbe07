// C ABI of the GB300 radioBEAR forward model (include/radiobear_gb300.h):
// handle, device-memory management, catalogue preprocessing, frequency
// plans and the launch sequences.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <functional>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/radiobear_gb300.h"
#include "rb_args.cuh"

namespace {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

#define RB_CUDA(call)                                                                  \
  do {                                                                                 \
    cudaError_t e_ = (call);                                                           \
    if (e_ != cudaSuccess)                                                             \
      return fail(e_ == cudaErrorMemoryAllocation ? RB_ENOMEM : RB_ECUDA, "%s: %s (%s:%d)", \
                  #call, cudaGetErrorString(e_), __FILE__, __LINE__);                  \
  } while (0)

// Counts (re)allocations of device and pinned host buffers: a captured
// CUDA graph holds buffer addresses and is replayed only while this count
// is unchanged.
std::atomic<unsigned long long> g_alloc_epoch{0};

struct DBuf {
  void* p = nullptr;
  size_t cap = 0;
  cudaError_t ensure(size_t bytes) {
    if (bytes <= cap) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    ++g_alloc_epoch;
    size_t want = std::max(bytes, (size_t)256);
    cudaError_t e = cudaMalloc(&p, want);
    if (e == cudaSuccess) cap = want;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    if (p) ++g_alloc_epoch;
    p = nullptr;
    cap = 0;
  }
  template <class T>
  T* as() const { return reinterpret_cast<T*>(p); }
};

// Pinned host staging buffer.
struct HBuf {
  void* p = nullptr;
  size_t cap = 0;
  cudaError_t ensure(size_t bytes) {
    if (bytes <= cap) return cudaSuccess;
    if (p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
    ++g_alloc_epoch;
    size_t want = std::max(bytes, (size_t)4096);
    cudaError_t e = cudaHostAlloc(&p, want, cudaHostAllocDefault);
    if (e == cudaSuccess) cap = want;
    return e;
  }
  void release() {
    if (p) cudaFreeHost(p);
    if (p) ++g_alloc_epoch;
    p = nullptr;
    cap = 0;
  }
  template <class T>
  T* as() const { return reinterpret_cast<T*>(p); }
};

// Shape of an rb_forward / rb_adjoint call from host buffers: everything a
// captured graph of it bakes in (sizes, kernel scalars, configuration,
// addresses).
struct FwdKey {
  int nL = -1, nf = 0, nb = 0, disc = 0, gtype = 0, limb = 0, flags = 0;
  double Req = 0, Rpol = 0, o0 = 0, o1 = 0;
  unsigned long long cfg = 0, epoch = 0;
  bool operator==(const FwdKey& o) const {
    return nL == o.nL && nf == o.nf && nb == o.nb && disc == o.disc && gtype == o.gtype &&
           limb == o.limb && flags == o.flags && Req == o.Req && Rpol == o.Rpol && o0 == o.o0 &&
           o1 == o.o1 && cfg == o.cfg && epoch == o.epoch;
  }
};

// The graph of the last call shape that ran twice, and the shape of the
// last call that ran directly.
struct GraphCache {
  FwdKey seen, key;
  cudaGraphExec_t exec = nullptr;
  int launches = 0;
  void release() {
    if (exec) cudaGraphExecDestroy(exec);
    exec = nullptr;
  }
};

// A batch of atmospheres (rb_forward_batch_device): variant v owns layers
// [off[v], off[v+1]) of the concatenated arrays and rays [v nb, (v+1) nb)
// with the shared impact parameters.
struct Batch {
  int nvar = 0;
  const int* d_off = nullptr;   // device [nvar + 1]
  int max_nL = 0;
};

int family_ncols(int fam) {
  switch (fam) {
    case rb::FAM_NH3_INV: return 4;
    case rb::FAM_NH3_ROT: return 6;
    case rb::FAM_NH3_V2: return 3;
    case rb::FAM_NH3_SJS: return 4;
    case rb::FAM_H2O: return 10;
    case rb::FAM_H2S: return 4;
    case rb::FAM_PH3: return 6;
  }
  return -1;
}

struct FamilyStore {
  int n = 0;
  std::vector<double> centre;   // sorted, host copy (near-range search)
  float l2Imax = 0.f, Emin = 0.f, Emax = 0.f;
  DBuf c2h, c2l, ch, cl, l2Ih, l2Il, Eh, El, w1, w2, w3, x1, x2, x3;
  rb::LineTable table() const {
    rb::LineTable t{};
    t.n = n;
    t.c2h = c2h.as<float>();
    t.c2l = c2l.as<float>();
    t.ch = ch.as<float>();
    t.cl = cl.as<float>();
    t.l2Ih = l2Ih.as<float>();
    t.l2Il = l2Il.as<float>();
    t.Eh = Eh.as<float>();
    t.El = El.as<float>();
    t.w1 = w1.as<float>();
    t.w2 = w2.as<float>();
    t.w3 = w3.as<float>();
    t.x1 = x1.as<float>();
    t.x2 = x2.as<float>();
    t.x3 = x3.as<float>();
    t.l2Imax = l2Imax;
    t.Emin = Emin;
    t.Emax = Emax;
    return t;
  }
  void release() {
    for (DBuf* b : {&c2h, &c2l, &ch, &cl, &l2Ih, &l2Il, &Eh, &El, &w1, &w2, &w3, &x1, &x2, &x3})
      b->release();
  }
};

}  // namespace

struct rb_handle {
  int device = 0;
  cudaStream_t st = nullptr, side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  // The last _device call's work on its stream (recorded when that stream
  // was not capturing): later calls on other streams, and the handle's own
  // stream, wait for it before touching the handle's workspaces.
  cudaEvent_t ev_dev = nullptr;
  bool dev_pending = false;
  FamilyStore fam[rb::NFAM];
  rb::AlphaConfig cfg{rb::NH3_HS_SJS, 1, 1, 1, 1, 'e', 0, 0, 0, rb::CO_VOIGT, 0, 0};
  // co_ddb lines (co.npz: f0 GHz, I0, E cm^-1), float64
  int nco = 0;
  DBuf d_co_f0, d_co_I0, d_co_E;
  DBuf d_extra, d_xgrad;   // [2][nL][nf] co / cloud absorption; [nL][2] their adjoint
  DBuf d_agas, d_acl, d_aout, d_aclout, d_aprop, d_agrid, d_aoff;   // atmosphere producer
  // frequency plan
  std::vector<double> plan_f;
  int plan_M = 0, plan_W = 0, plan_spt = 0, plan_ntile = 0, plan_nslot = 0, plan_ntmpl = 0;
  int plan_grid = 0;
  int plan_vbeg[rb::NFAM] = {}, plan_vend[rb::NFAM] = {};
  int tile_M = 0, tile_W = 0, item_lines = 0;   // rb_set_alpha_tiling (0: automatic)
  int jvp_ft = 0, jvp_ctas = 0, jvp_threads = 0, scan_lanes = 0;   // rb_set_tuning (0: automatic)
  int adj_mode = 0;                                                  // RB_TUNE_ADJ_MODE
  size_t dev_mem = 0;                                                // device memory (bytes)
  DBuf d_f, d_fhs, d_jfreq, d_chains, d_tflags, d_wsets, d_tmpl, d_sj, d_sF, d_sFhs, d_sf, d_swJ, d_sset, d_counter,
      d_res, d_base;
  // adjoint workspaces
  DBuf d_ga, d_gs, d_lt, d_jpart, d_grad, d_dth, d_adjS, d_voff, d_dal, d_iw32;
  std::vector<int> batch_off;   // layer offsets of the last batch (d_voff)
  // workspaces
  DBuf d_P, d_T, d_X, d_scale, d_lp, d_a32, d_l64, d_g64, d_R, d_N, d_b, d_w, d_nseg, d_ds,
      d_layer, d_r4, d_ll, d_end, d_Tb, d_avg, d_iw, d_tau, d_W, d_tbl, d_x, d_dR, d_sR, d_R32,
      d_T32, d_hds, d_Tb32, d_part, d_rstart;
  int launches = 0;
  // rb_forward from host buffers: the inputs are staged in one pinned block
  // and uploaded with one copy, the outputs come back the same way, and a
  // call whose shape has run before is replayed from a captured graph
  unsigned long long cfg_gen = 0;   // bumped by every setter and re-plan
  HBuf h_in, h_out;
  DBuf d_in;
  GraphCache g_fwd, g_adj;
  // phase timing (rb_set_profiling)
  int profiling = 0;
  cudaEvent_t pev[10] = {};
  float phase_ms[5] = {0, 0, 0, 0, 0};
  DBuf d_probe;
};

namespace rb {
// Lets other translation units of the library report through rb_last_error.
void set_last_error(const char* msg) { g_err = msg; }
}  // namespace rb

namespace {
bool capturing(cudaStream_t st) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  return cudaStreamIsCapturing(st, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone;
}

// A call about to use the handle's workspaces on `st` waits for the work the
// last _device call enqueued on its own stream (a _device call returns
// before its kernels run; a host call or a _device call on another stream
// would otherwise overwrite buffers those kernels still read or
// accumulate into).  Skipped while `st` is being captured: a captured
// graph may not wait on work outside it.
cudaError_t order_after_device(rb_handle* h, cudaStream_t st) {
  if (!h->dev_pending || capturing(st)) return cudaSuccess;
  return cudaStreamWaitEvent(st, h->ev_dev, 0);
}

// After a _device call enqueued its work on `st`.
cudaError_t mark_device(rb_handle* h, cudaStream_t st) {
  if (capturing(st)) return cudaSuccess;
  h->dev_pending = true;
  return cudaEventRecord(h->ev_dev, st);
}
}  // namespace

// launchers implemented in the kernel translation units
namespace rb {
cudaError_t launch_prep(const PrepArgs& pa, cudaStream_t st);
cudaError_t launch_alpha_lines(const AlphaArgs& aa, int nblocks, cudaStream_t st);
cudaError_t launch_alpha_assemble(const AlphaArgs& aa, cudaStream_t st);
cudaError_t launch_extra(const ExtraArgs& a, cudaStream_t st);
cudaError_t launch_atm_props(const AtmPropArgs& a, int nvar, cudaStream_t st);
cudaError_t launch_atm_regrid(const AtmRegridArgs& a, int nvar, cudaStream_t st);
int alpha_lines_occupancy(int M, int W);
cudaError_t launch_adjoint(const TbAdjArgs& ta, const TanArgs& tn, const JvpArgs& jv,
                           const ExtraArgs* ea, float* galpha,
                           double* gsrc, double* dT, double* dP, double* dlnX, cudaStream_t st);
cudaError_t launch_adjoint_sweep(const TbAdjArgs& ta, cudaStream_t st);
cudaError_t launch_jvp_store(const TanArgs& tn, const JvpArgs& jv, cudaStream_t st);
cudaError_t launch_adjoint_contract(const JvpArgs& jv, const ExtraArgs* ea, const float* galpha,
                                    const double* gsrc, double* dT, double* dP, double* dlnX,
                                    cudaStream_t st);
int adjoint_tiles(int nf, int ft_forced);
int adjoint_ft(int nf, int ft_forced);
cudaError_t launch_geom_prep(int nL, const double* R, const double* T, float2* dR2, float* dR,
                             float* R32, float* T32, const int* var_off, int nvar, cudaStream_t st);
cudaError_t launch_raypath(const RayArgs& a, cudaStream_t st);
cudaError_t launch_tb_seq(const TbArgs& a, cudaStream_t st);
cudaError_t launch_tb_chunked(const TbArgs& a, cudaStream_t st);
int tb_nchunk(int max_seg);
cudaError_t launch_disc_avg(int nb, int nf, const float* Tb32, const double* w, double* out,
                            cudaStream_t st, int nvar = 1);
cudaError_t launch_e2(int order, int n, const double* x, double* out, cudaStream_t st);
cudaError_t launch_fp32_probe(int blocks, int iters, float* sink, int packed, cudaStream_t st);
}  // namespace rb

namespace {

bool finite_all(const double* v, size_t n) {
  for (size_t i = 0; i < n; ++i)
    if (!std::isfinite(v[i])) return false;
  return true;
}

template <class T>
cudaError_t upload(DBuf& b, const T* src, size_t count, cudaStream_t st) {
  cudaError_t e = b.ensure(count * sizeof(T));
  if (e != cudaSuccess || count == 0) return e;
  return cudaMemcpyAsync(b.p, src, count * sizeof(T), cudaMemcpyHostToDevice, st);
}

// Frequency plan and line-sum work decomposition.
//  * nh3_hs output order (nh3_hs.py:70-88): slot j evaluates nh3_hs at the
//    j-th element of [freqs <= 30 GHz in order, freqs > 30 GHz in order] and
//    takes coefficient set 1 when that frequency is above 30 GHz;
//  * slot s = j, padded at the end to whole tiles of 32 M W slots; lane i of
//    warp w owns slot 32 block(w, k) + i of its tile as chain k, the block
//    partition chosen per tile to minimise the double-float work;
//  * per chain and family, the index range of lines whose centre is within
//    [0.75 fmin, 1.3 fmax] of the chain's frequencies (those take the
//    double-float path);
//  * template entries: each family's lines cut into items of item_lines,
//    heaviest family first (nh3_sjs, inversion, h2o, rotational, nu2, h2s,
//    ph3).  Inversion items build the records of both coefficient sets
//    when the tile needs both.
int plan_frequencies(rb_handle* h, int nf, const double* freqs, cudaStream_t st) {
  if (nf < 1) return fail(RB_EINVAL, "nf must be >= 1");
  // Frequencies, like line centres, at most 2e4 GHz: the line sums multiply
  // two lines' float32 denominators ((f^2 + fo^2)^2 each), whose product
  // then stays over two decades below the float32 range.
  for (int i = 0; i < nf; ++i)
    if (!std::isfinite(freqs[i]) || freqs[i] < 0.0 || freqs[i] > 2.0e4)
      return fail(RB_EINVAL, "frequency %d: %g GHz outside [0, 2e4]", i, freqs[i]);
  if ((int)h->plan_f.size() == nf && std::equal(freqs, freqs + nf, h->plan_f.begin()))
    return RB_OK;
  std::vector<double> fhs;
  fhs.reserve(nf);
  for (int i = 0; i < nf; ++i)
    if (freqs[i] <= 30.0) fhs.push_back(freqs[i]);
  const int n_lo = (int)fhs.size();
  for (int i = 0; i < nf; ++i)
    if (freqs[i] > 30.0) fhs.push_back(freqs[i]);
  // tiling: forced by rb_set_alpha_tiling, else by the number of 32-slot blocks
  int M = h->tile_M, W = h->tile_W;
  if (M <= 0 || W <= 0) {
    const int blocks = (nf + 31) / 32;
    if (blocks >= 8) { M = 2; W = 4; }
    else if (blocks >= 4) { M = 2; W = 2; }
    else { M = 2; W = 1; }
  }
  const int spt = 32 * M * W;
  const int ntile = (nf + spt - 1) / spt;
  const int nslot = ntile * spt;
  std::vector<int> slot_j(nslot, -1);
  std::vector<float2> sF(nslot), sFhs(nslot), sf(nslot);
  std::vector<float> swJ(nslot, 0.f);
  std::vector<int> sset(nslot, 0);
  for (int s = 0; s < nslot; ++s) {
    const int j = s < nf ? s : -1;
    const int jj = j >= 0 ? j : nf - 1;   // padding repeats the last frequency
    slot_j[s] = j;
    const double f = freqs[jj], fh = fhs[jj];
    float a, b;
    rb::split_double(f * f, a, b);
    sF[s] = make_float2(a, b);
    rb::split_double(fh * fh, a, b);
    sFhs[s] = make_float2(a, b);
    rb::split_double(f, a, b);
    sf[s] = make_float2(a, b);
    swJ[s] = f <= 26.0 ? 0.f : (f >= 34.0 ? 1.f : (float)((f - 26.0) / 8.0));
    sset[s] = jj >= n_lo ? 1 : 0;
  }
  // per 32-slot block: set flags and the double-float line window of each family
  const int nbk = M * W;
  std::vector<rb::ChainPlan> blocks((size_t)ntile * nbk);
  std::vector<int> tflags(ntile, 0);
  for (int t = 0; t < ntile; ++t)
    for (int bk = 0; bk < nbk; ++bk) {
      rb::ChainPlan& c = blocks[(size_t)t * nbk + bk];
      c = rb::ChainPlan{};
      c.block = bk;
      double lo = INFINITY, hi = -INFINITY, lo_h = INFINITY, hi_h = -INFINITY;
      for (int i = 0; i < 32; ++i) {
        const int s = t * spt + 32 * bk + i;
        const int j = slot_j[s];
        if (j < 0) continue;
        c.flags |= rb::CH_VALID | (sset[s] ? rb::CH_SET1 : rb::CH_SET0);
        lo = std::min(lo, freqs[j]);
        hi = std::max(hi, freqs[j]);
        lo_h = std::min(lo_h, fhs[j]);
        hi_h = std::max(hi_h, fhs[j]);
      }
      tflags[t] |= c.flags;
      for (int fam = 0; fam < rb::NFAM; ++fam) {
        c.near[fam] = make_int2(0, 0);
        if (!(c.flags & rb::CH_VALID)) continue;
        const bool hs = fam == rb::FAM_NH3_INV || fam == rb::FAM_NH3_ROT || fam == rb::FAM_NH3_V2;
        const double l = hs ? lo_h : lo, u = hs ? hi_h : hi;
        const std::vector<double>& cen = h->fam[fam].centre;
        const int a = (int)(std::lower_bound(cen.begin(), cen.end(), 0.75 * l) - cen.begin());
        const int b = (int)(std::upper_bound(cen.begin(), cen.end(), 1.3 * u) - cen.begin());
        c.near[fam] = make_int2(a, std::max(a, b));
      }
    }
  // Partition of each tile's blocks into W warps of M chains.  With M = 2 a
  // chain runs the double-float tier over its own window; with M = 4 a warp
  // runs it over the hull of its chains' windows, so blocks whose windows
  // overlap are grouped.  The cost is the modelled packed-op
  // count (fast / double-float per line quad and chain: Ben-Reuven 10 / 16,
  // Gross 8 / 12, VVW 10 / 22), the objective half the sum and half W times
  // the largest warp (warps of a CTA meet at a barrier every chunk).
  auto group_cost = [&](int t, const std::vector<int>& g) {
    static const int fams[6] = {rb::FAM_NH3_INV, rb::FAM_NH3_ROT, rb::FAM_NH3_V2,
                                rb::FAM_H2O, rb::FAM_H2S, rb::FAM_PH3};
    static const double cf[6] = {10, 8, 8, 10, 10, 10}, cp[6] = {16, 12, 12, 22, 16, 16};
    // M = 2: each chain takes the double-float form inside its own window;
    // M = 4: every chain of the warp inside the hull of the windows
    double cost = 0.0;
    for (int q = 0; q < 6; ++q) {
      const int n = h->fam[fams[q]].n;
      if (n == 0) continue;
      int lo = n, hi = 0;
      for (int bk : g) {
        const int2 r = blocks[(size_t)t * nbk + bk].near[fams[q]];
        if (r.x < r.y) {
          lo = std::min(lo, r.x);
          hi = std::max(hi, r.y);
          if (M == 2) cost += (r.y - r.x) * (cp[q] - cf[q]);
        }
      }
      const int hull = M == 2 ? 0 : std::max(0, hi - lo);
      cost += (double)g.size() * ((n - hull) * cf[q] + hull * cp[q]);
    }
    return cost;
  };
  std::vector<rb::ChainPlan> chains((size_t)ntile * W * M);
  for (int t = 0; t < ntile; ++t) {
    std::vector<std::vector<int>> best(W, std::vector<int>(M));
    for (int w = 0; w < W; ++w)
      for (int k = 0; k < M; ++k) best[w][k] = k * W + w;   // default: interleaved
    if (W > 1 && nbk <= 8) {
      double best_obj = INFINITY;
      std::vector<std::vector<int>> cur;
      std::vector<int> used(nbk, 0);
      std::function<void()> rec = [&]() {
        int first = -1;
        for (int b = 0; b < nbk; ++b)
          if (!used[b]) { first = b; break; }
        if (first < 0) {
          double sum = 0.0, mx = 0.0;
          for (auto& g : cur) {
            const double c = group_cost(t, g);
            sum += c;
            mx = std::max(mx, c);
          }
          const double obj = 0.5 * sum + 0.5 * W * mx;
          if (obj < best_obj - 1e-9) {
            best_obj = obj;
            best = cur;
          }
          return;
        }
        // groups are built from the lowest unused block upward (each
        // unordered partition is visited once)
        std::vector<int> g{first};
        used[first] = 1;
        std::function<void(int)> pick = [&](int from) {
          if ((int)g.size() == M) {
            cur.push_back(g);
            rec();
            cur.pop_back();
            return;
          }
          for (int b = from; b < nbk; ++b) {
            if (used[b]) continue;
            used[b] = 1;
            g.push_back(b);
            pick(b + 1);
            g.pop_back();
            used[b] = 0;
          }
        };
        pick(first + 1);
        used[first] = 0;
      };
      rec();
    }
    for (int w = 0; w < W; ++w) {
      std::sort(best[w].begin(), best[w].end());
      for (int k = 0; k < M; ++k) chains[((size_t)t * W + w) * M + k] = blocks[(size_t)t * nbk + best[w][k]];
    }
  }
  // per warp: chains [0, KS) take inversion set 0, chain KS may mix both
  // sets, the rest take set 1 (slots are in frequency order, so the set is
  // monotone in the chain index); chains without a valid slot follow the
  // set-1 records when the tile builds them, else the set-0 records.
  std::vector<int> wsets((size_t)ntile * W, M);
  for (int t = 0; t < ntile; ++t)
    for (int w = 0; w < W; ++w) {
      int ks = 0;
      bool mix = false;
      for (int k = 0; k < M; ++k) {
        const int f = chains[((size_t)t * W + w) * M + k].flags;
        const bool set0_only = (f & rb::CH_VALID) ? !(f & rb::CH_SET1) : !(tflags[t] & rb::CH_SET1);
        if (set0_only && ks == k) {
          ++ks;
        } else if (ks == k && (f & rb::CH_SET0) && (f & rb::CH_SET1)) {
          mix = true;
        }
      }
      for (int k = ks + (mix ? 1 : 0); k < M; ++k) {   // the rest must take set 1
        const int f = chains[((size_t)t * W + w) * M + k].flags;
        if ((f & rb::CH_VALID) && (f & rb::CH_SET0))
          return fail(RB_ESTATE, "frequency plan: coefficient sets not monotone in a warp");
      }
      wsets[(size_t)t * W + w] = ks | (mix ? 256 : 0);
    }
  // template entries, heaviest family first
  const int order[rb::NFAM] = {rb::FAM_NH3_SJS, rb::FAM_NH3_INV, rb::FAM_H2O, rb::FAM_NH3_ROT,
                               rb::FAM_NH3_V2,  rb::FAM_H2S,     rb::FAM_PH3};
  // Lines per item scale with the per-line cost so items take similar time:
  // nh3_sjs (frequency-dependent widths, double-float everywhere) half the
  // base, the inversion lines (mostly double-float near 18-26 GHz) the
  // base, the others twice the base.
  const int base_lines = std::max(128, (h->item_lines > 0 ? h->item_lines : 1024) / 128 * 128);
  std::vector<rb::TmplEntry> tmpl;
  for (int v = 0; v < rb::NFAM; ++v) {
    const int fam = order[v];
    const int n = h->fam[fam].n;
    const int lines = fam == rb::FAM_NH3_SJS   ? std::max(128, base_lines / 2 / 128 * 128)
                      : fam == rb::FAM_NH3_INV ? base_lines
                                               : 2 * base_lines;
    h->plan_vbeg[fam] = (int)tmpl.size();
    for (int l0 = 0; l0 < n; l0 += lines) tmpl.push_back(rb::TmplEntry{fam, l0, std::min(n, l0 + lines), 0});
    h->plan_vend[fam] = (int)tmpl.size();
  }
  int dev_sms = 0;
  RB_CUDA(cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, h->device));
  const int occ = std::max(1, rb::alpha_lines_occupancy(M, W));
  RB_CUDA(upload(h->d_f, freqs, nf, st));
  RB_CUDA(upload(h->d_fhs, fhs.data(), nf, st));
  // per-frequency values of the absorption JVP (see rb::JvFreq)
  std::vector<rb::JvFreq> jfreq(nf);
  for (int i = 0; i < nf; ++i) {
    const double f = freqs[i], fh = fhs[i];
    rb::JvFreq& q = jfreq[i];
    rb::split_double(f * f, q.F, q.FL);
    rb::split_double(fh * fh, q.Fh, q.FhL);
    rb::split_double(f, q.fq, q.fql);
    q.set = fh > 30.0 ? 1 : 0;
    q.wJ = f <= 26.0 ? 0.f : (f >= 34.0 ? 1.f : (float)(f - 26.0) * 0.125f);   // (f - 26) / 8
  }
  RB_CUDA(upload(h->d_jfreq, jfreq.data(), jfreq.size(), st));
  RB_CUDA(upload(h->d_chains, chains.data(), chains.size(), st));
  RB_CUDA(upload(h->d_tflags, tflags.data(), tflags.size(), st));
  RB_CUDA(upload(h->d_wsets, wsets.data(), wsets.size(), st));
  RB_CUDA(upload(h->d_tmpl, tmpl.data(), tmpl.size(), st));
  RB_CUDA(upload(h->d_sj, slot_j.data(), slot_j.size(), st));
  RB_CUDA(upload(h->d_sF, sF.data(), sF.size(), st));
  RB_CUDA(upload(h->d_sFhs, sFhs.data(), sFhs.size(), st));
  RB_CUDA(upload(h->d_sf, sf.data(), sf.size(), st));
  RB_CUDA(upload(h->d_swJ, swJ.data(), swJ.size(), st));
  RB_CUDA(upload(h->d_sset, sset.data(), sset.size(), st));
  RB_CUDA(h->d_counter.ensure(sizeof(int)));
  RB_CUDA(cudaStreamSynchronize(st));
  h->plan_f.assign(freqs, freqs + nf);
  ++h->cfg_gen;
  h->plan_M = M;
  h->plan_W = W;
  h->plan_spt = spt;
  h->plan_ntile = ntile;
  h->plan_nslot = nslot;
  h->plan_ntmpl = (int)tmpl.size();
  h->plan_grid = dev_sms * occ;
  return RB_OK;
}

int validate_atm(int nL, const double* P, const double* T, const double* X) {
  if (nL < 1) return fail(RB_EINVAL, "nL must be >= 1");
  for (int i = 0; i < nL; ++i) {
    if (!(P[i] > 0.0) || !std::isfinite(P[i])) return fail(RB_EINVAL, "P[%d] must be > 0", i);
    if (!(T[i] > 0.0) || !std::isfinite(T[i])) return fail(RB_EINVAL, "T[%d] must be > 0", i);
  }
  if (!finite_all(X, (size_t)rb::NX * nL)) return fail(RB_EINVAL, "X has non-finite entries");
  return RB_OK;
}

// Arguments of the co_ddb / clouds_idp kernels (device inputs, d_extra
// already sized for nL layers).
void extra_args(rb_handle* h, rb::ExtraArgs& ea, int nL, const double* dP, const double* dT,
                const double* dX) {
  ea.nL = nL;
  ea.nf = (int)h->plan_f.size();
  ea.P = dP;
  ea.T = dT;
  ea.X = dX;
  ea.freqs = h->d_f.as<double>();
  ea.nco = h->nco;
  ea.co_f0 = h->d_co_f0.as<double>();
  ea.co_I0 = h->d_co_I0.as<double>();
  ea.co_E = h->d_co_E.as<double>();
  ea.cfg = h->cfg;
  ea.out = h->d_extra.as<double>();
}

// Layer prep arguments (d_lp must hold nL LayerParams).
static rb::PrepArgs prep_args(rb_handle* h, int nL, const double* dP, const double* dT,
                              const double* dX, const double* dscale, int units_db) {
  rb::PrepArgs pa{};
  pa.nL = nL;
  pa.P = dP;
  pa.T = dT;
  pa.X = dX;
  pa.scale = dscale;
  pa.cfg = h->cfg;
  pa.cfg.units_db = units_db;
  for (int f = 0; f < rb::NFAM; ++f) {
    pa.l2Imax[f] = h->fam[f].l2Imax;
    pa.Emin[f] = h->fam[f].Emin;
    pa.Emax[f] = h->fam[f].Emax;
    pa.cmax[f] = h->fam[f].n > 0 ? (float)h->fam[f].centre.back() : 0.f;
    pa.nlines[f] = h->fam[f].n;
  }
  pa.out = h->d_lp.as<rb::LayerParams>();
  pa.counter = h->d_counter.as<int>();
  return pa;
}

// Layer tangents and the JVP of the stored-tangent adjoint (launched in
// place of the forward line sums).
struct AlphaJvp {
  rb::TanArgs tn;
  rb::JvpArgs jv;
};

// Stored-tangent forward absorption: prep, [co / clouds,] layer tangents and
// the JVP, which writes the scan's float32 alpha into d_a32 and
// d alpha / d theta into d_dal.
static int enqueue_alpha_jvp(rb_handle* h, cudaStream_t st, int nL, const double* dP,
                             const double* dT, const double* dX, const double* dscale,
                             const AlphaJvp& aj) {
  const int nf = (int)h->plan_f.size();
  RB_CUDA(h->d_lp.ensure(sizeof(rb::LayerParams) * (size_t)nL));
  RB_CUDA(h->d_a32.ensure(sizeof(float) * (size_t)nL * nf));
  RB_CUDA(h->d_lt.ensure(sizeof(rb::LayerTan) * nL));
  RB_CUDA(h->d_dal.ensure(sizeof(float) * (size_t)nL * rb::NTH * nf));
  const rb::PrepArgs pa = prep_args(h, nL, dP, dT, dX, dscale, 0);
  rb::TanArgs tn = aj.tn;
  tn.out = h->d_lt.as<rb::LayerTan>();
  rb::JvpArgs jv = aj.jv;
  jv.lp = h->d_lp.as<rb::LayerParams>();
  jv.lt = h->d_lt.as<rb::LayerTan>();
  jv.alpha_out = h->d_a32.as<float>();
  jv.dal_out = h->d_dal.as<float>();
  jv.galpha = nullptr;
  jv.extra = nullptr;
  rb::ExtraArgs ea{};
  const bool extra = h->cfg.use_co || h->cfg.use_clouds;
  if (extra) {
    if (h->cfg.use_co && h->nco == 0) return fail(RB_ESTATE, "co_ddb selected but no CO lines uploaded");
    RB_CUDA(h->d_extra.ensure(sizeof(double) * 2 * (size_t)nL * nf));
    extra_args(h, ea, nL, dP, dT, dX);
    jv.extra = ea.out;
  }
  if (h->profiling) RB_CUDA(cudaEventRecord(h->pev[0], st));
  RB_CUDA(rb::launch_prep(pa, st));
  if (extra) RB_CUDA(rb::launch_extra(ea, st));
  if (h->profiling) RB_CUDA(cudaEventRecord(h->pev[1], st));
  RB_CUDA(rb::launch_jvp_store(tn, jv, st));
  if (h->profiling) RB_CUDA(cudaEventRecord(h->pev[8], st));
  if (h->profiling) RB_CUDA(cudaEventRecord(h->pev[2], st));
  h->launches += (extra ? 1 : 0) + 3;   // prep, [extra,] tangents, JVP
  return RB_OK;
}

int enqueue_alpha(rb_handle* h, cudaStream_t st, int nL, const double* dP, const double* dT,
                  const double* dX, const double* dscale, int units_db, double* d_layers64,
                  double* d_gas64) {
  RB_CUDA(h->d_lp.ensure(sizeof(rb::LayerParams) * (size_t)nL));
  const int nf = (int)h->plan_f.size();
  RB_CUDA(h->d_a32.ensure(sizeof(float) * (size_t)nL * nf));
  const rb::PrepArgs pa = prep_args(h, nL, dP, dT, dX, dscale, units_db);
  rb::AlphaArgs aa{};
  aa.nL = nL;
  aa.nf = nf;
  aa.nslot = h->plan_nslot;
  aa.M = h->plan_M;
  aa.W = h->plan_W;
  aa.spt = h->plan_spt;
  aa.ntile = h->plan_ntile;
  aa.sp.j = h->d_sj.as<int>();
  aa.sp.F = h->d_sF.as<float2>();
  aa.sp.Fhs = h->d_sFhs.as<float2>();
  aa.sp.f = h->d_sf.as<float2>();
  aa.sp.wJ = h->d_swJ.as<float>();
  aa.sp.set = h->d_sset.as<int>();
  aa.chains = h->d_chains.as<rb::ChainPlan>();
  aa.tile_flags = h->d_tflags.as<int>();
  aa.warp_sets = h->d_wsets.as<int>();
  aa.tmpl = h->d_tmpl.as<rb::TmplEntry>();
  aa.ntmpl = h->plan_ntmpl;
  for (int v = 0; v < rb::NFAM; ++v) {
    aa.vbeg[v] = h->plan_vbeg[v];
    aa.vend[v] = h->plan_vend[v];
    for (int t = h->plan_vbeg[v]; t < h->plan_vend[v] && t < 16; ++t) aa.tfam[t] = (unsigned char)v;
  }
  aa.nitems = aa.ntmpl * nL * aa.ntile;
  aa.counter = h->d_counter.as<int>();
  RB_CUDA(h->d_res.ensure(sizeof(float) * std::max<size_t>(1, (size_t)nL * aa.ntile * aa.ntmpl * aa.spt)));
  RB_CUDA(h->d_base.ensure(sizeof(float) * std::max<size_t>(1, (size_t)nL * aa.ntile * aa.ntmpl)));
  aa.res = h->d_res.as<float>();
  aa.base = h->d_base.as<float>();
  aa.freqs = h->d_f.as<double>();
  aa.freqs_hs = h->d_fhs.as<double>();
  aa.lp = h->d_lp.as<rb::LayerParams>();
  for (int f = 0; f < rb::NFAM; ++f) aa.tab[f] = h->fam[f].table();
  aa.cfg = pa.cfg;
  aa.alpha32 = h->d_a32.as<float>();
  aa.layers64 = d_layers64;
  aa.gas64 = d_gas64;
  aa.extra = nullptr;
  rb::ExtraArgs ea{};
  const bool extra = h->cfg.use_co || h->cfg.use_clouds;
  if (extra) {
    if (h->cfg.use_co && h->nco == 0) return fail(RB_ESTATE, "co_ddb selected but no CO lines uploaded");
    RB_CUDA(h->d_extra.ensure(sizeof(double) * 2 * (size_t)nL * nf));
    extra_args(h, ea, nL, dP, dT, dX);
    aa.extra = ea.out;
  }
  if (h->profiling) RB_CUDA(cudaEventRecord(h->pev[0], st));
  RB_CUDA(rb::launch_prep(pa, st));
  if (extra) RB_CUDA(rb::launch_extra(ea, st));
  if (h->profiling) RB_CUDA(cudaEventRecord(h->pev[1], st));
  RB_CUDA(rb::launch_alpha_lines(aa, h->plan_grid, st));
  if (h->profiling) RB_CUDA(cudaEventRecord(h->pev[8], st));
  RB_CUDA(rb::launch_alpha_assemble(aa, st));
  if (h->profiling) RB_CUDA(cudaEventRecord(h->pev[2], st));
  // prep, [extra,] [line sums,] assembly
  h->launches += (extra ? 1 : 0) + 1 + (aa.nitems > 0 ? 2 : 1);
  return RB_OK;
}

void aspect_matrix(double Req, double Rpol, double o0, double o1, double* M) {
  // computeAspect (raypath.py:39-44) and rotate2planet = rotX(rotate) rotZ(tip)
  const double f = 1.0 - Rpol / Req;
  const double tip = -o0 * M_PI / 180.0;
  const double rotate = -std::atan(std::tan(o1 * M_PI / 180.0) * (1.0 - f) * (1.0 - f));
  const double cz = std::cos(tip), sz = std::sin(tip), cx = std::cos(rotate), sx = std::sin(rotate);
  M[0] = cz;
  M[1] = -sz;
  M[2] = 0.0;
  M[3] = cx * sz;
  M[4] = cx * cz;
  M[5] = -sx;
  M[6] = sx * sz;
  M[7] = sx * cz;
  M[8] = cx;
}

// Geometry tables (float radii differences, float T) then the ray walk.
// T may be null (no float temperature table needed).
// Ray count from which the ray set-up runs one ray per thread in its own kernel.
constexpr int RAY_SETUP_KERNEL_MIN = 2048;

int enqueue_raypath(rb_handle* h, cudaStream_t st, int nL, const double* dR, const double* dN,
                    const double* dT, double Req, double Rpol, double o0, double o1, int gtype,
                    int limb, int nb, const double* db, int max_seg, int* dnseg, double* dds,
                    float* dhds, int* dlayer, double* dr4, double* dll, int* dend,
                    const Batch* bt = nullptr, int rays_per_var = 0) {
  RB_CUDA(h->d_dR.ensure(sizeof(float) * nL));
  RB_CUDA(h->d_sR.ensure(sizeof(float2) * nL));
  RB_CUDA(h->d_R32.ensure(sizeof(float) * nL));
  RB_CUDA(h->d_T32.ensure(sizeof(float) * nL));
  RB_CUDA(rb::launch_geom_prep(nL, dR, dT, h->d_sR.as<float2>(), h->d_dR.as<float>(),
                               h->d_R32.as<float>(), h->d_T32.as<float>(), bt ? bt->d_off : nullptr,
                               bt ? bt->nvar : 1, st));
  rb::RayArgs ra{};
  ra.nL = nL;
  ra.var_off = bt ? bt->d_off : nullptr;
  ra.rays_per_var = rays_per_var;
  ra.R = dR;
  ra.N = dN;
  ra.dR2 = h->d_sR.as<float2>();
  ra.dR = h->d_dR.as<float>();
  ra.R32 = h->d_R32.as<float>();
  ra.k = gtype == RB_GTYPE_ELLIPSE ? Rpol / Req : 1.0;
  aspect_matrix(Req, Rpol, o0, o1, ra.rot);
  ra.limb_sec = limb == RB_LIMB_SEC;
  ra.nb = nb;
  ra.b = db;
  ra.max_seg = max_seg;
  ra.nseg = dnseg;
  ra.ds = dds;
  ra.hds = dhds;
  ra.layer = dlayer;
  ra.r4ds = dr4;
  ra.latlng = dll;
  ra.end_code = dend;
  // The float64 set-up of a ray (findEdge, first refraction) costs the same
  // per warp instruction for one lane as for 32: with many rays it runs one
  // ray per thread in its own kernel; with few, inside the walk's warp, so
  // the walk starts (and takes its SM slots, ahead of the line sums on the
  // other stream) without waiting for a second launch.
  const bool setup_kernel = nb >= RAY_SETUP_KERNEL_MIN;
  if (setup_kernel) {
    RB_CUDA(h->d_rstart.ensure(sizeof(rb::RayStart) * nb));
    ra.start = h->d_rstart.as<rb::RayStart>();
  }
  if (h->profiling) RB_CUDA(cudaEventRecord(h->pev[3], st));
  RB_CUDA(rb::launch_raypath(ra, st));
  if (h->profiling) RB_CUDA(cudaEventRecord(h->pev[4], st));
  h->launches += nb > 0 ? (setup_kernel ? 3 : 2) : 1;
  return RB_OK;
}

int validate_geom(int nL, const double* R, const double* N, double Req, double Rpol, int gtype,
                  int limb, int nb, const double* b) {
  if (nL < 2) return fail(RB_EINVAL, "ray paths need nL >= 2");
  if (!(Req > 0.0) || !(Rpol > 0.0)) return fail(RB_EINVAL, "Req and Rpol must be > 0");
  if (gtype != RB_GTYPE_ELLIPSE && gtype != RB_GTYPE_SPHERE)
    return fail(RB_EINVAL, "gtype must be RB_GTYPE_ELLIPSE or RB_GTYPE_SPHERE");
  if (limb != RB_LIMB_SHAPE && limb != RB_LIMB_SEC)
    return fail(RB_EINVAL, "limb must be RB_LIMB_SHAPE or RB_LIMB_SEC");
  if (nb < 0) return fail(RB_EINVAL, "nb must be >= 0");
  if (!finite_all(R, nL) || !finite_all(N, nL)) return fail(RB_EINVAL, "R/N not finite");
  if (!(R[0] > 0.0)) return fail(RB_EINVAL, "R[0] must be > 0");
  if (nb && !finite_all(b, 2 * (size_t)nb)) return fail(RB_EINVAL, "b not finite");
  return RB_OK;
}

}  // namespace

extern "C" {

int rb_abi_version(void) { return RB_ABI_VERSION; }

const char* rb_last_error(void) { return g_err.c_str(); }

int rb_create(rb_handle** out, int device) {
  if (!out) return fail(RB_EINVAL, "out is null");
  *out = nullptr;
  int ndev = 0;
  RB_CUDA(cudaGetDeviceCount(&ndev));
  if (device < 0 || device >= ndev) return fail(RB_EINVAL, "device %d not present (%d)", device, ndev);
  RB_CUDA(cudaSetDevice(device));
  rb_handle* h = new rb_handle();
  h->device = device;
  cudaError_t e = cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->side, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_dev, cudaEventDisableTiming);
  size_t mem_free = 0;
  if (e == cudaSuccess) e = cudaMemGetInfo(&mem_free, &h->dev_mem);
  if (e != cudaSuccess) {
    rb_destroy(h);
    return fail(RB_ECUDA, "stream/event creation: %s", cudaGetErrorString(e));
  }
  *out = h;
  return RB_OK;
}

int rb_destroy(rb_handle* h) {
  if (!h) return RB_OK;
  cudaSetDevice(h->device);
  if (h->st) cudaStreamSynchronize(h->st);
  if (h->side) cudaStreamSynchronize(h->side);
  for (auto& f : h->fam) f.release();
  for (DBuf* b : {&h->d_sj, &h->d_sF, &h->d_sFhs, &h->d_sf, &h->d_swJ, &h->d_sset, &h->d_dR,
                  &h->d_sR, &h->d_R32, &h->d_T32, &h->d_hds, &h->d_Tb32, &h->d_part, &h->d_rstart})
    b->release();
  for (DBuf* b : {&h->d_chains, &h->d_tflags, &h->d_wsets, &h->d_tmpl, &h->d_counter, &h->d_res, &h->d_base,
                  &h->d_ga, &h->d_gs, &h->d_lt, &h->d_jpart, &h->d_grad, &h->d_dth,
                  &h->d_adjS, &h->d_voff, &h->d_dal, &h->d_iw32, &h->d_co_f0, &h->d_co_I0, &h->d_co_E, &h->d_extra,
                  &h->d_xgrad, &h->d_agas, &h->d_acl, &h->d_aout, &h->d_aclout, &h->d_aprop,
                  &h->d_agrid, &h->d_aoff})
    b->release();
  for (DBuf* b : {&h->d_f, &h->d_fhs, &h->d_jfreq, &h->d_P, &h->d_T, &h->d_X, &h->d_scale, &h->d_lp,
                  &h->d_a32, &h->d_l64, &h->d_g64, &h->d_R, &h->d_N, &h->d_b, &h->d_w, &h->d_nseg,
                  &h->d_ds, &h->d_layer, &h->d_r4, &h->d_ll, &h->d_end, &h->d_Tb, &h->d_avg,
                  &h->d_iw, &h->d_tau, &h->d_W, &h->d_tbl, &h->d_x})
    b->release();
  for (auto& e : h->pev)
    if (e) cudaEventDestroy(e);
  h->d_probe.release();
  h->d_in.release();
  h->h_in.release();
  h->h_out.release();
  h->g_fwd.release();
  h->g_adj.release();
  if (h->ev_fork) cudaEventDestroy(h->ev_fork);
  if (h->ev_join) cudaEventDestroy(h->ev_join);
  if (h->ev_dev) cudaEventDestroy(h->ev_dev);
  if (h->st) cudaStreamDestroy(h->st);
  if (h->side) cudaStreamDestroy(h->side);
  delete h;
  return RB_OK;
}

// co_ddb lines: f0, I0, E kept in float64 (no line-sum kernel involved).
static int set_co_lines(rb_handle* h, int n, int ncols, const double* cols) {
  if (ncols != 3) return fail(RB_EINVAL, "family %d takes 3 columns, got %d", RB_FAM_CO, ncols);
  if (n < 0 || (n > 0 && !cols)) return fail(RB_EINVAL, "bad line count / pointer");
  if (!finite_all(cols, (size_t)n * 3)) return fail(RB_EINVAL, "line columns not finite");
  for (int i = 0; i < n; ++i)
    if (!(cols[i] > 0.0)) return fail(RB_EINVAL, "line %d: centre must be > 0", i);
  RB_CUDA(cudaSetDevice(h->device));
  RB_CUDA(order_after_device(h, h->st));
  h->nco = 0;
  cudaStream_t st = h->st;
  RB_CUDA(upload(h->d_co_f0, cols, n, st));
  RB_CUDA(upload(h->d_co_I0, cols + n, n, st));
  RB_CUDA(upload(h->d_co_E, cols + 2 * (size_t)n, n, st));
  RB_CUDA(cudaStreamSynchronize(st));
  h->nco = n;
  return RB_OK;
}

int rb_set_lines(rb_handle* h, int family, int n, int ncols, const double* cols) {
  if (!h) return fail(RB_EINVAL, "null handle");
  ++h->cfg_gen;
  if (family == RB_FAM_CO) return set_co_lines(h, n, ncols, cols);
  if (family < 0 || family >= rb::NFAM) return fail(RB_EINVAL, "unknown family %d", family);
  if (ncols != family_ncols(family))
    return fail(RB_EINVAL, "family %d takes %d columns, got %d", family, family_ncols(family), ncols);
  if (n < 0 || (n > 0 && !cols)) return fail(RB_EINVAL, "bad line count / pointer");
  RB_CUDA(cudaSetDevice(h->device));
  RB_CUDA(order_after_device(h, h->st));
  FamilyStore& F = h->fam[family];
  h->plan_f.clear();
  if (!finite_all(cols, (size_t)n * ncols)) return fail(RB_EINVAL, "line columns not finite");
  auto col = [&](int c, int i) { return cols[(size_t)c * n + i]; };
  std::vector<double> centre(n);
  for (int i = 0; i < n; ++i) {
    const double fo = col(0, i);
    if (!(fo > 0.0) || fo > 2.0e4)
      return fail(RB_EINVAL, "line %d: centre %g GHz outside (0, 2e4]", i, fo);
    const double I = col(1, i);
    if (I < 0.0) return fail(RB_EINVAL, "line %d: negative intensity", i);
    centre[i] = family == rb::FAM_H2O ? fo + col(9, i) : fo;
    if (family == rb::FAM_H2O && !(centre[i] > 0.0))
      return fail(RB_EINVAL, "line %d: f_o + SR must be > 0", i);
  }
  std::vector<int> order(n);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return centre[a] < centre[b]; });
  std::vector<float> c2h(n), c2l(n), ch(n), cl(n), w1(n), w2(n), w3(n), x1(n), x2(n), x3(n),
      l2Ih(n), l2Il(n), Eh(n), El(n);
  std::vector<double> cs(n);
  double l2max = -INFINITY, emin = INFINITY, emax = -INFINITY;
  for (int k = 0; k < n; ++k) {
    const int i = order[k];
    const double fo = col(0, i);
    const double I = col(1, i);
    cs[k] = centre[i];
    rb::split_double(fo * fo, c2h[k], c2l[k]);
    rb::split_double(centre[i], ch[k], cl[k]);
    const double E = col(2, i);
    rb::split_double(E, Eh[k], El[k]);
    double lI = I > 0.0 ? std::log(I) : -INFINITY;
    w1[k] = w2[k] = w3[k] = 0.f;
    x1[k] = x2[k] = x3[k] = 0.f;
    switch (family) {
      case rb::FAM_NH3_INV:  // fo Io Eo gammaNH3o
        lI -= 2.0 * std::log(fo);
        w1[k] = (float)col(3, i);
        break;
      case rb::FAM_NH3_ROT:  // fo Io Eo gNH3 gH2 gHe
        w1[k] = (float)col(4, i);
        w2[k] = (float)col(5, i);
        w3[k] = (float)col(3, i);
        break;
      case rb::FAM_NH3_V2:   // fixed widths (nh3_hs.py:272-274)
        w1[k] = 1.4f;
        w2[k] = 0.68f;
        w3[k] = 9.5f;
        break;
      case rb::FAM_NH3_SJS:  // f0 I0 E G0
      case rb::FAM_H2S:      // f0 I0 E GH2S
        lI -= 2.0 * std::log(fo);
        w1[k] = (float)col(3, i);
        break;
      case rb::FAM_PH3: {    // f0 I0 E WgtI0 WgtFGB WgtSB
        const double wI = col(3, i);
        if (wI < 0.0) return fail(RB_EINVAL, "line %d: negative WgtI0", i);
        lI = (I > 0.0 && wI > 0.0) ? std::log(I * wI) - 2.0 * std::log(fo) : -INFINITY;
        w1[k] = (float)col(4, i);
        w2[k] = (float)col(5, i);
        break;
      }
      case rb::FAM_H2O:      // f_o I_o E_o w_s x_s w_h2 w_he x_h2 x_he SR
        lI -= 2.0 * std::log(fo) + std::log(M_PI);
        w1[k] = (float)col(3, i);
        x1[k] = (float)col(4, i);
        w2[k] = (float)col(5, i);
        x2[k] = (float)col(7, i);
        w3[k] = (float)col(6, i);
        x3[k] = (float)col(8, i);
        break;
    }
    const double l2 = lI * 1.4426950408889634;     // log2
    if (std::isfinite(l2)) {
      rb::split_double(l2, l2Ih[k], l2Il[k]);
      l2max = std::max(l2max, l2);
    } else {
      l2Ih[k] = -1.0e30f;                           // zero strength
      l2Il[k] = 0.f;
    }
    emin = std::min(emin, E);
    emax = std::max(emax, E);
  }
  F.n = 0;
  F.centre = cs;
  F.l2Imax = n > 0 && std::isfinite(l2max) ? (float)l2max + 1e-3f : 0.f;
  F.Emin = n > 0 ? (float)emin : 0.f;
  F.Emax = n > 0 ? (float)emax : 0.f;
  cudaStream_t st = h->st;
  RB_CUDA(upload(F.c2h, c2h.data(), n, st));
  RB_CUDA(upload(F.c2l, c2l.data(), n, st));
  RB_CUDA(upload(F.ch, ch.data(), n, st));
  RB_CUDA(upload(F.cl, cl.data(), n, st));
  RB_CUDA(upload(F.l2Ih, l2Ih.data(), n, st));
  RB_CUDA(upload(F.l2Il, l2Il.data(), n, st));
  RB_CUDA(upload(F.Eh, Eh.data(), n, st));
  RB_CUDA(upload(F.El, El.data(), n, st));
  RB_CUDA(upload(F.w1, w1.data(), n, st));
  RB_CUDA(upload(F.w2, w2.data(), n, st));
  RB_CUDA(upload(F.w3, w3.data(), n, st));
  RB_CUDA(upload(F.x1, x1.data(), n, st));
  RB_CUDA(upload(F.x2, x2.data(), n, st));
  RB_CUDA(upload(F.x3, x3.data(), n, st));
  RB_CUDA(cudaStreamSynchronize(st));
  F.n = n;
  return RB_OK;
}

int rb_set_formalisms(rb_handle* h, int nh3, int use_h2, int use_h2o, int use_h2s, int use_ph3,
                      int h2state) {
  if (!h) return fail(RB_EINVAL, "null handle");
  ++h->cfg_gen;
  if (nh3 < RB_NH3_OFF || nh3 > RB_NH3_DBS_SJS) return fail(RB_EINVAL, "bad nh3 formalism %d", nh3);
  if (h2state != 'e' && h2state != 'n') return fail(RB_EINVAL, "h2state must be 'e' or 'n'");
  // nh3_dbs / nh3_dbs_sjs: the nh3_hs / nh3_hs_sjs structure with the
  // nh3_dbs inversion coefficients (nh3_dbs_sjs.py:6-26 blends nh3_dbs
  // with nh3_sjs exactly as nh3_hs_sjs blends nh3_hs)
  h->cfg.inv_table = (nh3 == RB_NH3_DBS || nh3 == RB_NH3_DBS_SJS) ? 1 : 0;
  h->cfg.nh3_mode = nh3 == RB_NH3_DBS ? rb::NH3_HS : (nh3 == RB_NH3_DBS_SJS ? rb::NH3_HS_SJS : nh3);
  h->cfg.use_h2 = use_h2 != 0;
  h->cfg.use_h2o = use_h2o != 0;
  h->cfg.use_h2s = use_h2s != 0;
  h->cfg.use_ph3 = use_ph3 != 0;
  h->cfg.h2state = h2state;
  return RB_OK;
}

int rb_set_co_clouds(rb_handle* h, int co, int coshape, int clouds, int cloud_mask) {
  if (!h) return fail(RB_EINVAL, "null handle");
  ++h->cfg_gen;
  if (coshape < RB_COSHAPE_VOIGT || coshape > RB_COSHAPE_STD) return fail(RB_EINVAL, "bad coshape %d", coshape);
  if (cloud_mask & ~63) return fail(RB_EINVAL, "bad cloud mask %d", cloud_mask);
  h->cfg.use_co = co != 0;
  h->cfg.coshape = coshape;
  h->cfg.use_clouds = clouds != 0;
  h->cfg.cloud_mask = cloud_mask;
  return RB_OK;
}

int rb_set_alpha_tiling(rb_handle* h, int M, int W, int item_lines) {
  if (!h) return fail(RB_EINVAL, "null handle");
  ++h->cfg_gen;
  if (!(M == 0 || M == 2 || M == 4)) return fail(RB_EINVAL, "M must be 0, 2 or 4");
  if (W < 0 || W > 4) return fail(RB_EINVAL, "W must be in 0..4");
  if ((M == 0) != (W == 0)) return fail(RB_EINVAL, "M and W are set together");
  if (item_lines < 0 || item_lines % 128) return fail(RB_EINVAL, "item_lines must be a multiple of 128");
  h->tile_M = M;
  h->tile_W = W;
  h->item_lines = item_lines;
  h->plan_f.clear();
  return RB_OK;
}

int rb_set_tuning(rb_handle* h, int param, int value) {
  if (!h) return fail(RB_EINVAL, "null handle");
  const bool pow2 = value > 0 && (value & (value - 1)) == 0;
  switch (param) {
    case RB_TUNE_JVP_FREQS:
      if (!(value == 0 || value == 32 || value == 64 || value == 128))
        return fail(RB_EINVAL, "RB_TUNE_JVP_FREQS must be 0, 32, 64 or 128");
      h->jvp_ft = value;
      break;
    case RB_TUNE_JVP_CTAS:
      if (!(value == 0 || (value >= 3 && value <= 6)))
        return fail(RB_EINVAL, "RB_TUNE_JVP_CTAS must be 0 or 3..6");
      h->jvp_ctas = value;
      break;
    case RB_TUNE_JVP_THREADS:
      if (!(value == 0 || value == 128 || value == 256))
        return fail(RB_EINVAL, "RB_TUNE_JVP_THREADS must be 0, 128 or 256");
      h->jvp_threads = value;
      break;
    case RB_TUNE_SCAN_LANES:
      if (!(value == 0 || (pow2 && value >= 4 && value <= 128)))
        return fail(RB_EINVAL, "RB_TUNE_SCAN_LANES must be 0 or a power of two in 4..128");
      h->scan_lanes = value;
      break;
    case RB_TUNE_ADJ_MODE:
      if (value < 0 || value > 2) return fail(RB_EINVAL, "RB_TUNE_ADJ_MODE must be 0, 1 or 2");
      h->adj_mode = value;
      break;
    default:
      return fail(RB_EINVAL, "unknown tuning parameter %d", param);
  }
  ++h->cfg_gen;
  return RB_OK;
}

int rb_alpha(rb_handle* h, int nL, const double* P, const double* T, const double* X, int nf,
             const double* freqs, const double* scale, int units_db, double* layers_out,
             double* gas_out) {
  if (!h) return fail(RB_EINVAL, "null handle");
  if (!P || !T || !X || !freqs) return fail(RB_EINVAL, "null input array");
  int rc = validate_atm(nL, P, T, X);
  if (rc) return rc;
  if (scale && !finite_all(scale, (size_t)nL * rb::NGAS)) return fail(RB_EINVAL, "scale not finite");
  RB_CUDA(cudaSetDevice(h->device));
  RB_CUDA(order_after_device(h, h->st));
  cudaStream_t st = h->st;
  if ((rc = plan_frequencies(h, nf, freqs, st))) return rc;
  RB_CUDA(upload(h->d_P, P, nL, st));
  RB_CUDA(upload(h->d_T, T, nL, st));
  RB_CUDA(upload(h->d_X, X, (size_t)rb::NX * nL, st));
  const double* dscale = nullptr;
  if (scale) {
    RB_CUDA(upload(h->d_scale, scale, (size_t)nL * rb::NGAS, st));
    dscale = h->d_scale.as<double>();
  }
  double* dl = nullptr;
  double* dg = nullptr;
  if (layers_out) {
    RB_CUDA(h->d_l64.ensure(sizeof(double) * (size_t)nf * nL));
    dl = h->d_l64.as<double>();
  }
  if (gas_out) {
    RB_CUDA(h->d_g64.ensure(sizeof(double) * (size_t)nf * nL * rb::NGAS));
    dg = h->d_g64.as<double>();
  }
  h->launches = 0;
  if ((rc = enqueue_alpha(h, st, nL, h->d_P.as<double>(), h->d_T.as<double>(), h->d_X.as<double>(),
                          dscale, units_db, dl, dg)))
    return rc;
  if (dl) RB_CUDA(cudaMemcpyAsync(layers_out, dl, sizeof(double) * (size_t)nf * nL, cudaMemcpyDeviceToHost, st));
  if (dg)
    RB_CUDA(cudaMemcpyAsync(gas_out, dg, sizeof(double) * (size_t)nf * nL * rb::NGAS,
                            cudaMemcpyDeviceToHost, st));
  RB_CUDA(cudaStreamSynchronize(st));
  return RB_OK;
}

int rb_raypath(rb_handle* h, int nL, const double* R, const double* N, double Req, double Rpol,
               double orient0, double orient1, int gtype, int limb, int nb, const double* b,
               int max_seg, int32_t* nseg, double* ds, int32_t* layer, double* r4ds,
               double* latlng, int32_t* end_code) {
  if (!h) return fail(RB_EINVAL, "null handle");
  if (!R || !N || (nb > 0 && (!b || !nseg || !ds || !layer))) return fail(RB_EINVAL, "null array");
  int rc = validate_geom(nL, R, N, Req, Rpol, gtype, limb, nb, b);
  if (rc) return rc;
  if (max_seg < 1) return fail(RB_EINVAL, "max_seg must be >= 1");
  if (nb == 0) return RB_OK;
  RB_CUDA(cudaSetDevice(h->device));
  RB_CUDA(order_after_device(h, h->st));
  cudaStream_t st = h->st;
  RB_CUDA(upload(h->d_R, R, nL, st));
  RB_CUDA(upload(h->d_N, N, nL, st));
  RB_CUDA(upload(h->d_b, b, 2 * (size_t)nb, st));
  const size_t ns = (size_t)nb * max_seg;
  RB_CUDA(h->d_nseg.ensure(sizeof(int) * nb));
  RB_CUDA(h->d_end.ensure(sizeof(int) * nb));
  RB_CUDA(h->d_ds.ensure(sizeof(double) * ns));
  RB_CUDA(h->d_layer.ensure(sizeof(int) * ns));
  if (r4ds) RB_CUDA(h->d_r4.ensure(sizeof(double) * ns));
  if (latlng) RB_CUDA(h->d_ll.ensure(sizeof(double) * (size_t)nb * (max_seg + 1) * 2));
  h->launches = 0;
  if ((rc = enqueue_raypath(h, st, nL, h->d_R.as<double>(), h->d_N.as<double>(), nullptr, Req,
                            Rpol, orient0, orient1, gtype, limb, nb, h->d_b.as<double>(), max_seg,
                            h->d_nseg.as<int>(), h->d_ds.as<double>(), nullptr,
                            h->d_layer.as<int>(), r4ds ? h->d_r4.as<double>() : nullptr,
                            latlng ? h->d_ll.as<double>() : nullptr, h->d_end.as<int>())))
    return rc;
  RB_CUDA(cudaMemcpyAsync(nseg, h->d_nseg.p, sizeof(int) * nb, cudaMemcpyDeviceToHost, st));
  RB_CUDA(cudaMemcpyAsync(ds, h->d_ds.p, sizeof(double) * ns, cudaMemcpyDeviceToHost, st));
  RB_CUDA(cudaMemcpyAsync(layer, h->d_layer.p, sizeof(int) * ns, cudaMemcpyDeviceToHost, st));
  if (r4ds) RB_CUDA(cudaMemcpyAsync(r4ds, h->d_r4.p, sizeof(double) * ns, cudaMemcpyDeviceToHost, st));
  if (latlng)
    RB_CUDA(cudaMemcpyAsync(latlng, h->d_ll.p, sizeof(double) * (size_t)nb * (max_seg + 1) * 2,
                            cudaMemcpyDeviceToHost, st));
  if (end_code) RB_CUDA(cudaMemcpyAsync(end_code, h->d_end.p, sizeof(int) * nb, cudaMemcpyDeviceToHost, st));
  RB_CUDA(cudaStreamSynchronize(st));
  return RB_OK;
}

int rb_brightness(rb_handle* h, int nL, const double* T, int nf, const double* layers, int nb,
                  const int32_t* nseg, const double* ds, const int32_t* layer, int max_seg,
                  int disc, double* Tb_out, double* intW_out, double* tau_out, double* W_out,
                  double* TbL_out) {
  if (!h) return fail(RB_EINVAL, "null handle");
  if (nL < 1 || nf < 1 || nb < 0 || max_seg < 1) return fail(RB_EINVAL, "bad sizes");
  if (!T || !layers || (nb > 0 && (!nseg || !ds || !layer || !Tb_out))) return fail(RB_EINVAL, "null array");
  const bool prof = tau_out || W_out || TbL_out;
  if (prof && !(tau_out && W_out && TbL_out)) return fail(RB_EINVAL, "profiles need tau, W and TbL");
  if (nb == 0) return RB_OK;
  for (int r = 0; r < nb; ++r) {
    if (nseg[r] < 0 || nseg[r] > max_seg) return fail(RB_EINVAL, "nseg[%d] out of range", r);
    for (int i = 0; i < nseg[r]; ++i) {
      const int l = layer[(size_t)r * max_seg + i];
      if (l < -nL || l >= nL) return fail(RB_EINVAL, "layer index %d out of range", l);
    }
  }
  RB_CUDA(cudaSetDevice(h->device));
  RB_CUDA(order_after_device(h, h->st));
  cudaStream_t st = h->st;
  // absorption as float32 [nL][nf], T as float, ds/2 in cm as float
  std::vector<float> a32((size_t)nL * nf), t32(nL), hd((size_t)nb * max_seg, 0.f);
  for (int f = 0; f < nf; ++f)
    for (int l = 0; l < nL; ++l) a32[(size_t)l * nf + f] = (float)layers[(size_t)f * nL + l];
  for (int l = 0; l < nL; ++l) t32[l] = (float)T[l];
  for (int r = 0; r < nb; ++r)
    for (int i = 0; i < nseg[r]; ++i)
      hd[(size_t)r * max_seg + i] = (float)(ds[(size_t)r * max_seg + i] * 1.0e3 / 1.0e-2 / 2.0);
  RB_CUDA(upload(h->d_a32, a32.data(), a32.size(), st));
  RB_CUDA(upload(h->d_T32, t32.data(), t32.size(), st));
  RB_CUDA(upload(h->d_nseg, nseg, nb, st));
  RB_CUDA(upload(h->d_hds, hd.data(), hd.size(), st));
  RB_CUDA(upload(h->d_layer, layer, (size_t)nb * max_seg, st));
  RB_CUDA(h->d_Tb.ensure(sizeof(double) * (size_t)nb * nf));
  RB_CUDA(h->d_iw.ensure(sizeof(double) * (size_t)nb * nf));
  const size_t np = (size_t)nb * nf * max_seg;
  if (prof) {
    RB_CUDA(h->d_tau.ensure(sizeof(double) * np));
    RB_CUDA(h->d_W.ensure(sizeof(double) * np));
    RB_CUDA(h->d_tbl.ensure(sizeof(double) * np));
  }
  rb::TbArgs ta{};
  ta.nL = nL;
  ta.nf = nf;
  ta.nb = nb;
  ta.max_seg = max_seg;
  ta.alpha32 = h->d_a32.as<float>();
  ta.T32 = h->d_T32.as<float>();
  ta.nseg = h->d_nseg.as<int>();
  ta.hds = h->d_hds.as<float>();
  ta.layer = h->d_layer.as<int>();
  ta.disc = disc != 0;
  ta.Tb = h->d_Tb.as<double>();
  ta.intW = h->d_iw.as<double>();
  ta.tau = prof ? h->d_tau.as<double>() : nullptr;
  ta.W = prof ? h->d_W.as<double>() : nullptr;
  ta.TbL = prof ? h->d_tbl.as<double>() : nullptr;
  if (prof || disc) {
    h->launches = 1;
    RB_CUDA(rb::launch_tb_seq(ta, st));
  } else {
    ta.nchunk = rb::tb_nchunk(max_seg);
    ta.lanes = h->scan_lanes;
    RB_CUDA(h->d_part.ensure(sizeof(float4) * (size_t)nb * ta.nchunk * nf));
    ta.part = h->d_part.as<float4>();
    h->launches = 2;
    RB_CUDA(rb::launch_tb_chunked(ta, st));
  }
  RB_CUDA(cudaMemcpyAsync(Tb_out, ta.Tb, sizeof(double) * (size_t)nb * nf, cudaMemcpyDeviceToHost, st));
  if (intW_out)
    RB_CUDA(cudaMemcpyAsync(intW_out, ta.intW, sizeof(double) * (size_t)nb * nf, cudaMemcpyDeviceToHost, st));
  if (prof) {
    RB_CUDA(cudaMemcpyAsync(tau_out, ta.tau, sizeof(double) * np, cudaMemcpyDeviceToHost, st));
    RB_CUDA(cudaMemcpyAsync(W_out, ta.W, sizeof(double) * np, cudaMemcpyDeviceToHost, st));
    RB_CUDA(cudaMemcpyAsync(TbL_out, ta.TbL, sizeof(double) * np, cudaMemcpyDeviceToHost, st));
  }
  RB_CUDA(cudaStreamSynchronize(st));
  return RB_OK;
}

// Planet.run's b loop (planet.py:118-133 -> planet_base.py:244-274 ->
// Brightness.single) for every ray of one atmosphere at once, given the
// absorption the run computed (Alpha.layers): ray paths into device
// buffers, then the chunked scan, the absorption uploaded once per call.
int rb_bright_run(rb_handle* h, int nL, const double* T, const double* R, const double* N,
                  double Req, double Rpol, double orient0, double orient1, int gtype, int limb,
                  int nf, const double* layers, int nb, const double* b, double* Tb_out,
                  double* intW_out, int32_t* nseg_out) {
  if (!h) return fail(RB_EINVAL, "null handle");
  if (nf < 1) return fail(RB_EINVAL, "nf must be >= 1");
  if (!T || !R || !N || !layers || (nb > 0 && (!b || !Tb_out))) return fail(RB_EINVAL, "null array");
  int rc = validate_geom(nL, R, N, Req, Rpol, gtype, limb, nb, b);
  if (rc) return rc;
  if (!finite_all(T, nL)) return fail(RB_EINVAL, "T not finite");
  if (!finite_all(layers, (size_t)nf * nL)) return fail(RB_EINVAL, "layers not finite");
  if (nb == 0) return RB_OK;
  RB_CUDA(cudaSetDevice(h->device));
  RB_CUDA(order_after_device(h, h->st));
  cudaStream_t st = h->st;
  const int max_seg = 2 * nL + 4;
  const size_t ns = (size_t)nb * max_seg;
  std::vector<float> a32((size_t)nL * nf);
  for (int f = 0; f < nf; ++f)
    for (int l = 0; l < nL; ++l) a32[(size_t)l * nf + f] = (float)layers[(size_t)f * nL + l];
  RB_CUDA(upload(h->d_R, R, nL, st));
  RB_CUDA(upload(h->d_N, N, nL, st));
  RB_CUDA(upload(h->d_T, T, nL, st));
  RB_CUDA(upload(h->d_b, b, 2 * (size_t)nb, st));
  RB_CUDA(upload(h->d_a32, a32.data(), a32.size(), st));
  RB_CUDA(h->d_nseg.ensure(sizeof(int) * nb));
  RB_CUDA(h->d_hds.ensure(sizeof(float) * ns));
  RB_CUDA(h->d_layer.ensure(sizeof(int) * ns));
  RB_CUDA(h->d_Tb.ensure(sizeof(double) * (size_t)nb * nf));
  RB_CUDA(h->d_iw.ensure(sizeof(double) * (size_t)nb * nf));
  const int nchunk = rb::tb_nchunk(max_seg);
  RB_CUDA(h->d_part.ensure(sizeof(float4) * (size_t)nb * nchunk * nf));
  h->launches = 0;
  if ((rc = enqueue_raypath(h, st, nL, h->d_R.as<double>(), h->d_N.as<double>(),
                            h->d_T.as<double>(), Req, Rpol, orient0, orient1, gtype, limb, nb,
                            h->d_b.as<double>(), max_seg, h->d_nseg.as<int>(), nullptr,
                            h->d_hds.as<float>(), h->d_layer.as<int>(), nullptr, nullptr, nullptr)))
    return rc;
  rb::TbArgs ta{};
  ta.nL = nL;
  ta.nf = nf;
  ta.nb = nb;
  ta.max_seg = max_seg;
  ta.alpha32 = h->d_a32.as<float>();
  ta.T32 = h->d_T32.as<float>();
  ta.nseg = h->d_nseg.as<int>();
  ta.hds = h->d_hds.as<float>();
  ta.layer = h->d_layer.as<int>();
  ta.Tb = h->d_Tb.as<double>();
  ta.intW = h->d_iw.as<double>();
  ta.nchunk = nchunk;
  ta.lanes = h->scan_lanes;
  ta.part = h->d_part.as<float4>();
  RB_CUDA(rb::launch_tb_chunked(ta, st));
  h->launches += 2;
  RB_CUDA(cudaMemcpyAsync(Tb_out, ta.Tb, sizeof(double) * (size_t)nb * nf, cudaMemcpyDeviceToHost, st));
  if (intW_out)
    RB_CUDA(cudaMemcpyAsync(intW_out, ta.intW, sizeof(double) * (size_t)nb * nf, cudaMemcpyDeviceToHost, st));
  if (nseg_out) RB_CUDA(cudaMemcpyAsync(nseg_out, ta.nseg, sizeof(int) * nb, cudaMemcpyDeviceToHost, st));
  RB_CUDA(cudaStreamSynchronize(st));
  return RB_OK;
}

// One forward pass: ray paths on the side stream concurrent with the
// absorption, then the scan and the quadrature average.  nb = rays per
// atmosphere; with a batch (bt), nL is the total layer count and the
// arrays are the variants' concatenation.
// Runs a host-buffer call's work on st: replayed from the cached graph when
// the call shape, configuration and buffer addresses match it; captured
// and replayed when the same shape ran directly last time (every buffer is
// sized then, so nothing is allocated while capturing); else run directly.
static int run_cached(rb_handle* h, GraphCache& gc, FwdKey key, cudaStream_t st,
                      const std::function<int()>& enqueue) {
  key.cfg = h->cfg_gen;
  key.epoch = g_alloc_epoch.load();
  const bool graphs = !h->profiling;
  if (graphs && gc.exec && key == gc.key) {
    RB_CUDA(cudaGraphLaunch(gc.exec, st));
    h->launches = gc.launches;
    return RB_OK;
  }
  if (graphs && key == gc.seen) {
    RB_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    const int rc = enqueue();
    cudaGraph_t g = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(st, &g);
    if (rc || ec != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      return rc ? rc : fail(RB_ECUDA, "graph capture: %s", cudaGetErrorString(ec));
    }
    cudaGraphExec_t ex = nullptr;
    const cudaError_t ei = cudaGraphInstantiate(&ex, g, 0);
    cudaGraphDestroy(g);
    if (ei != cudaSuccess) return fail(RB_ECUDA, "graph instantiation: %s", cudaGetErrorString(ei));
    gc.release();
    gc.exec = ex;
    gc.key = key;
    gc.launches = h->launches;
    RB_CUDA(cudaGraphLaunch(ex, st));
    return RB_OK;
  }
  const int rc = enqueue();
  if (rc) return rc;
  key.epoch = g_alloc_epoch.load();   // after the buffers this shape needs exist
  gc.seen = graphs ? key : FwdKey{};
  return RB_OK;
}

static int forward_core(rb_handle* h, cudaStream_t st, int nL, const double* dP, const double* dT,
                        const double* dX, const double* dR, const double* dN, const double* dscale,
                        double Req, double Rpol, double o0, double o1, int gtype, int limb, int nb,
                        const double* db, const double* dw, int disc, double* dTb, double* davg,
                        double* dl64, const Batch* bt = nullptr, const AlphaJvp* aj = nullptr,
                        float* iw32 = nullptr) {
  const int nf = (int)h->plan_f.size();
  const int max_seg = 2 * (bt ? bt->max_nL : nL) + 4;
  const int nvar = bt ? bt->nvar : 1;
  const int nbt = nb * nvar;
  const size_t ns = (size_t)std::max(nbt, 1) * max_seg;
  RB_CUDA(h->d_nseg.ensure(sizeof(int) * std::max(nbt, 1)));
  RB_CUDA(h->d_hds.ensure(sizeof(float) * ns));
  RB_CUDA(h->d_layer.ensure(sizeof(int) * ns));
  RB_CUDA(h->d_Tb32.ensure(sizeof(float) * (size_t)std::max(nbt, 1) * nf));
  const int nchunk = rb::tb_nchunk(max_seg);
  if (!disc) RB_CUDA(h->d_part.ensure(sizeof(float4) * (size_t)std::max(nbt, 1) * nchunk * nf));
  h->launches = 0;
  // geometry + ray paths on the side stream, concurrent with the absorption
  RB_CUDA(cudaEventRecord(h->ev_fork, st));
  RB_CUDA(cudaStreamWaitEvent(h->side, h->ev_fork, 0));
  int rc;
  if ((rc = enqueue_raypath(h, h->side, nL, dR, dN, dT, Req, Rpol, o0, o1, gtype, limb,
                            std::max(nbt, 0), db, max_seg, h->d_nseg.as<int>(), nullptr,
                            h->d_hds.as<float>(), h->d_layer.as<int>(), nullptr, nullptr, nullptr,
                            bt, nb)))
    return rc;
  RB_CUDA(cudaEventRecord(h->ev_join, h->side));
  if (aj) rc = enqueue_alpha_jvp(h, st, nL, dP, dT, dX, dscale, *aj);
  else rc = enqueue_alpha(h, st, nL, dP, dT, dX, dscale, 0, dl64, nullptr);
  if (rc) return rc;
  RB_CUDA(cudaStreamWaitEvent(st, h->ev_join, 0));
  if (nbt > 0) {
    rb::TbArgs ta{};
    ta.nL = nL;
    ta.nf = nf;
    ta.nb = nbt;
    ta.max_seg = max_seg;
    ta.var_off = bt ? bt->d_off : nullptr;
    ta.rays_per_var = nb;
    ta.alpha32 = h->d_a32.as<float>();
    ta.T32 = h->d_T32.as<float>();
    ta.nseg = h->d_nseg.as<int>();
    ta.hds = h->d_hds.as<float>();
    ta.layer = h->d_layer.as<int>();
    ta.disc = disc != 0;
    ta.Tb = dTb;
    ta.Tb32 = h->d_Tb32.as<float>();
    ta.nchunk = nchunk;
    ta.lanes = h->scan_lanes;
    ta.part = h->d_part.as<float4>();
    ta.iw32 = iw32;   // the adjoint's chunk state (null: forward only)
    if (h->profiling) RB_CUDA(cudaEventRecord(h->pev[5], st));
    if (disc) {
      RB_CUDA(rb::launch_tb_seq(ta, st));
      h->launches += 1;
    } else {
      RB_CUDA(rb::launch_tb_chunked(ta, st));
      h->launches += 2;
    }
    if (h->profiling) RB_CUDA(cudaEventRecord(h->pev[6], st));
    if (davg && dw) {
      RB_CUDA(rb::launch_disc_avg(nb, nf, h->d_Tb32.as<float>(), dw, davg, st, nvar));
      h->launches += 1;
    }
    if (h->profiling) RB_CUDA(cudaEventRecord(h->pev[7], st));
  }
  return RB_OK;
}

int rb_forward(rb_handle* h, int nL, const double* P, const double* T, const double* X,
               const double* R, const double* N, int nf, const double* freqs, const double* scale,
               double Req, double Rpol, double orient0, double orient1, int gtype, int limb,
               int nb, const double* b, const double* weights, int disc, double* Tb_out,
               double* Tb_avg, double* layers_out) {
  if (!h) return fail(RB_EINVAL, "null handle");
  if (!P || !T || !X || !R || !N || !freqs || (nb > 0 && !b)) return fail(RB_EINVAL, "null input array");
  if (nL < 1) return fail(RB_EINVAL, "nL must be >= 1");
  if (nb < 0) return fail(RB_EINVAL, "nb must be >= 0");
  if (Tb_avg && !weights) return fail(RB_EINVAL, "Tb_avg needs weights");
  std::vector<double> bb;
  if (disc) {  // 'disc' evaluates the nadir ray (brightness.py:32-34)
    bb.assign(2 * (size_t)nb, 0.0);
    b = bb.data();
  }
  int rc = validate_atm(nL, P, T, X);
  if (!rc) rc = validate_geom(nL, R, N, Req, Rpol, gtype, limb, nb, b);
  if (!rc && weights && !finite_all(weights, nb)) rc = fail(RB_EINVAL, "weights not finite");
  if (!rc && scale && !finite_all(scale, (size_t)nL * rb::NGAS)) rc = fail(RB_EINVAL, "scale not finite");
  if (rc) return rc;
  RB_CUDA(cudaSetDevice(h->device));
  RB_CUDA(order_after_device(h, h->st));
  cudaStream_t st = h->st;
  if ((rc = plan_frequencies(h, nf, freqs, st))) return rc;
  // one staged input block (each array at a 256-byte boundary) and one output block
  auto al = [](size_t n) { return (n + 31) / 32 * 32; };
  const bool has_w = weights && nb > 0;
  const size_t oP = 0, oT = oP + al(nL), oX = oT + al(nL), oR = oX + al((size_t)rb::NX * nL),
               oN = oR + al(nL), ob = oN + al(nL), osc = ob + al(2 * (size_t)nb),
               ow = osc + (scale ? al((size_t)rb::NGAS * nL) : 0), nin = ow + (has_w ? al(nb) : 0);
  const size_t nTb = Tb_out && nb > 0 ? (size_t)nb * nf : 0, navg = Tb_avg && nb > 0 ? (size_t)nf : 0,
               nlay = layers_out ? (size_t)nf * nL : 0;
  const size_t oTb = 0, oavg = al(nTb), olay = oavg + al(navg), nout = olay + nlay;
  RB_CUDA(h->h_in.ensure(sizeof(double) * nin));
  RB_CUDA(h->h_out.ensure(sizeof(double) * std::max<size_t>(nout, 1)));
  RB_CUDA(h->d_in.ensure(sizeof(double) * nin));
  RB_CUDA(h->d_Tb.ensure(sizeof(double) * std::max((size_t)nb * nf, (size_t)1)));
  RB_CUDA(h->d_avg.ensure(sizeof(double) * nf));
  if (layers_out) RB_CUDA(h->d_l64.ensure(sizeof(double) * (size_t)nf * nL));
  double* hin = h->h_in.as<double>();
  std::memcpy(hin + oP, P, sizeof(double) * nL);
  std::memcpy(hin + oT, T, sizeof(double) * nL);
  std::memcpy(hin + oX, X, sizeof(double) * rb::NX * (size_t)nL);
  std::memcpy(hin + oR, R, sizeof(double) * nL);
  std::memcpy(hin + oN, N, sizeof(double) * nL);
  if (nb > 0) std::memcpy(hin + ob, b, sizeof(double) * 2 * (size_t)nb);
  if (scale) std::memcpy(hin + osc, scale, sizeof(double) * rb::NGAS * (size_t)nL);
  if (has_w) std::memcpy(hin + ow, weights, sizeof(double) * nb);
  const double* din = h->d_in.as<double>();
  double* dl = layers_out ? h->d_l64.as<double>() : nullptr;
  double* hout = h->h_out.as<double>();
  auto enqueue = [&]() -> int {
    RB_CUDA(cudaMemcpyAsync(h->d_in.p, hin, sizeof(double) * nin, cudaMemcpyHostToDevice, st));
    int r = forward_core(h, st, nL, din + oP, din + oT, din + oX, din + oR, din + oN,
                         scale ? din + osc : nullptr, Req, Rpol, orient0, orient1, gtype, limb, nb,
                         din + ob, has_w ? din + ow : nullptr, disc, h->d_Tb.as<double>(),
                         Tb_avg ? h->d_avg.as<double>() : nullptr, dl);
    if (r) return r;
    if (nTb) RB_CUDA(cudaMemcpyAsync(hout + oTb, h->d_Tb.p, sizeof(double) * nTb, cudaMemcpyDeviceToHost, st));
    if (navg) RB_CUDA(cudaMemcpyAsync(hout + oavg, h->d_avg.p, sizeof(double) * navg, cudaMemcpyDeviceToHost, st));
    if (nlay) RB_CUDA(cudaMemcpyAsync(hout + olay, dl, sizeof(double) * nlay, cudaMemcpyDeviceToHost, st));
    return RB_OK;
  };
  FwdKey key;
  key.nL = nL;
  key.nf = nf;
  key.nb = nb;
  key.disc = disc;
  key.gtype = gtype;
  key.limb = limb;
  key.flags = (scale ? 1 : 0) | (has_w ? 2 : 0) | (nTb ? 4 : 0) | (navg ? 8 : 0) | (nlay ? 16 : 0);
  key.Req = Req;
  key.Rpol = Rpol;
  key.o0 = orient0;
  key.o1 = orient1;
  if ((rc = run_cached(h, h->g_fwd, key, st, enqueue))) return rc;
  RB_CUDA(cudaStreamSynchronize(st));
  if (nTb) std::memcpy(Tb_out, hout + oTb, sizeof(double) * nTb);
  if (navg) std::memcpy(Tb_avg, hout + oavg, sizeof(double) * navg);
  if (nlay) std::memcpy(layers_out, hout + olay, sizeof(double) * nlay);
  return RB_OK;
}

int rb_forward_device(rb_handle* h, void* stream, int nL, const double* P, const double* T,
                      const double* X, const double* R, const double* N, int nf,
                      const double* freqs_host, const double* scale, double Req, double Rpol,
                      double orient0, double orient1, int gtype, int limb, int nb,
                      const double* b, const double* weights, int disc, double* Tb_out,
                      double* Tb_avg) {
  if (!h) return fail(RB_EINVAL, "null handle");
  if (!P || !T || !X || !R || !N || !freqs_host || (nb > 0 && (!b || !Tb_out)))
    return fail(RB_EINVAL, "null array");
  if (nL < 2 || nb < 0) return fail(RB_EINVAL, "bad sizes");
  if (Tb_avg && !weights) return fail(RB_EINVAL, "Tb_avg needs weights");
  if (gtype != RB_GTYPE_ELLIPSE && gtype != RB_GTYPE_SPHERE) return fail(RB_EINVAL, "bad gtype");
  if (limb != RB_LIMB_SHAPE && limb != RB_LIMB_SEC) return fail(RB_EINVAL, "bad limb");
  RB_CUDA(cudaSetDevice(h->device));
  RB_CUDA(order_after_device(h, h->st));
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  RB_CUDA(order_after_device(h, st));
  int rc;
  if ((rc = plan_frequencies(h, nf, freqs_host, h->st))) return rc;
  if ((rc = forward_core(h, st, nL, P, T, X, R, N, scale, Req, Rpol, orient0, orient1, gtype, limb,
                         nb, b, weights, disc, Tb_out, Tb_avg, nullptr)))
    return rc;
  RB_CUDA(mark_device(h, st));
  return RB_OK;
}

// Forward (recomputed) then the adjoint sweep: d loss / d alpha from the
// scan adjoint, alpha recomputed with its layer derivatives and contracted.
static int adjoint_core(rb_handle* h, cudaStream_t st, int nL, const double* P, const double* T,
                        const double* X, const double* R, const double* N, const double* scale,
                        double Req, double Rpol, double orient0, double orient1, int gtype,
                        int limb, int nb, const double* b, const double* weights, int disc,
                        const double* grad, double* Tb_out, double* Tb_avg, double* dT, double* dP,
                        double* dlnX, const Batch* bt = nullptr) {
  const int nf = (int)h->plan_f.size();
  const int nvar = bt ? bt->nvar : 1;
  const int nbt = nb * nvar;
  RB_CUDA(h->d_Tb.ensure(sizeof(double) * (size_t)nbt * nf));
  RB_CUDA(h->d_avg.ensure(sizeof(double) * (size_t)nvar * nf));
  double* dTb = Tb_out ? Tb_out : h->d_Tb.as<double>();
  double* davg = Tb_avg ? Tb_avg : (weights ? h->d_avg.as<double>() : nullptr);
  rb::TanArgs tn{};
  tn.nL = nL;
  tn.P = P;
  tn.T = T;
  tn.X = X;
  tn.nh3_mode = h->cfg.nh3_mode;
  tn.h2state = h->cfg.h2state;
  tn.inv_table = h->cfg.inv_table;
  rb::JvpArgs jv{};
  jv.nL = nL;
  jv.nf = nf;
  jv.ft = rb::adjoint_ft(nf, h->jvp_ft);
  jv.ctas = h->jvp_ctas;
  jv.threads = h->jvp_threads;
  if (jv.threads && jv.threads % jv.ft)
    return fail(RB_EINVAL, "JVP threads per CTA (%d) must be a multiple of its frequencies per CTA (%d)",
                jv.threads, jv.ft);
  jv.fplan = h->d_jfreq.as<rb::JvFreq>();
  for (int f = 0; f < rb::NFAM; ++f) jv.tab[f] = h->fam[f].table();
  jv.cfg = h->cfg;
  jv.cfg.units_db = 0;
  // d alpha / d theta stored from a JVP run before the scan (which also
  // gives the scan's alpha), or recomputed after the reverse sweep
  const size_t dal_bytes = sizeof(float) * (size_t)nL * rb::NTH * nf;
  const bool store = h->adj_mode == 1 || (h->adj_mode == 0 && dal_bytes <= h->dev_mem / 8);
  AlphaJvp aj{tn, jv};
  RB_CUDA(h->d_iw32.ensure(sizeof(float) * (size_t)std::max(nbt, 1) * nf));
  int rc;
  if ((rc = forward_core(h, st, nL, P, T, X, R, N, scale, Req, Rpol, orient0, orient1, gtype, limb,
                         nb, b, weights, disc, dTb, davg, nullptr, bt, store ? &aj : nullptr,
                         disc ? nullptr : h->d_iw32.as<float>())))
    return rc;
  const int launches = h->launches;
  const int max_seg = 2 * (bt ? bt->max_nL : nL) + 4;
  const int ntile = rb::adjoint_tiles(nf, h->jvp_ft);
  RB_CUDA(h->d_ga.ensure(sizeof(float) * (size_t)nL * nf));
  RB_CUDA(h->d_gs.ensure(sizeof(double) * (size_t)nL));
  RB_CUDA(h->d_lt.ensure(sizeof(rb::LayerTan) * nL));
  if (!store) RB_CUDA(h->d_jpart.ensure(sizeof(float2) * (size_t)nL * ntile * rb::NTH));
  rb::TbAdjArgs ta{};
  ta.nL = nL;
  ta.nf = nf;
  ta.nb = nbt;
  ta.max_seg = max_seg;
  ta.var_off = bt ? bt->d_off : nullptr;
  ta.rays_per_var = nb;
  ta.alpha32 = h->d_a32.as<float>();
  ta.T = T;
  ta.nseg = h->d_nseg.as<int>();
  ta.hds = h->d_hds.as<float>();
  ta.layer = h->d_layer.as<int>();
  ta.weights = weights;
  ta.grad = grad;
  ta.ga = h->d_ga.as<float>();
  ta.gs = h->d_gs.as<double>();
  ta.nchunk = rb::tb_nchunk(max_seg);
  ta.disc = disc != 0;
  if (disc) {   // sequential E2 sweep: {tau, 2 E2} per node instead of chunk sums
    RB_CUDA(h->d_adjS.ensure(sizeof(double2) * (size_t)nbt * max_seg * nf));
    ta.tauE = h->d_adjS.as<double2>();
  } else {
    ta.part = h->d_part.as<float4>();
    ta.Tb32 = h->d_Tb32.as<float>();
    ta.iw32 = h->d_iw32.as<float>();
    RB_CUDA(h->d_adjS.ensure(sizeof(float) * (size_t)nbt * ta.nchunk * nf));
    ta.S = h->d_adjS.as<float>();
  }
  tn.out = h->d_lt.as<rb::LayerTan>();
  jv.lp = h->d_lp.as<rb::LayerParams>();
  jv.lt = h->d_lt.as<rb::LayerTan>();
  jv.galpha = h->d_ga.as<float>();
  jv.part = h->d_jpart.as<float2>();
  jv.dal_out = h->d_dal.as<float>();
  rb::ExtraArgs ea{};
  const bool extra = h->cfg.use_co || h->cfg.use_clouds;
  if (extra) {
    RB_CUDA(h->d_xgrad.ensure(sizeof(double) * 2 * (size_t)nL));
    extra_args(h, ea, nL, P, T, X);
    ea.galpha = h->d_ga.as<float>();
    ea.scale = scale;
    ea.grad = h->d_xgrad.as<double>();
  }
  const int nsweep = disc ? 1 : 3;   // [lambda, suffix, grad] or the sequential 'disc' sweep
  if (store) {
    RB_CUDA(rb::launch_adjoint_sweep(ta, st));
    RB_CUDA(rb::launch_adjoint_contract(jv, extra ? &ea : nullptr, h->d_ga.as<float>(),
                                        h->d_gs.as<double>(), dT, dP, dlnX, st));
    h->launches = launches + nsweep + (extra ? 1 : 0) + 1;
  } else {
    RB_CUDA(rb::launch_adjoint(ta, tn, jv, extra ? &ea : nullptr, h->d_ga.as<float>(),
                               h->d_gs.as<double>(), dT, dP, dlnX, st));
    h->launches = launches + nsweep + (extra ? 1 : 0) + 3;   // sweep, tangents, JVP, [extra,] final
  }
  return RB_OK;
}

int rb_adjoint_device(rb_handle* h, void* stream, int nL, const double* P, const double* T,
                      const double* X, const double* R, const double* N, int nf,
                      const double* freqs_host, const double* scale, double Req, double Rpol,
                      double orient0, double orient1, int gtype, int limb, int nb, const double* b,
                      const double* weights, int disc, const double* grad, double* Tb_out,
                      double* Tb_avg, double* dT, double* dP, double* dlnX) {
  if (!h) return fail(RB_EINVAL, "null handle");
  if (!P || !T || !X || !R || !N || !freqs_host || !grad || !dT || !dP || !dlnX ||
      (nb > 0 && !b))
    return fail(RB_EINVAL, "null array");
  if (nL < 2 || nb < 1) return fail(RB_EINVAL, "bad sizes");
  if (Tb_avg && !weights) return fail(RB_EINVAL, "Tb_avg needs weights");
  if (gtype != RB_GTYPE_ELLIPSE && gtype != RB_GTYPE_SPHERE) return fail(RB_EINVAL, "bad gtype");
  if (limb != RB_LIMB_SHAPE && limb != RB_LIMB_SEC) return fail(RB_EINVAL, "bad limb");
  RB_CUDA(cudaSetDevice(h->device));
  RB_CUDA(order_after_device(h, h->st));
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  RB_CUDA(order_after_device(h, st));
  int rc;
  if ((rc = plan_frequencies(h, nf, freqs_host, h->st))) return rc;
  if ((rc = adjoint_core(h, st, nL, P, T, X, R, N, scale, Req, Rpol, orient0, orient1, gtype, limb,
                         nb, b, weights, disc, grad, Tb_out, Tb_avg, dT, dP, dlnX)))
    return rc;
  RB_CUDA(mark_device(h, st));
  return RB_OK;
}

// Batch descriptor from the host layer counts (offsets uploaded once per
// distinct batch shape).
static int make_batch(rb_handle* h, int nvar, const int32_t* nL_host, Batch& bt, int& NLT) {
  if (nvar < 1 || !nL_host) return fail(RB_EINVAL, "batch needs nvar >= 1 and layer counts");
  std::vector<int> off(nvar + 1, 0);
  int mx = 0;
  for (int v = 0; v < nvar; ++v) {
    if (nL_host[v] < 2) return fail(RB_EINVAL, "variant %d has %d layers (need >= 2)", v, nL_host[v]);
    off[v + 1] = off[v] + nL_host[v];
    mx = std::max(mx, (int)nL_host[v]);
  }
  if (h->batch_off != off) {
    RB_CUDA(upload(h->d_voff, off.data(), off.size(), h->st));
    RB_CUDA(cudaStreamSynchronize(h->st));
    h->batch_off = off;
  }
  bt.nvar = nvar;
  bt.d_off = h->d_voff.as<int>();
  bt.max_nL = mx;
  NLT = off[nvar];
  return RB_OK;
}

int rb_forward_batch_device(rb_handle* h, void* stream, int nvar, const int32_t* nL_host,
                            const double* P, const double* T, const double* X, const double* R,
                            const double* N, int nf, const double* freqs_host, const double* scale,
                            double Req,
                            double Rpol, double orient0, double orient1, int gtype, int limb,
                            int nb, const double* b, const double* weights, double* Tb_avg) {
  if (!h) return fail(RB_EINVAL, "null handle");
  if (!P || !T || !X || !R || !N || !freqs_host || !b || !weights || !Tb_avg)
    return fail(RB_EINVAL, "null array");
  if (nb < 1) return fail(RB_EINVAL, "nb must be >= 1");
  if (gtype != RB_GTYPE_ELLIPSE && gtype != RB_GTYPE_SPHERE) return fail(RB_EINVAL, "bad gtype");
  if (limb != RB_LIMB_SHAPE && limb != RB_LIMB_SEC) return fail(RB_EINVAL, "bad limb");
  RB_CUDA(cudaSetDevice(h->device));
  RB_CUDA(order_after_device(h, h->st));
  int rc, NLT = 0;
  Batch bt;
  if ((rc = make_batch(h, nvar, nL_host, bt, NLT))) return rc;
  if ((rc = plan_frequencies(h, nf, freqs_host, h->st))) return rc;
  RB_CUDA(h->d_Tb.ensure(sizeof(double) * (size_t)nvar * nb * nf));
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  RB_CUDA(order_after_device(h, st));
  if ((rc = forward_core(h, st, NLT, P, T, X, R, N, scale, Req, Rpol, orient0, orient1, gtype, limb,
                         nb, b, weights, 0, h->d_Tb.as<double>(), Tb_avg, nullptr, &bt)))
    return rc;
  RB_CUDA(mark_device(h, st));
  return RB_OK;
}

int rb_adjoint_batch_device(rb_handle* h, void* stream, int nvar, const int32_t* nL_host,
                            const double* P, const double* T, const double* X, const double* R,
                            const double* N, int nf, const double* freqs_host, const double* scale,
                            double Req,
                            double Rpol, double orient0, double orient1, int gtype, int limb,
                            int nb, const double* b, const double* weights, const double* grad,
                            double* Tb_avg, double* dT, double* dP, double* dlnX) {
  if (!h) return fail(RB_EINVAL, "null handle");
  if (!P || !T || !X || !R || !N || !freqs_host || !b || !weights || !grad || !dT || !dP || !dlnX)
    return fail(RB_EINVAL, "null array");
  if (nb < 1) return fail(RB_EINVAL, "nb must be >= 1");
  if (gtype != RB_GTYPE_ELLIPSE && gtype != RB_GTYPE_SPHERE) return fail(RB_EINVAL, "bad gtype");
  if (limb != RB_LIMB_SHAPE && limb != RB_LIMB_SEC) return fail(RB_EINVAL, "bad limb");
  RB_CUDA(cudaSetDevice(h->device));
  RB_CUDA(order_after_device(h, h->st));
  int rc, NLT = 0;
  Batch bt;
  if ((rc = make_batch(h, nvar, nL_host, bt, NLT))) return rc;
  if ((rc = plan_frequencies(h, nf, freqs_host, h->st))) return rc;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  RB_CUDA(order_after_device(h, st));
  if ((rc = adjoint_core(h, st, NLT, P, T, X, R, N, scale, Req, Rpol, orient0, orient1, gtype,
                         limb, nb, b, weights, 0, grad, nullptr, Tb_avg, dT, dP, dlnX, &bt)))
    return rc;
  RB_CUDA(mark_device(h, st));
  return RB_OK;
}

int rb_adjoint(rb_handle* h, int nL, const double* P, const double* T, const double* X,
               const double* R, const double* N, int nf, const double* freqs, const double* scale,
               double Req, double Rpol, double orient0, double orient1, int gtype, int limb, int nb,
               const double* b, const double* weights, int disc, const double* grad,
               double* Tb_out, double* Tb_avg, double* dT, double* dP, double* dlnX) {
  if (!h) return fail(RB_EINVAL, "null handle");
  if (!P || !T || !X || !R || !N || !freqs || !grad || !dT || !dP || !dlnX || (nb > 0 && !b))
    return fail(RB_EINVAL, "null array");
  if (nL < 1) return fail(RB_EINVAL, "nL must be >= 1");
  if (nb < 1) return fail(RB_EINVAL, "nb must be >= 1");
  if (nf < 1) return fail(RB_EINVAL, "nf must be >= 1");
  std::vector<double> bb;
  if (disc) {  // 'disc' evaluates the nadir ray (brightness.py:32-34)
    bb.assign(2 * (size_t)nb, 0.0);
    b = bb.data();
  }
  int rc = validate_atm(nL, P, T, X);
  if (!rc) rc = validate_geom(nL, R, N, Req, Rpol, gtype, limb, nb, b);
  if (!rc && weights && !finite_all(weights, nb)) rc = fail(RB_EINVAL, "weights not finite");
  const size_t ng = weights ? (size_t)nf : (size_t)nb * nf;
  if (!rc && !finite_all(grad, ng)) rc = fail(RB_EINVAL, "grad not finite");
  if (!rc && scale && !finite_all(scale, (size_t)nL * rb::NGAS)) rc = fail(RB_EINVAL, "scale not finite");
  if (rc) return rc;
  RB_CUDA(cudaSetDevice(h->device));
  RB_CUDA(order_after_device(h, h->st));
  cudaStream_t st = h->st;
  if ((rc = plan_frequencies(h, nf, freqs, st))) return rc;
  // one staged input block (each array at a 256-byte boundary) and one output block
  auto al = [](size_t n) { return (n + 31) / 32 * 32; };
  const size_t oP = 0, oT = oP + al(nL), oX = oT + al(nL), oR = oX + al((size_t)rb::NX * nL),
               oN = oR + al(nL), ob = oN + al(nL), og = ob + al(2 * (size_t)nb), osc = og + al(ng),
               ow = osc + (scale ? al((size_t)rb::NGAS * nL) : 0), nin = ow + (weights ? al(nb) : 0);
  const size_t nTb = Tb_out ? (size_t)nb * nf : 0, navg = Tb_avg && weights ? (size_t)nf : 0;
  const size_t oTb = 0, oavg = al(nTb), oth = oavg + al(navg), nout = oth + 5 * (size_t)nL;
  RB_CUDA(h->h_in.ensure(sizeof(double) * nin));
  RB_CUDA(h->h_out.ensure(sizeof(double) * nout));
  RB_CUDA(h->d_in.ensure(sizeof(double) * nin));
  RB_CUDA(h->d_Tb.ensure(sizeof(double) * (size_t)nb * nf));
  RB_CUDA(h->d_avg.ensure(sizeof(double) * nf));
  RB_CUDA(h->d_dth.ensure(sizeof(double) * 5 * (size_t)nL));
  double* hin = h->h_in.as<double>();
  std::memcpy(hin + oP, P, sizeof(double) * nL);
  std::memcpy(hin + oT, T, sizeof(double) * nL);
  std::memcpy(hin + oX, X, sizeof(double) * rb::NX * (size_t)nL);
  std::memcpy(hin + oR, R, sizeof(double) * nL);
  std::memcpy(hin + oN, N, sizeof(double) * nL);
  std::memcpy(hin + ob, b, sizeof(double) * 2 * (size_t)nb);
  std::memcpy(hin + og, grad, sizeof(double) * ng);
  if (scale) std::memcpy(hin + osc, scale, sizeof(double) * rb::NGAS * (size_t)nL);
  if (weights) std::memcpy(hin + ow, weights, sizeof(double) * nb);
  const double* din = h->d_in.as<double>();
  double* dd = h->d_dth.as<double>();
  double* hout = h->h_out.as<double>();
  auto enqueue = [&]() -> int {
    RB_CUDA(cudaMemcpyAsync(h->d_in.p, hin, sizeof(double) * nin, cudaMemcpyHostToDevice, st));
    int r = adjoint_core(h, st, nL, din + oP, din + oT, din + oX, din + oR, din + oN,
                         scale ? din + osc : nullptr, Req, Rpol, orient0, orient1, gtype, limb, nb,
                         din + ob, weights ? din + ow : nullptr, disc, din + og, h->d_Tb.as<double>(),
                         weights ? h->d_avg.as<double>() : nullptr, dd, dd + nL, dd + 2 * (size_t)nL);
    if (r) return r;
    if (nTb) RB_CUDA(cudaMemcpyAsync(hout + oTb, h->d_Tb.p, sizeof(double) * nTb, cudaMemcpyDeviceToHost, st));
    if (navg) RB_CUDA(cudaMemcpyAsync(hout + oavg, h->d_avg.p, sizeof(double) * navg, cudaMemcpyDeviceToHost, st));
    RB_CUDA(cudaMemcpyAsync(hout + oth, dd, sizeof(double) * 5 * (size_t)nL, cudaMemcpyDeviceToHost, st));
    return RB_OK;
  };
  FwdKey key;
  key.nL = nL;
  key.nf = nf;
  key.nb = nb;
  key.gtype = gtype;
  key.limb = limb;
  key.flags = (scale ? 1 : 0) | (weights ? 2 : 0) | (nTb ? 4 : 0) | (navg ? 8 : 0);
  key.disc = disc;
  key.Req = Req;
  key.Rpol = Rpol;
  key.o0 = orient0;
  key.o1 = orient1;
  if ((rc = run_cached(h, h->g_adj, key, st, enqueue))) return rc;
  RB_CUDA(cudaStreamSynchronize(st));
  if (nTb) std::memcpy(Tb_out, hout + oTb, sizeof(double) * nTb);
  if (navg) std::memcpy(Tb_avg, hout + oavg, sizeof(double) * navg);
  std::memcpy(dT, hout + oth, sizeof(double) * nL);
  std::memcpy(dP, hout + oth + nL, sizeof(double) * nL);
  std::memcpy(dlnX, hout + oth + 2 * (size_t)nL, sizeof(double) * 3 * nL);
  return RB_OK;
}

int rb_last_launch_count(rb_handle* h) { return h ? h->launches : 0; }

// ------------------------------------------------------------ atmosphere producer
// Column roles [Z, T, P, DZ] and chemistry [3][ncol] (amu, c_p / R, refr)
// -> the kernel's column description.
static int atm_cols(int ncol, const int32_t* roles, const double* chem, rb::AtmCols& c) {
  if (ncol < 4 || ncol > rb::ATM_MAXCOL) return fail(RB_EINVAL, "ncol must be in 4..%d", rb::ATM_MAXCOL);
  if (!roles) return fail(RB_EINVAL, "null column roles");
  for (int r = 0; r < 4; ++r)
    if (roles[r] < 0 || roles[r] >= ncol) return fail(RB_EINVAL, "column role %d out of range", r);
  c.ncol = ncol;
  c.iz = roles[0];
  c.it = roles[1];
  c.ip = roles[2];
  c.idz = roles[3];
  for (int k = 0; k < ncol; ++k) {
    c.amu[k] = chem ? chem[k] : 0.0;
    c.cp[k] = chem ? chem[ncol + k] : 0.0;
    c.refr[k] = chem ? chem[2 * ncol + k] : 0.0;
  }
  if (chem && !finite_all(chem, 3 * (size_t)ncol)) return fail(RB_EINVAL, "chemistry not finite");
  return RB_OK;
}

static int atm_check_table(int n, int ncol, int ip, int it, const double* tab, bool need_T) {
  if (!finite_all(tab, (size_t)ncol * n)) return fail(RB_EINVAL, "table has non-finite entries");
  const double* P = tab + (size_t)ip * n;
  for (int i = 0; i < n; ++i) {
    if (!(P[i] > 0.0)) return fail(RB_EINVAL, "P[%d] must be > 0", i);
    if (i && !(P[i] > P[i - 1])) return fail(RB_EINVAL, "P must increase (layer %d)", i);
    if (need_T && !(tab[(size_t)it * n + i] > 0.0)) return fail(RB_EINVAL, "T[%d] must be > 0", i);
  }
  return RB_OK;
}

static int atm_offsets(rb_handle* h, int nvar, const int32_t* n_host, int minn, int& tot) {
  if (nvar < 1 || !n_host) return fail(RB_EINVAL, "need nvar >= 1 and layer counts");
  std::vector<int> off(nvar + 1, 0);
  for (int v = 0; v < nvar; ++v) {
    if (n_host[v] < minn) return fail(RB_EINVAL, "atmosphere %d has %d layers (need >= %d)", v, n_host[v], minn);
    off[v + 1] = off[v] + n_host[v];
  }
  RB_CUDA(upload(h->d_aoff, off.data(), off.size(), h->st));
  RB_CUDA(cudaStreamSynchronize(h->st));
  tot = off[nvar];
  return RB_OK;
}

int rb_atm_props_device(rb_handle* h, void* stream, int nvar, const int32_t* nL_host, int ncol,
                        const int32_t* roles, const double* chem, const double* gas, double Req,
                        double p_ref, double GM_ref, double* prop) {
  if (!h) return fail(RB_EINVAL, "null handle");
  if (!gas || !prop) return fail(RB_EINVAL, "null array");
  rb::AtmPropArgs a{};
  int rc;
  if ((rc = atm_cols(ncol, roles, chem, a.cols))) return rc;
  RB_CUDA(cudaSetDevice(h->device));
  RB_CUDA(order_after_device(h, h->st));
  int tot = 0;
  if ((rc = atm_offsets(h, nvar, nL_host, 1, tot))) return rc;
  a.gas = gas;
  a.ld = tot;
  a.off = h->d_aoff.as<int>();
  a.Req = Req;
  a.p_ref = p_ref;
  a.GM_ref = GM_ref;
  a.prop = prop;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  RB_CUDA(order_after_device(h, st));
  RB_CUDA(rb::launch_atm_props(a, nvar, st));
  h->launches = 1;
  RB_CUDA(mark_device(h, st));
  return RB_OK;
}

int rb_atm_props(rb_handle* h, int nL, int ncol, const int32_t* roles, const double* chem,
                 const double* gas, double Req, double p_ref, double GM_ref, double* prop) {
  if (!h) return fail(RB_EINVAL, "null handle");
  if (!gas || !prop) return fail(RB_EINVAL, "null array");
  if (nL < 1) return fail(RB_EINVAL, "nL must be >= 1");
  rb::AtmCols c{};
  int rc;
  if ((rc = atm_cols(ncol, roles, chem, c))) return rc;
  if ((rc = atm_check_table(nL, ncol, c.ip, c.it, gas, true))) return rc;
  RB_CUDA(cudaSetDevice(h->device));
  RB_CUDA(order_after_device(h, h->st));
  cudaStream_t st = h->st;
  RB_CUDA(upload(h->d_agas, gas, (size_t)ncol * nL, st));
  RB_CUDA(h->d_aprop.ensure(sizeof(double) * rb::NPROP * (size_t)nL));
  const int32_t n1 = nL;
  if ((rc = rb_atm_props_device(h, st, 1, &n1, ncol, roles, chem, h->d_agas.as<double>(), Req, p_ref,
                                GM_ref, h->d_aprop.as<double>())))
    return rc;
  RB_CUDA(cudaMemcpyAsync(prop, h->d_aprop.p, sizeof(double) * rb::NPROP * (size_t)nL,
                          cudaMemcpyDeviceToHost, st));
  RB_CUDA(cudaStreamSynchronize(st));
  return RB_OK;
}

int rb_regrid_device(rb_handle* h, void* stream, int nvar, const int32_t* nin_host, int ncol,
                     const int32_t* roles, const double* chem, const double* gas_in, int ncl,
                     const int32_t* roles_cl, const double* cloud_in, int nout, const double* pgrid,
                     int pgrid_stride, double Req, double p_ref, double GM_ref, double* gas_out,
                     double* cloud_out) {
  if (!h) return fail(RB_EINVAL, "null handle");
  if (!gas_in || !gas_out || !pgrid) return fail(RB_EINVAL, "null array");
  if (nout < 2) return fail(RB_EINVAL, "nout must be >= 2");
  if (pgrid_stride != 0 && pgrid_stride < nout) return fail(RB_EINVAL, "pgrid_stride must be 0 or >= nout");
  if ((cloud_in == nullptr) != (cloud_out == nullptr)) return fail(RB_EINVAL, "cloud_in and cloud_out go together");
  rb::AtmRegridArgs a{};
  int rc;
  if ((rc = atm_cols(ncol, roles, chem, a.cols))) return rc;
  if (cloud_in && (rc = atm_cols(ncl, roles_cl, nullptr, a.cloud_cols))) return rc;
  RB_CUDA(cudaSetDevice(h->device));
  RB_CUDA(order_after_device(h, h->st));
  int tot = 0;
  if ((rc = atm_offsets(h, nvar, nin_host, 2, tot))) return rc;
  a.gas_in = gas_in;
  a.cloud_in = cloud_in;
  a.ld_in = tot;
  a.in_off = h->d_aoff.as<int>();
  a.nout = nout;
  a.pgrid = pgrid;
  a.pgrid_stride = pgrid_stride;
  a.ld_out = nvar * nout;
  a.Req = Req;
  a.p_ref = p_ref;
  a.GM_ref = GM_ref;
  a.gas_out = gas_out;
  a.cloud_out = cloud_out;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  RB_CUDA(order_after_device(h, st));
  RB_CUDA(rb::launch_atm_regrid(a, nvar, st));
  h->launches = 1;
  RB_CUDA(mark_device(h, st));
  return RB_OK;
}

int rb_regrid(rb_handle* h, int nin, int ncol, const int32_t* roles, const double* chem,
              const double* gas_in, int ncl, const int32_t* roles_cl, const double* cloud_in,
              int nout, const double* Pgrid, double Req, double p_ref, double GM_ref,
              double* gas_out, double* cloud_out) {
  if (!h) return fail(RB_EINVAL, "null handle");
  if (!gas_in || !gas_out || !Pgrid) return fail(RB_EINVAL, "null array");
  if (nin < 2 || nout < 2) return fail(RB_EINVAL, "need >= 2 input layers and grid points");
  rb::AtmCols c{}, cl{};
  int rc;
  if ((rc = atm_cols(ncol, roles, chem, c))) return rc;
  if ((rc = atm_check_table(nin, ncol, c.ip, c.it, gas_in, true))) return rc;
  if (cloud_in) {
    if ((rc = atm_cols(ncl, roles_cl, nullptr, cl))) return rc;
    if ((rc = atm_check_table(nin, ncl, cl.ip, cl.it, cloud_in, false))) return rc;
  }
  for (int i = 0; i < nout; ++i) {
    if (!(Pgrid[i] > 0.0) || !std::isfinite(Pgrid[i])) return fail(RB_EINVAL, "Pgrid[%d] must be > 0", i);
    if (i && !(Pgrid[i] > Pgrid[i - 1])) return fail(RB_EINVAL, "Pgrid must increase");
  }
  RB_CUDA(cudaSetDevice(h->device));
  RB_CUDA(order_after_device(h, h->st));
  cudaStream_t st = h->st;
  RB_CUDA(upload(h->d_agas, gas_in, (size_t)ncol * nin, st));
  RB_CUDA(upload(h->d_agrid, Pgrid, (size_t)nout, st));
  RB_CUDA(h->d_aout.ensure(sizeof(double) * (size_t)ncol * nout));
  if (cloud_in) {
    RB_CUDA(upload(h->d_acl, cloud_in, (size_t)ncl * nin, st));
    RB_CUDA(h->d_aclout.ensure(sizeof(double) * (size_t)ncl * nout));
  }
  const int32_t n1 = nin;
  if ((rc = rb_regrid_device(h, st, 1, &n1, ncol, roles, chem, h->d_agas.as<double>(), ncl, roles_cl,
                             cloud_in ? h->d_acl.as<double>() : nullptr, nout,
                             h->d_agrid.as<double>(), 0, Req, p_ref, GM_ref, h->d_aout.as<double>(),
                             cloud_in ? h->d_aclout.as<double>() : nullptr)))
    return rc;
  RB_CUDA(cudaMemcpyAsync(gas_out, h->d_aout.p, sizeof(double) * (size_t)ncol * nout,
                          cudaMemcpyDeviceToHost, st));
  if (cloud_in)
    RB_CUDA(cudaMemcpyAsync(cloud_out, h->d_aclout.p, sizeof(double) * (size_t)ncl * nout,
                            cudaMemcpyDeviceToHost, st));
  RB_CUDA(cudaStreamSynchronize(st));
  return RB_OK;
}

int rb_set_profiling(rb_handle* h, int on) {
  if (!h) return fail(RB_EINVAL, "null handle");
  RB_CUDA(cudaSetDevice(h->device));
  RB_CUDA(order_after_device(h, h->st));
  if (on && !h->pev[0])
    for (auto& e : h->pev) RB_CUDA(cudaEventCreate(&e));
  h->profiling = on != 0;
  return RB_OK;
}

int rb_phase_times(rb_handle* h, double* ms, int n) {
  if (!h || !ms) return fail(RB_EINVAL, "null argument");
  if (!h->profiling) return fail(RB_ESTATE, "profiling is off (rb_set_profiling)");
  RB_CUDA(cudaSetDevice(h->device));
  RB_CUDA(order_after_device(h, h->st));
  RB_CUDA(cudaEventSynchronize(h->pev[7]));
  float t[6] = {0, 0, 0, 0, 0, 0};
  RB_CUDA(cudaEventElapsedTime(&t[0], h->pev[0], h->pev[1]));
  RB_CUDA(cudaEventElapsedTime(&t[1], h->pev[1], h->pev[8]));
  RB_CUDA(cudaEventElapsedTime(&t[2], h->pev[3], h->pev[4]));
  RB_CUDA(cudaEventElapsedTime(&t[3], h->pev[5], h->pev[6]));
  RB_CUDA(cudaEventElapsedTime(&t[4], h->pev[6], h->pev[7]));
  RB_CUDA(cudaEventElapsedTime(&t[5], h->pev[8], h->pev[2]));
  for (int i = 0; i < n && i < 6; ++i) ms[i] = t[i];
  return RB_OK;
}

int rb_probe_fp32_peak(rb_handle* h, double* tflops) {
  if (!h || !tflops) return fail(RB_EINVAL, "null argument");
  RB_CUDA(cudaSetDevice(h->device));
  RB_CUDA(order_after_device(h, h->st));
  int sms = 0;
  RB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device));
  RB_CUDA(h->d_probe.ensure(256 * sizeof(float)));
  cudaEvent_t e0, e1;
  RB_CUDA(cudaEventCreate(&e0));
  RB_CUDA(cudaEventCreate(&e1));
  const int blocks = sms * 8, iters = 1 << 14;
  double best_tf = 0.0;
  for (int packed = 0; packed < 2; ++packed) {
    float best = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {
      RB_CUDA(cudaEventRecord(e0, h->st));
      RB_CUDA(rb::launch_fp32_probe(blocks, iters, h->d_probe.as<float>(), packed, h->st));
      RB_CUDA(cudaEventRecord(e1, h->st));
      RB_CUDA(cudaEventSynchronize(e1));
      float ms = 0;
      RB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      if (rep > 0) best = std::min(best, ms);
    }
    const double flops = 2.0 * 8.0 * (packed ? 2.0 : 1.0) * (double)iters * blocks * 256.0;
    best_tf = std::max(best_tf, flops / (best * 1e-3) / 1e12);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *tflops = best_tf;
  return RB_OK;
}

static int debug_expint(rb_handle* h, int order, int n, const double* x, double* out) {
  if (!h) return fail(RB_EINVAL, "null handle");
  if (n < 0 || (n > 0 && (!x || !out))) return fail(RB_EINVAL, "bad arguments");
  if (n == 0) return RB_OK;
  RB_CUDA(cudaSetDevice(h->device));
  RB_CUDA(order_after_device(h, h->st));
  RB_CUDA(upload(h->d_x, x, n, h->st));
  RB_CUDA(h->d_iw.ensure(sizeof(double) * n));
  RB_CUDA(rb::launch_e2(order, n, h->d_x.as<double>(), h->d_iw.as<double>(), h->st));
  RB_CUDA(cudaMemcpyAsync(out, h->d_iw.p, sizeof(double) * n, cudaMemcpyDeviceToHost, h->st));
  RB_CUDA(cudaStreamSynchronize(h->st));
  return RB_OK;
}

int rb_debug_e2(rb_handle* h, int n, const double* x, double* out) {
  return debug_expint(h, 2, n, x, out);
}

int rb_debug_e1(rb_handle* h, int n, const double* x, double* out) {
  return debug_expint(h, 1, n, x, out);
}

}  // extern "C"
