// rb_brightness_noalloc: brightness temperatures from device-resident inputs
// without allocating device memory.
//
// Some callers cannot allocate: a host application that reserves all device
// memory up front and hands out only pre-sized buffers (memory-pool owners,
// plugins running inside a framework that owns the allocator), or a
// real-time pipeline that forbids cudaMalloc / cudaFree after start-up
// because they can synchronise the device and take unbounded time. This
// entry point serves them: the caller passes device pointers for every input
// and output, and the only scratch the scan needs -- one float4 partial sum
// per (ray, chunk of 128 segments, frequency) -- lives in the file-scope
// array below, which is part of the loaded module (every GPU that loads the
// library holds its 8 MiB until the process exits).
//
// Set-up: the first call on a device looks up the array's device address
// with cudaGetSymbolAddress while that device is current, checks the result
// and caches it per device; make that first call before any stream capture.
// The cached address belongs to the device's primary context as it was when
// the first call ran: after cudaDeviceReset (or any reset of the primary
// context) the module is loaded again at a new address, so do not use this
// entry point in a process that resets a device it has already used.
// All calls share the one array, so calls that overlap on the GPU (different
// streams, or the same array from several host threads) race; serialise
// them. Each call writes every scratch element it later reads, so nothing
// needs clearing between calls.
//
// The scan is the one of rb_tb.cu (Brightness.single, brightness.py:53-117):
// chunks scanned in parallel from a local optical depth of zero, then
// combined as sum_c exp(-tau_c) * partial_c.
#include <cstdio>
#include <mutex>

#include "../../include/radiobear_gb300.h"
#include "rb_args.cuh"

namespace rb {
void set_last_error(const char* msg);   // rb_api.cu: the message rb_last_error returns
}

namespace {

constexpr int NA_CHUNK = 128;
constexpr double NA_T_CMB = 2.725;   // utils.py:77
// Maximum scratch: nb * ceil(max_seg / 128) * nf float4 elements (8 MiB).
constexpr size_t NA_SCRATCH_ELEMS = RB_NOALLOC_SCRATCH_ELEMS;

static __device__ __align__(256) float4 g_rb_noalloc_scratch[NA_SCRATCH_ELEMS];

constexpr int NA_MAX_DEVICES = 64;
std::mutex g_na_mu;
float4* g_na_addr[NA_MAX_DEVICES] = {};

__device__ __forceinline__ void na_two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

__device__ __forceinline__ void na_kahan(float& s, float& c, float v) {
  const float y = v - c;
  const float t = s + y;
  c = (t - s) - y;
  s = t;
}

// Layer index with Python wrap; out-of-range values are clamped so a bad
// index can never address outside alpha / T.
__device__ __forceinline__ int na_layer(int l, int nL) {
  l = l < 0 ? l + nL : l;
  return l < 0 ? 0 : (l >= nL ? nL - 1 : l);
}

__global__ void __launch_bounds__(128)
    rb_tb_chunk_noalloc_kernel(int nL, int nf, int max_seg, int nchunk, const float* alpha32,
                               const double* T, const int* nseg_in, const double* ds,
                               const int* layer, float4* part_all) {
  // rays in blockIdx.x (up to 2^31 - 1 of them), chunks in y, frequency blocks in z
  const int ray = blockIdx.x;
  const int ch = blockIdx.y;
  const int f = blockIdx.z * blockDim.x + threadIdx.x;
  const int nseg = min(max(nseg_in[ray], 0), max_seg);
  const int nsteps = nseg - 1;
  const int i0 = ch * NA_CHUNK;
  float4* part = part_all + ((size_t)ray * nchunk + ch) * nf;
  if (i0 >= nsteps) {
    if (f < nf) part[f] = make_float4(0.f, 0.f, 0.f, 0.f);
    return;
  }
  const int n = min(NA_CHUNK, nsteps - i0);
  __shared__ int s_off[NA_CHUNK + 1];
  __shared__ float s_T[NA_CHUNK + 1];
  __shared__ float s_hd[NA_CHUNK];
  const double* dsr = ds + (size_t)ray * max_seg + i0;
  const int* lay = layer + (size_t)ray * max_seg + i0;
  for (int t = threadIdx.x; t <= n; t += blockDim.x) {
    const int l = na_layer(lay[t], nL);
    s_off[t] = l * nf;
    s_T[t] = (float)T[l];
    if (t < n) s_hd[t] = (float)(dsr[t] * 1.0e3 / 1.0e-2 / 2.0);   // km -> cm, halved
  }
  __syncthreads();
  if (f >= nf) return;
  const float* al = alpha32 + f;
  float th = 0.f, tl = 0.f;
  float a0 = al[s_off[0]];
  float W0 = (i0 == 0) ? 0.f : a0;     // W_0 = 0 on a path; otherwise relative to exp(-tau_start)
  float T0 = s_T[0];
  float iw = 0.f, iwc = 0.f, tb = 0.f, tbc = 0.f;
  for (int i = 0; i < n; ++i) {
    const float hd = s_hd[i];
    const float a1 = al[s_off[i + 1]];
    const float T1 = s_T[i + 1];
    float s, e;
    na_two_sum(th, (a0 + a1) * hd, s, e);
    e += tl;
    th = s + e;
    tl = e - (th - s);
    const float W1 = a1 * __expf(-th) * (1.f - tl);
    na_kahan(iw, iwc, (W1 + W0) * hd);
    na_kahan(tb, tbc, fmaf(T1, W1, T0 * W0) * hd);
    W0 = W1;
    T0 = T1;
    a0 = a1;
  }
  part[f] = make_float4(th, tl, iw - iwc, tb - tbc);
}

__global__ void __launch_bounds__(128)
    rb_tb_combine_noalloc_kernel(int nf, int max_seg, int nchunk, const int* nseg_in,
                                 const float4* part_all, double* Tb) {
  const int ray = blockIdx.x;
  const int f = blockIdx.y * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  const float4* part = part_all + (size_t)ray * nchunk * nf + f;
  const int nsteps = min(max(nseg_in[ray], 0), max_seg) - 1;
  const int nc = nsteps > 0 ? (nsteps + NA_CHUNK - 1) / NA_CHUNK : 0;
  float ph = 0.f, pl = 0.f;
  float iw = 0.f, iwc = 0.f, tb = 0.f, tbc = 0.f;
  for (int c = 0; c < nc; ++c) {
    const float4 p = part[(size_t)c * nf];
    const float sc = __expf(-ph) * (1.f - pl);
    na_kahan(iw, iwc, sc * p.z);
    na_kahan(tb, tbc, sc * p.w);
    float s, e;
    na_two_sum(ph, p.x, s, e);
    e += pl + p.y;
    ph = s + e;
    pl = e - (ph - s);
  }
  const float TbL = tb - tbc, IW = iw - iwc;
  // off the planet or no emission: T_cmb (utils.py:77) stored exactly in
  // double, as the allocating scan stores it
  const bool clamped = TbL < (float)NA_T_CMB;
  Tb[(size_t)ray * nf + f] = clamped ? NA_T_CMB : (double)(TbL / IW);
}

int na_fail(int code, const char* msg) {
  rb::set_last_error(msg);
  return code;
}

}  // namespace

extern "C" int rb_brightness_noalloc(void* stream, int nL, int nf, const float* alpha32,
                                     const double* T, int nb, const int32_t* nseg,
                                     const double* ds, const int32_t* layer, int max_seg,
                                     double* Tb) {
  if (nL < 1 || nf < 1 || nb < 0 || max_seg < 1) return na_fail(RB_EINVAL, "bad sizes");
  if (nb == 0) return RB_OK;
  if (!alpha32 || !T || !nseg || !ds || !layer || !Tb) return na_fail(RB_EINVAL, "null pointer");
  const int nchunk = (max_seg + NA_CHUNK - 1) / NA_CHUNK;
  const int nfblk = (nf + 127) / 128;
  if (nchunk > 65535 || nfblk > 65535)
    return na_fail(RB_EINVAL, "rb_brightness_noalloc: max_seg or nf beyond the launch grid "
                              "(ceil(max_seg/128) and ceil(nf/128) must be at most 65535)");
  const size_t need = (size_t)nb * nchunk * nf;
  if (need > NA_SCRATCH_ELEMS) {
    char msg[256];
    snprintf(msg, sizeof(msg),
             "rb_brightness_noalloc: nb * ceil(max_seg/128) * nf = %zu scratch elements exceeds "
             "the fixed maximum %zu (8 MiB); split the rays into smaller calls",
             need, (size_t)NA_SCRATCH_ELEMS);
    return na_fail(RB_EINVAL, msg);
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return na_fail(RB_ECUDA, "cudaGetDevice failed");
  if (dev < 0 || dev >= NA_MAX_DEVICES) return na_fail(RB_EINVAL, "device index out of range");
  float4* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_na_mu);
    if (!g_na_addr[dev]) {
      void* p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&p, g_rb_noalloc_scratch);
      if (e != cudaSuccess || !p) return na_fail(RB_ECUDA, cudaGetErrorString(e));
      g_na_addr[dev] = static_cast<float4*>(p);
    }
    scratch = g_na_addr[dev];
  }
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  dim3 grid(nb, nchunk, nfblk);
  rb_tb_chunk_noalloc_kernel<<<grid, 128, 0, st>>>(nL, nf, max_seg, nchunk, alpha32, T, nseg, ds,
                                                   layer, scratch);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return na_fail(RB_ECUDA, cudaGetErrorString(e));
  dim3 g2(nb, nfblk);
  rb_tb_combine_noalloc_kernel<<<g2, 128, 0, st>>>(nf, max_seg, nchunk, nseg, scratch, Tb);
  e = cudaGetLastError();
  if (e != cudaSuccess) return na_fail(RB_ECUDA, cudaGetErrorString(e));
  return RB_OK;
}
