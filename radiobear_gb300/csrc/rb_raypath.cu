// Ray path through the layered (ellipse-geoid) atmosphere: a restatement of
// raypath.compute_ds / findEdge (raypath.py:60-273) and Shape._calcEllipse
// (shape.py:223-274) for sm_103a.
//
// rb_ray_setup_kernel, one thread per ray (GB300 float64 costs the same
// per warp instruction whatever the number of active lanes, so the float64
// set-up is spread over the lanes, one ray each):
//  * findEdge's march (trial points 0.005 rNorm apart along the line of
//    sight, raypath.py:62-87) starts just before the line meets the sphere
//    r = max(1, k) rNorm that encloses the top shell (no trial before it can
//    be inside); each trial is tested with r1 < r2 rewritten without square
//    roots (|v|^2 - |v|^4 > (1 - k^2) v_y^2, v the trial point / rNorm); the
//    reference's own float64 formula then confirms the first inside trial
//    and gives the two distances that findEdge interpolates.
//  * The edge point, the first normal and the one refraction at the top
//    (nratio = nr[0]/nr[1]) follow in float64; the result is a RayStart.
// rb_raypath_kernel, one warp per ray:
//  * The shell walk is a dependent chain in float32 / double-float.
//    After the first step the reference sets nratio = 1, so the direction s
//    stays fixed (except the rare fold of arcsin(sin t) when the ray meets
//    the local normal beyond 90 degrees, handled in float64).  The ray is
//    r(S) = r0 + S s and the walk tracks w = u^2, u = r.s, as a double-float:
//    each step of raypath.py:191-196 satisfies exactly
//        u_{i+1}^2 = u_i^2 + D_i,   D_i = E_i^2 (R[next]^2 - R[cur]^2)
//    (= rdots^2 + rNext^2 - rNow^2), E_i^2 = k^2 sin^2(lat) + cos^2(lat) at the
//    current point.  So u_{i+1} = -/+ sqrt(w + D) (ingress / egress) and
//    ds_i = u_{i+1} - u_i, with D in double-float from float64 radius
//    differences.  Accumulating w instead of u keeps the along-ray coordinate
//    exact to ~1e-14 over the whole path, which the tangent chord -2u needs.
//  * disc = w + D < 0 on ingress -> tangent chord ds = -2u, then egress;
//                      on egress  -> leave the atmosphere (raypath.py:197-209).
//  * Blocks of 32 steps run in parallel, one step per lane: with the E^2
//    values at the steps' start points fixed, w after each step is a prefix
//    sum of D over the lanes.  E^2 depends on the position only weakly, so a
//    Jacobi iteration (E^2 guessed, points computed, E^2 re-evaluated) reaches
//    the recurrence's fixed point bitwise in one or two rounds.  Steps with
//    an event (tangent, exit, fold, end of layers) and blocks that do not
//    settle within four rounds are taken sequentially.
#include "rb_args.cuh"
#include <math_constants.h>

namespace rb {

__device__ __forceinline__ void rot_apply(const double* M, double x, double y, double z, double& ox,
                                          double& oy, double& oz) {
  ox = M[0] * x + M[1] * y + M[2] * z;
  oy = M[3] * x + M[4] * y + M[5] * z;
  oz = M[6] * x + M[7] * y + M[8] * z;
}

// sin/cos of planetocentric latitude and longitude of point v, with the
// lat == 0 -> 1e-6 rad rule of shape.py:232-234.
struct LatLng {
  double sl, cl, sg, cg;
};

constexpr double SIN_1EM6 = 9.9999999999983336e-07;   // sin(1e-6)
constexpr double COS_1EM6 = 0.99999999999950007;      // cos(1e-6)

__device__ __forceinline__ LatLng latlng_of(double x, double y, double z) {
  LatLng o;
  const double rho2 = x * x + z * z;
  const double rho = sqrt(rho2);
  const double rr = sqrt(rho2 + y * y);
  if (y == 0.0) {
    o.sl = SIN_1EM6;
    o.cl = COS_1EM6;
  } else {
    o.sl = y / rr;
    o.cl = rho / rr;
  }
  if (rho == 0.0) {
    o.sg = 0.0;
    o.cg = 1.0;
  } else {
    o.sg = x / rho;
    o.cg = z / rho;
  }
  return o;
}

__device__ __forceinline__ double ellipse_factor2(const LatLng& g, double k) {
  return (k * g.sl) * (k * g.sl) + g.cl * g.cl;   // (|[0, k a sin, a cos]| / a)^2
}

__device__ __forceinline__ void ellipse_normal(const LatLng& g, double k, double& nx, double& ny,
                                               double& nz) {
  // rotY(lng, [0, a sin, b cos]/|.|)
  const double v1 = g.sl, v2 = k * g.cl;
  const double inv = 1.0 / sqrt(v1 * v1 + v2 * v2);
  nx = g.sg * (v2 * inv);
  ny = v1 * inv;
  nz = g.cg * (v2 * inv);
}

__device__ __forceinline__ int wrap(int idx, int nL) { return idx < 0 ? idx + nL : idx; }

// R[(c+1)%nL]^2 - R[c]^2 as a double-float (float64 product of the float64
// difference and sum), R[(c+1)%nL] - R[c] and float copies of R and T.
// With var_off (batches), the wrap is within each variant's layers.
__global__ void rb_geom_prep_kernel(int nL, const double* R, const double* T, float2* dR2,
                                    float* dR, float* R32, float* T32, const int* var_off,
                                    int nvar) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nL) return;
  int first = 0, end = nL;
  if (var_off) {   // variant of layer c: var_off[v] <= c < var_off[v+1]
    int lo = 0, hi = nvar;
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (var_off[mid] <= c) lo = mid; else hi = mid;
    }
    first = var_off[lo];
    end = var_off[lo + 1];
  }
  const int n = (c + 1 < end) ? c + 1 : first;
  const double d = R[n] - R[c];
  const double q = d * (R[n] + R[c]);
  float h, l;
  split_double(q, h, l);
  dR2[c] = make_float2(h, l);
  dR[c] = (float)d;
  R32[c] = (float)R[c];
  if (T) T32[c] = (float)T[c];
}

// ---------------- double-float helpers (products and renormalisations in
// _rn intrinsics, which the compiler does not contract into neighbouring
// additions: the error terms must describe the rounded values actually used)
struct df {
  float h, l;
};
__device__ __forceinline__ df df_make(double v) {
  df r;
  split_double(v, r.h, r.l);
  return r;
}
__device__ __forceinline__ df df_add(df a, df b) {
  float s, e;
  two_sum(a.h, b.h, s, e);
  e += a.l + b.l;
  df r;
  r.h = __fadd_rn(s, e);
  r.l = __fsub_rn(e, __fsub_rn(r.h, s));
  return r;
}
__device__ __forceinline__ df df_neg(df a) { return {-a.h, -a.l}; }
// a * b for a double-float and a float
__device__ __forceinline__ df df_mulf(df a, float b) {
  const float p = __fmul_rn(a.h, b);
  const float e = fmaf(a.h, b, -p) + a.l * b;
  df r;
  r.h = __fadd_rn(p, e);
  r.l = __fsub_rn(e, __fsub_rn(r.h, p));
  return r;
}
// a + b without the final renormalisation (prefix scans: the low words
// stay a few ulp of the high word and are renormalised once at the end)
__device__ __forceinline__ df df_add_lazy(df a, df b) {
  float s, e;
  two_sum(a.h, b.h, s, e);
  return {s, e + (a.l + b.l)};
}
// float value of a + b (the high word of the normalised sum)
__device__ __forceinline__ float df_sum(df a, df b) {
  float s, e;
  two_sum(a.h, b.h, s, e);
  return s + (e + (a.l + b.l));
}
// a * b for a double-float and a float, not renormalised
__device__ __forceinline__ df df_mulf_lazy(df a, float b) {
  const float p = __fmul_rn(a.h, b);
  return {p, fmaf(a.h, b, -p) + a.l * b};
}
__device__ __forceinline__ df df_norm(df a) {
  df r;
  r.h = __fadd_rn(a.h, a.l);
  r.l = __fsub_rn(a.l, __fsub_rn(r.h, a.h));
  return r;
}
// sqrt of a positive double-float: one Newton correction of sqrtf(hi); the
// correction (~1e-7 of the result) takes an approximate reciprocal
__device__ __forceinline__ df df_sqrt(df a) {
  const float y = sqrtf(a.h);
  if (y == 0.f) return {0.f, 0.f};
  const float r = fmaf(-y, y, a.h) + a.l;
  df o;
  o.h = y;
  o.l = r * rcp_approx(2.f * y);
  const float t = __fadd_rn(o.h, o.l);
  o.l = __fsub_rn(o.l, __fsub_rn(t, o.h));
  o.h = t;
  return o;
}
__device__ __forceinline__ float df_val(df a) { return a.h + a.l; }
__device__ __forceinline__ double df_d(df a) { return (double)a.h + (double)a.l; }

// findEdge's distance r1 - r2 of trial point z (raypath.py:66-80), float64
// exactly as the reference forms it.
__device__ __forceinline__ double edge_dist(const double* rot, double b0, double b1, double z,
                                            double rNorm, double k) {
  double vx, vy, vz;
  rot_apply(rot, b0, b1, z, vx, vy, vz);
  const double r1 = sqrt(vx * vx + vy * vy + vz * vz) * rNorm;
  const LatLng g = latlng_of(vx, vy, vz);
  const double r2 = rNorm * sqrt(ellipse_factor2(g, k));
  return r1 - r2;
}

// Trial points of findEdge (raypath.py:62-87, numpy arange semantics) and
// the first one that can be inside: the line v(z) = p + z q (rNorm units)
// meets the sphere of radius max(1, k) that encloses the top shell at
// z = -B +/- sqrt(B^2 - A + K^2); every trial above the upper crossing is
// outside.  i0 = -1: the line misses that sphere (no trial is inside).
// Guard band of the float32 trial test: |g| below it is decided in float64.
// g = |v|^2 - |v|^4 - (1 - k^2) v_y^2 with |v| <= ~1.1 carries a float32
// error below ~2e-6 (trial point, rotation and products each within a few
// ulp of 1).
constexpr float EDGE_G_BAND = 3e-5f;

struct EdgeMarch {
  double b0, b1, start, delta, c, ef2_eq;
  long ntrial, i0;
  float px, py, pz, qx, qy, qz, startf, deltaf, cf;   // trial point = P + z Q in float32
  __device__ __forceinline__ double z(long i) const { return i == 0 ? start : start + (double)i * delta; }
  // r1 < r2 of raypath.py:66-80 without square roots:
  // |v|^2 < (k^2 v_y^2 + v_x^2 + v_z^2) / |v|^2  <=>  |v|^2 - |v|^4 > (1 - k^2) v_y^2
  // (v_y == 0 takes the reference's lat = 1e-6 rad rule).
  __device__ __forceinline__ bool inside64(const double* rot, long i) const {
    double vx, vy, vz;
    rot_apply(rot, b0, b1, z(i), vx, vy, vz);
    const double rho = vx * vx + vy * vy + vz * vz;
    return vy == 0.0 ? rho < ef2_eq : rho - rho * rho > c * (vy * vy);
  }
  // The same test, decided in float32 where g is outside the guard band
  // (GB300 runs float32 ~64x faster per warp instruction than float64); the
  // first inside trial is therefore the float64 march's.
  __device__ __forceinline__ bool inside(const double* rot, long i) const {
    const float zf = i == 0 ? startf : fmaf((float)i, deltaf, startf);
    const float vx = fmaf(zf, qx, px), vy = fmaf(zf, qy, py), vz = fmaf(zf, qz, pz);
    const float rho = fmaf(vx, vx, fmaf(vy, vy, vz * vz));
    const float g = fmaf(-rho, rho, rho) - cf * (vy * vy);
    if (g > EDGE_G_BAND) return true;
    if (g < -EDGE_G_BAND) return false;
    return inside64(rot, i);
  }
};

__device__ __forceinline__ EdgeMarch edge_march(const double* rot, double b0, double b1, double k) {
  EdgeMarch m;
  m.b0 = b0;
  m.b1 = b1;
  const double tmp = b0 * b0 + b1 * b1;
  m.start = sqrt(1.0 - tmp) * 1.01;
  m.ntrial = (long)ceil((0.0 - m.start) / -0.005);
  m.delta = (m.start + -0.005) - m.start;
  m.c = 1.0 - k * k;
  m.ef2_eq = ellipse_factor2(latlng_of(1.0, 0.0, 1.0), k);
  double px, py, pz, qx, qy, qz;
  rot_apply(rot, b0, b1, 0.0, px, py, pz);
  rot_apply(rot, 0.0, 0.0, 1.0, qx, qy, qz);
  m.px = (float)px;
  m.py = (float)py;
  m.pz = (float)pz;
  m.qx = (float)qx;
  m.qy = (float)qy;
  m.qz = (float)qz;
  m.startf = (float)m.start;
  m.deltaf = (float)m.delta;
  m.cf = (float)m.c;
  const double K2 = k > 1.0 ? k * k : 1.0;
  const double A = px * px + py * py + pz * pz, B = px * qx + py * qy + pz * qz;
  const double disc = B * B - A + K2;
  m.i0 = disc > 0.0 ? (long)fmax(0.0, floor((m.start - (-B + sqrt(disc))) / 0.005) - 2.0) : -1;
  return m;
}

// From a candidate first-inside trial to findEdge's edge point: the
// reference's own float64 distance confirms the first inside trial (moving
// the candidate if the two tests disagree at the surface) and gives the two
// distances it interpolates.  Returns false if no trial is inside.
__device__ __forceinline__ bool edge_point(const RayArgs& a, const EdgeMarch& m, long hit,
                                           double rNorm, double k, double& zQ) {
  if (hit < 0) return false;
  double d_hit = edge_dist(a.rot, m.b0, m.b1, m.z(hit), rNorm, k), d_prev = 0.0;
  while (!(d_hit < 0.0) && hit + 1 < m.ntrial) {
    ++hit;
    d_hit = edge_dist(a.rot, m.b0, m.b1, m.z(hit), rNorm, k);
  }
  if (!(d_hit < 0.0)) return false;
  while (hit > 0) {
    d_prev = edge_dist(a.rot, m.b0, m.b1, m.z(hit - 1), rNorm, k);
    if (!(d_prev < 0.0)) break;
    --hit;
    d_hit = d_prev;
  }
  if (hit == 0) {
    zQ = m.z(0);   // np.interp on a single point
  } else {         // np.interp(0, [d_hit, d_prev], [z_hit, z_prev])
    const double z_hit = m.z(hit), z_prev = m.z(hit - 1);
    const double slope = (z_prev - z_hit) / (d_prev - d_hit);
    zQ = slope * (0.0 - d_hit) + z_hit;
  }
  return true;
}

// Edge point, first normal and the one refraction (raypath.py:106-160).
__device__ __forceinline__ void ray_start(const RayArgs& a, double b0, double b1, double zQ,
                                          double rNorm, double k, const double* N_, RayStart& o) {
  double ex, ey, ez;
  rot_apply(a.rot, b0, b1, zQ, ex, ey, ez);
  ex *= rNorm;
  ey *= rNorm;
  ez *= rNorm;
  const LatLng g0 = latlng_of(ex, ey, ez);
  o.r0[0] = g0.sg * (rNorm * g0.cl);
  o.r0[1] = k * rNorm * g0.sl;
  o.r0[2] = g0.cg * (rNorm * g0.cl);
  double nx, ny, nz;
  ellipse_normal(g0, k, nx, ny, nz);
  double sx, sy, sz;
  rot_apply(a.rot, 0.0, 0.0, -1.0, sx, sy, sz);
  {
    // raypath.py:150-160: t_inc = arccos(c0), t_tran = arcsin(nratio sin t_inc),
    // cf = nratio cos t_inc - cos t_tran, with sin(arccos c0) = sqrt(1 - c0^2)
    // and cos(arcsin x) = sqrt(1 - x^2) (no trigonometric calls; nan where
    // numpy's arccos / arcsin give nan)
    const double c0 = -(sx * nx + sy * ny + sz * nz);
    const double nratio = N_[0] / N_[1];
    const double s2 = fma(-c0, c0, 1.0);                      // sin^2 t_inc
    const double ct2 = fma(-(nratio * nratio), s2, 1.0);      // cos^2 t_tran
    const double cf = (c0 >= -1.0 && c0 <= 1.0) ? nratio * c0 - sqrt(ct2) : CUDART_NAN;
    sx = nratio * sx + cf * nx;
    sy = nratio * sy + cf * ny;
    sz = nratio * sz + cf * nz;
  }
  o.s[0] = sx;
  o.s[1] = sy;
  o.s[2] = sz;
  o.u0 = o.r0[0] * sx + o.r0[1] * sy + o.r0[2] * sz;
  o.ll0[0] = o.ll0[1] = 0.0;
  if (a.latlng) {
    o.ll0[0] = (g0.sl == SIN_1EM6) ? 0.0 : asin(g0.sl) * 180.0 / CUDART_PI;
    o.ll0[1] = atan2(g0.sg, g0.cg) * 180.0 / CUDART_PI;
  }
  o.em1 = (float)(ellipse_factor2(g0, k) - 1.0);   // step 0 uses the edge's latitude
  o.em1_eq = (float)(ellipse_factor2(latlng_of(1.0, 0.0, 1.0), k) - 1.0);
  o.mu = (float)sqrt(1.0 - b0 * b0 - b1 * b1);
  o.hit = 1;
}

// Impact parameter and layer block of ray `ray`.
__device__ __forceinline__ void ray_geometry(const RayArgs& a, int ray, double& b0, double& b1,
                                             int& off, int& nL) {
  const int bi = a.var_off ? ray % a.rays_per_var : ray;
  b0 = a.b[2 * bi];
  b1 = a.b[2 * bi + 1];
  off = 0;
  nL = a.nL;
  if (a.var_off) {
    const int v = ray / a.rays_per_var;
    off = a.var_off[v];
    nL = a.var_off[v + 1] - off;
  }
}

// One thread per ray (many rays): findEdge trial by trial from the first
// trial that can be inside, then the start of the walk.
__global__ void __launch_bounds__(128) rb_ray_setup_kernel(RayArgs a) {
  const int ray = blockIdx.x * blockDim.x + threadIdx.x;
  if (ray >= a.nb) return;
  RayStart o{};
  double b0, b1;
  int off, nL;
  ray_geometry(a, ray, b0, b1, off, nL);
  const double rNorm = a.R[off];
  if (b0 * b0 + b1 * b1 < 1.0) {   // raypath.py:126-127
    const EdgeMarch m = edge_march(a.rot, b0, b1, a.k);
    long hit = -1;
    if (m.i0 >= 0)
      for (long i = m.i0; i < m.ntrial; ++i)
        if (m.inside(a.rot, i)) {
          hit = i;
          break;
        }
    double zQ;
    if (edge_point(a, m, hit, rNorm, a.k, zQ)) ray_start(a, b0, b1, zQ, rNorm, a.k, a.N + off, o);
  }
  a.start[ray] = o;
}

// One warp per ray (few rays): findEdge 32 trials a pass, the rest of the
// set-up evaluated alike on every lane (the walk then starts at once).
__device__ __forceinline__ void ray_setup_warp(const RayArgs& a, int ray, int lane, RayStart& o) {
  o = RayStart{};
  double b0, b1;
  int off, nL;
  ray_geometry(a, ray, b0, b1, off, nL);
  const double rNorm = a.R[off];
  if (b0 * b0 + b1 * b1 >= 1.0) return;   // raypath.py:126-127
  const EdgeMarch m = edge_march(a.rot, b0, b1, a.k);
  long hit = -1;
  if (m.i0 >= 0)
    for (long base = m.i0; base < m.ntrial && hit < 0; base += 32) {
      const long i = base + lane;
      const unsigned in = __ballot_sync(0xffffffffu, i < m.ntrial && m.inside(a.rot, i));
      if (in) hit = base + __ffs(in) - 1;
    }
  double zQ;
  if (edge_point(a, m, hit, rNorm, a.k, zQ)) ray_start(a, b0, b1, zQ, rNorm, a.k, a.N + off, o);
}

// One warp per ray, WPC rays per CTA (64 registers either way).
template <int WPC>
__global__ void __launch_bounds__(32 * WPC, 32 / WPC) rb_raypath_kernel(RayArgs a) {
  const int ray = blockIdx.x * WPC + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (ray >= a.nb) return;   // whole warps
  int off = 0, nL = a.nL;
  if (a.var_off) {
    const int v = ray / a.rays_per_var;
    off = a.var_off[v];
    nL = a.var_off[v + 1] - off;
  }
  const double* R_ = a.R + off;
  const float2* dR2_ = a.dR2 + off;
  const float* dR_ = a.dR + off;
  const float* R32_ = a.R32 + off;
  const double rNorm = R_[0];
  const double k = a.k;
  double* ds_out = a.ds ? a.ds + (size_t)ray * a.max_seg : nullptr;
  float* hds_out = a.hds ? a.hds + (size_t)ray * a.max_seg : nullptr;
  int* lay_out = a.layer + (size_t)ray * a.max_seg;
  double* r4_out = a.r4ds ? a.r4ds + (size_t)ray * a.max_seg : nullptr;
  double* ll_out = a.latlng ? a.latlng + (size_t)ray * (a.max_seg + 1) * 2 : nullptr;
  RayStart rs;
  if (a.start) rs = a.start[ray];
  else ray_setup_warp(a, ray, lane, rs);
  if (!rs.hit) {
    if (lane == 0) {
      a.nseg[ray] = 0;
      if (a.end_code) a.end_code[ray] = 0;
    }
    return;
  }
  // every lane holds the same state; lane 0 writes the outputs of
  // sequential steps, lane i those of the i-th step of a parallel block
  double r0x = rs.r0[0], r0y = rs.r0[1], r0z = rs.r0[2];
  double sx = rs.s[0], sy = rs.s[1], sz = rs.s[2];
  double nx, ny, nz;
  const float mu = rs.mu;
  const float omk2 = (float)(1.0 - k * k);
  // parametrisation r(S) = r0 + S s; S = u - u0
  double u0 = rs.u0;
  df u = df_make(u0);
  df mu0 = df_neg(u);
  df w = df_make(u0 * u0);
  float R0sq = (float)(r0x * r0x + r0y * r0y + r0z * r0z);
  float twou0 = (float)(2.0 * u0);
  float y0 = (float)r0y, syf = (float)sy;
  // E^2 - 1 at the current point (step 0 uses the edge's latitude)
  float em1 = rs.em1;
  const float kf = (float)k;
  const float em1_eq = rs.em1_eq;
  const unsigned FULL = 0xffffffffu;

  int layer = 0;
  int dir = 1;   // +1 ingress, -1 egress
  int nseg = 0;
  int code = 1;
  const bool par_ok = !a.limb_sec && !ll_out;
  bool done = false;
  while (!done) {
    // nr[layer] / nr[layer + dir] index check (raypath.py:253-264) after the
    // steps of a parallel block
    if (layer < -nL || layer >= nL || layer + dir < -nL || layer + dir >= nL) {
      code = 1;
      break;
    }
    // ======== parallel block: up to 32 steps, one per lane
    int taken = 0;
    if (par_ok) {
      const int c = layer + lane * dir;
      const bool inrange = c >= -nL && c < nL && c + dir >= -nL && c + dir < nL;
      df dr2 = {0.f, 0.f};
      if (inrange) {
        const float2 q2 = dR2_[dir > 0 ? c : wrap(c - 1, nL)];
        dr2 = dir > 0 ? df{q2.x, q2.y} : df{-q2.x, -q2.y};
      }
      float g = em1;            // E^2 - 1 at this lane's start point (guess)
      df W = w, un = u;
      float em1n = em1;
      int first = 32;
      bool conv = false;
      for (int it = 0; it < 4 && !conv; ++it) {
        const df D = df_add_lazy(dr2, df_mulf_lazy(dr2, g));   // renormalised after the scan
        df v = D;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const float h = __shfl_up_sync(FULL, v.h, o), l = __shfl_up_sync(FULL, v.l, o);
          if (lane >= o) v = df_add_lazy(df{h, l}, v);
        }
        W = df_norm(df_add_lazy(w, v));
        const bool negl = W.h < 0.f || (W.h == 0.f && W.l < 0.f);
        const df r = df_sqrt(negl ? df{0.f, 0.f} : W);
        un = dir == 1 ? df_neg(r) : r;
        const float S = df_sum(un, mu0);
        const float rr2 = fmaf(S, S + twou0, R0sq);
        const float y = fmaf(S, syf, y0);
        em1n = (y == 0.f) ? em1_eq : -omk2 * __fdividef(y * y, rr2);
        if (it == 0) {   // predictor: one shared guess almost never is the fixed point
          g = __shfl_up_sync(FULL, em1n, 1);
          if (lane == 0) g = em1;
          continue;
        }
        // fold check at the new point (c < 0 <=> dir (k u + (1-k) s_y y) > 0)
        const float uf = df_val(un);
        const float val = (float)dir * fmaf(kf, uf, (1.f - kf) * syf * y);
        const float tol = 1e-5f * (fabsf(kf * uf) + fabsf((1.f - kf) * syf * y));
        const bool ev = !inrange || negl || val > -tol;
        const unsigned evm = __ballot_sync(FULL, ev);
        first = evm ? __ffs(evm) - 1 : 32;
        float gn = __shfl_up_sync(FULL, em1n, 1);
        if (lane == 0) gn = em1;
        const unsigned diff = __ballot_sync(FULL, gn != g);
        const unsigned below = first >= 32 ? FULL : ((1u << first) - 1u);
        conv = (diff & below) == 0;
        g = gn;
      }
      if (conv) {
        taken = min(first, a.max_seg - nseg);
        if (taken > 0) {
          const float uph = __shfl_up_sync(FULL, un.h, 1), upl = __shfl_up_sync(FULL, un.l, 1);
          const df uprev = lane == 0 ? u : df{uph, upl};
          if (lane < taken) {
            const float step = df_sum(un, df_neg(uprev));
            if (ds_out) ds_out[nseg + lane] = (double)step;
            if (hds_out) hds_out[nseg + lane] = step * 0.5e5f;
            lay_out[nseg + lane] = c;
            if (r4_out) r4_out[nseg + lane] = (double)(R32_[wrap(c, nL)] * sqrtf(1.f + g));
          }
          const int src = taken - 1;
          u.h = __shfl_sync(FULL, un.h, src);
          u.l = __shfl_sync(FULL, un.l, src);
          w.h = __shfl_sync(FULL, W.h, src);
          w.l = __shfl_sync(FULL, W.l, src);
          em1 = __shfl_sync(FULL, em1n, src);
          layer += taken * dir;
          nseg += taken;
          continue;   // events at lane `taken` are handled on the next pass
        }
      }
    }
    // ======== one sequential step (tangent, exit, fold, end of path, or
    //          a block that did not converge); identical on every lane
    if (ll_out && lane == 0) {   // float64 reconstruction of the current point
      if (nseg == 0) {
        ll_out[0] = rs.ll0[0];
        ll_out[1] = rs.ll0[1];
      } else {
        const double S64 = df_d(u) - u0;
        const LatLng g = latlng_of(r0x + S64 * sx, r0y + S64 * sy, r0z + S64 * sz);
        ll_out[2 * nseg] = (g.sl == SIN_1EM6) ? 0.0 : asin(g.sl) * 180.0 / CUDART_PI;
        ll_out[2 * nseg + 1] = atan2(g.sg, g.cg) * 180.0 / CUDART_PI;
      }
    }
    const int j = dir > 0 ? layer : wrap(layer - 1, nL);
    const float2 q2 = dR2_[j];
    df dr2 = {q2.x, q2.y};
    if (dir < 0) dr2 = df_neg(dr2);                  // R[c-1]^2 - R[c]^2
    const df D = df_add(dr2, df_mulf(dr2, em1));     // E^2 (R[next]^2 - R[cur]^2)
    const df wn = df_add(w, D);
    const bool neg = wn.h < 0.f || (wn.h == 0.f && wn.l < 0.f);
    bool tangent = false;
    float step;
    df un;
    if (neg) {
      if (dir == 1) {
        tangent = true;
        step = -2.f * df_val(u);
        if ((double)step > rNorm) {
          code = 2;
          break;
        }
        un = df_neg(u);                              // egress starts at -u, w unchanged
      } else {
        code = 2;
        break;
      }
    } else {
      const df r = df_sqrt(wn);
      un = dir == 1 ? df_neg(r) : r;
      step = df_sum(un, df_neg(u));
      w = wn;
    }
    if (step < 0.f) {
      code = 2;
      break;
    }
    if (a.limb_sec) {
      // the secant step moves the point by |rNext - rNow| / mu instead
      step = tangent ? 0.f : sqrtf(1.f + em1) * fabsf(dR_[j]) / mu;
      un = df_add(u, df{step, 0.f});
      w = df_make(df_d(un) * df_d(un));
    }
    if (nseg >= a.max_seg) {
      code = 3;
      break;
    }
    if (lane == 0) {
      if (ds_out) ds_out[nseg] = (double)step;
      if (hds_out) hds_out[nseg] = step * 0.5e5f;
      lay_out[nseg] = layer;
      if (r4_out) r4_out[nseg] = (double)(R32_[wrap(layer, nL)] * sqrtf(1.f + em1));
    }
    ++nseg;
    // advance along the ray
    u = un;
    const float S = df_sum(u, mu0);
    const float rr2 = fmaf(S, S + twou0, R0sq);
    const float y = fmaf(S, syf, y0);
    em1 = (y == 0.f) ? em1_eq : -omk2 * __fdividef(y * y, rr2);
    const int dv = tangent ? 0 : dir;
    layer += dv;
    if (tangent) {
      dir = -1;      // t_inc = pi/2: the next s-update is exactly zero
    } else {
      // c = -dir s.n with n ~ [k x, y, k z]:  c < 0  <=>  dir (k u + (1-k) s_y y) > 0
      const float un_f = df_val(u);
      const float val = (float)dir * fmaf(kf, un_f, (1.f - kf) * syf * y);
      const float tol = 1e-5f * (fabsf(kf * un_f) + fabsf((1.f - kf) * syf * y));
      if (val > -tol) {   // possible fold: decide and apply in float64
        const double S64 = df_d(u) - u0;
        const double rx = r0x + S64 * sx, ry = r0y + S64 * sy, rz = r0z + S64 * sz;
        const LatLng g = latlng_of(rx, ry, rz);
        ellipse_normal(g, k, nx, ny, nz);
        const double c = -(double)dir * (sx * nx + sy * ny + sz * nz);
        bool moved = false;
        if (c > 1.0 || c < -1.0) {
          sx = sy = sz = CUDART_NAN;       // numpy arccos -> nan
          moved = true;
        } else if (c < 0.0) {
          const double wgt = (double)dir * 2.0 * c;
          sx += wgt * nx;
          sy += wgt * ny;
          sz += wgt * nz;
          moved = true;
        }
        if (moved) {   // restart the parametrisation at this point
          r0x = rx;
          r0y = ry;
          r0z = rz;
          u0 = rx * sx + ry * sy + rz * sz;
          u = df_make(u0);
          mu0 = df_neg(u);
          w = df_make(u0 * u0);
          R0sq = (float)(rx * rx + ry * ry + rz * rz);
          twou0 = (float)(2.0 * u0);
          y0 = (float)ry;
          syf = (float)sy;
        }
      }
    }
    // nr[layer] / nr[layer + dir] index check (raypath.py:253-264)
    const int nxt = layer + dir;
    if (layer < -nL || layer >= nL || nxt < -nL || nxt >= nL) {
      code = 1;
      break;
    }
  }
  if (lane == 0) {
    if (ll_out && code != 3 && nseg == 0) {
      ll_out[0] = rs.ll0[0];
      ll_out[1] = rs.ll0[1];
    } else if (ll_out && code != 3) {
      const double S64 = df_d(u) - u0;
      const LatLng g = latlng_of(r0x + S64 * sx, r0y + S64 * sy, r0z + S64 * sz);
      ll_out[2 * nseg] = (g.sl == SIN_1EM6) ? 0.0 : asin(g.sl) * 180.0 / CUDART_PI;
      ll_out[2 * nseg + 1] = atan2(g.sg, g.cg) * 180.0 / CUDART_PI;
    }
    a.nseg[ray] = nseg;
    if (a.end_code) a.end_code[ray] = code;
  }
}

cudaError_t launch_geom_prep(int nL, const double* R, const double* T, float2* dR2, float* dR,
                             float* R32, float* T32, const int* var_off, int nvar,
                             cudaStream_t st) {
  rb_geom_prep_kernel<<<(nL + 127) / 128, 128, 0, st>>>(nL, R, T, dR2, dR, R32, T32, var_off, nvar);
  return cudaGetLastError();
}

// Few rays (the walk then runs beside the absorption's line sums): four
// rays per CTA, one warp on each scheduler of an SM.  A walk warp's 64
// registers do not fit in a scheduler's register file beside six line-sum
// warps, so each SM holding walk warps gives up one line-sum CTA while they
// run; packed four to a CTA they hold 16 SMs for 64 rays instead of 64.
// Many rays: one per CTA (a CTA's slot frees as soon as its ray ends).
cudaError_t launch_raypath(const RayArgs& a, cudaStream_t st) {
  if (a.nb <= 0) return cudaSuccess;
  if (a.start) rb_ray_setup_kernel<<<(a.nb + 127) / 128, 128, 0, st>>>(a);
  if (a.nb < 2048) rb_raypath_kernel<4><<<(a.nb + 3) / 4, 128, 0, st>>>(a);
  else rb_raypath_kernel<1><<<a.nb, 32, 0, st>>>(a);
  return cudaGetLastError();
}

}  // namespace rb
