// Ray path through the layered (ellipse-geoid) atmosphere: a float64
// restatement of raypath.compute_ds / findEdge (raypath.py:60-273) and
// Shape._calcEllipse (shape.py:223-274) for sm_103a.
//
// One warp per ray.  findEdge's trial points (a 0.005 rNorm march along the
// line of sight, raypath.py:62-87) are evaluated 32 at a time, one per lane,
// and the first point inside the top shell is found with a ballot.  The
// shell walk itself is a dependent chain and runs on lane 0.
//
// The walk follows the reference step by step:
//   * the shell radii are the ellipse radius of shell `layer` at the current
//     point's planetocentric latitude (rNow, rNext);
//   * ds = -r.s -/+ sqrt((r.s)^2 + rNext^2 - rNow^2) (ingress / egress);
//   * a negative discriminant on ingress is the tangent layer (chord -2 r.s,
//     then egress); on egress it ends the path (raypath.py:191-209);
//   * refraction only at the first step (nratio = nr[0]/nr[1]); afterwards
//     nratio = 1 so the s-update reduces to s += dir*(c-|c|)*n with
//     c = -dir s.n (zero unless the ray meets the local normal at more than
//     90 degrees, where the reference's arcsin(sin t) folds the angle);
//   * the path ends where the reference's `nr[layer + dir]` index check
//     raises (Python negative indices wrap, so egress runs out at layer -1).
// Latitude and longitude enter only through sin/cos, which are formed from
// the vector components directly (lat = 0 keeps the reference's 1e-6 rad
// substitution).
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

__device__ __forceinline__ LatLng latlng_of(double x, double y, double z) {
  LatLng o;
  const double rho2 = x * x + z * z;
  const double rho = sqrt(rho2);
  const double rr = sqrt(rho2 + y * y);
  if (y == 0.0) {
    o.sl = 9.9999999999983336e-07;   // sin(1e-6)
    o.cl = 0.99999999999950007;      // cos(1e-6)
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

__device__ __forceinline__ double ellipse_factor(const LatLng& g, double k) {
  // |[0, k a sin, a cos]| / a
  return sqrt((k * g.sl) * (k * g.sl) + g.cl * g.cl);
}

__device__ __forceinline__ void ellipse_normal(const LatLng& g, double k, double& nx, double& ny,
                                               double& nz) {
  // rotY(lng, [0, a sin, b cos]/|.|)
  const double v1 = g.sl, v2 = k * g.cl;
  const double inv = 1.0 / sqrt(v1 * v1 + v2 * v2);
  const double n1 = v1 * inv, n2 = v2 * inv;
  nx = g.sg * n2;
  ny = n1;
  nz = g.cg * n2;
}

__device__ __forceinline__ double layer_R(const double* R, int nL, int idx) {
  return R[idx < 0 ? idx + nL : idx];
}

__global__ void __launch_bounds__(32) rb_raypath_kernel(RayArgs a) {
  const int ray = blockIdx.x;
  const int lane = threadIdx.x;
  if (ray >= a.nb) return;
  const double b0 = a.b[2 * ray], b1 = a.b[2 * ray + 1];
  const int nL = a.nL;
  const double rNorm = a.R[0];
  const double k = a.k;
  double* ds_out = a.ds + (size_t)ray * a.max_seg;
  int* lay_out = a.layer + (size_t)ray * a.max_seg;
  double* r4_out = a.r4ds ? a.r4ds + (size_t)ray * a.max_seg : nullptr;
  double* ll_out = a.latlng ? a.latlng + (size_t)ray * (a.max_seg + 1) * 2 : nullptr;

  const double tmp = b0 * b0 + b1 * b1;
  if (tmp >= 1.0) {   // raypath.py:126-127
    if (lane == 0) {
      a.nseg[ray] = 0;
      if (a.end_code) a.end_code[ray] = 0;
    }
    return;
  }
  // ---------------- findEdge (raypath.py:60-105), numpy arange semantics
  const double start = sqrt(1.0 - tmp) * 1.01;
  const long ntrial = (long)ceil((0.0 - start) / -0.005);
  const double delta = (start + -0.005) - start;
  long hit = -1;
  double d_hit = 0.0, z_hit = 0.0, d_prev = 0.0, z_prev = 0.0;
  double d_last_lane31 = 0.0, z_last_lane31 = 0.0;
  for (long base = 0; base < ntrial && hit < 0; base += 32) {
    const long i = base + lane;
    double d = 0.0, z = 0.0;
    bool h = false;
    if (i < ntrial) {
      z = (i == 0) ? start : start + (double)i * delta;
      double vx, vy, vz;
      rot_apply(a.rot, b0, b1, z, vx, vy, vz);
      const double r1 = sqrt(vx * vx + vy * vy + vz * vz) * rNorm;
      const LatLng g = latlng_of(vx, vy, vz);
      const double r2 = rNorm * ellipse_factor(g, k);
      d = r1 - r2;
      h = r1 < r2;
    }
    const unsigned m = __ballot_sync(0xffffffffu, h);
    const double dprev_in = __shfl_up_sync(0xffffffffu, d, 1);
    const double zprev_in = __shfl_up_sync(0xffffffffu, z, 1);
    if (m) {
      const int first = __ffs(m) - 1;
      const double dp = (first == 0) ? d_last_lane31 : dprev_in;
      const double zp = (first == 0) ? z_last_lane31 : zprev_in;
      d_hit = __shfl_sync(0xffffffffu, d, first);
      z_hit = __shfl_sync(0xffffffffu, z, first);
      d_prev = __shfl_sync(0xffffffffu, dp, first);
      z_prev = __shfl_sync(0xffffffffu, zp, first);
      hit = base + first;
    }
    d_last_lane31 = __shfl_sync(0xffffffffu, d, 31);
    z_last_lane31 = __shfl_sync(0xffffffffu, z, 31);
  }
  if (lane != 0) return;
  if (hit < 0) {
    a.nseg[ray] = 0;
    if (a.end_code) a.end_code[ray] = 0;
    return;
  }
  double zQ;
  if (hit == 0) {
    zQ = z_hit;    // np.interp on a single point
  } else {         // np.interp(0, [d_hit, d_prev], [z_hit, z_prev])
    const double slope = (z_prev - z_hit) / (d_prev - d_hit);
    zQ = slope * (0.0 - d_hit) + z_hit;
  }
  double ex, ey, ez;
  rot_apply(a.rot, b0, b1, zQ, ex, ey, ez);
  ex *= rNorm;
  ey *= rNorm;
  ez *= rNorm;
  // ---------------- initial point on the top shell (raypath.py:130-160)
  LatLng g = latlng_of(ex, ey, ez);
  double E = ellipse_factor(g, k);
  double rx = g.sg * (rNorm * g.cl), ry = k * rNorm * g.sl, rz = g.cg * (rNorm * g.cl);
  double nx, ny, nz;
  ellipse_normal(g, k, nx, ny, nz);
  double rNow = rNorm * E;
  double sx, sy, sz;
  rot_apply(a.rot, 0.0, 0.0, -1.0, sx, sy, sz);
  {
    const double c0 = -(sx * nx + sy * ny + sz * nz);
    const double t_inc = (c0 >= -1.0 && c0 <= 1.0) ? acos(c0) : CUDART_NAN;
    const double nratio = a.N[0] / a.N[1];
    const double t_tran = asin(nratio * sin(t_inc));
    const double cf = nratio * cos(t_inc) - cos(t_tran);
    sx = nratio * sx + cf * nx;
    sy = nratio * sy + cf * ny;
    sz = nratio * sz + cf * nz;
  }
  const double mu = sqrt(1.0 - b0 * b0 - b1 * b1);
  int layer = 0;
  int dir = 1;   // +1 ingress, -1 egress
  int nseg = 0;
  int code = 1;
  while (true) {
    if (ll_out) {
      ll_out[2 * nseg] = asin(g.sl) * 180.0 / CUDART_PI;
      ll_out[2 * nseg + 1] = atan2(g.sg, g.cg) * 180.0 / CUDART_PI;
    }
    double rNext = layer_R(a.R, nL, layer + dir) * E;
    const double rdots = rx * sx + ry * sy + rz * sz;
    const double disc = rdots * rdots + rNext * rNext - rNow * rNow;
    bool tangent = false;
    double step;
    if (disc < 0.0) {
      if (dir == 1) {
        tangent = true;
        step = -2.0 * rdots;
        if (step > rNorm) {
          code = 2;
          break;
        }
        rNext = rNow;
      } else {
        code = 2;
        break;
      }
    } else {
      const double sq = sqrt(disc);
      step = (dir == 1) ? (-rdots - sq) : (-rdots + sq);
    }
    if (step < 0.0) {
      code = 2;
      break;
    }
    if (a.limb_sec) step = fabs(rNext - rNow) / mu;
    if (nseg >= a.max_seg) {
      code = 3;
      break;
    }
    ds_out[nseg] = step;
    lay_out[nseg] = layer;
    if (r4_out) r4_out[nseg] = rNow;
    ++nseg;
    rx += step * sx;
    ry += step * sy;
    rz += step * sz;
    g = latlng_of(rx, ry, rz);
    E = ellipse_factor(g, k);
    const int dv = tangent ? 0 : dir;
    rNow = layer_R(a.R, nL, layer + dv) * E;
    ellipse_normal(g, k, nx, ny, nz);
    layer += dv;
    if (tangent) {
      dir = -1;      // t_inc = pi/2: next s-update is exactly zero
    } else {
      const double c = -(double)dir * (sx * nx + sy * ny + sz * nz);
      if (c > 1.0 || c < -1.0) {
        sx = sy = sz = CUDART_NAN;     // numpy arccos -> nan
      } else if (c < 0.0) {
        const double u = (double)dir * 2.0 * c;
        sx += u * nx;
        sy += u * ny;
        sz += u * nz;
      }
    }
    // nr[layer] / nr[layer + dir] (raypath.py:253-264)
    const int nxt = layer + dir;
    if (layer < -nL || layer >= nL || nxt < -nL || nxt >= nL) {
      code = 1;
      break;
    }
  }
  if (ll_out && code != 3) {
    ll_out[2 * nseg] = asin(g.sl) * 180.0 / CUDART_PI;
    ll_out[2 * nseg + 1] = atan2(g.sg, g.cg) * 180.0 / CUDART_PI;
  }
  a.nseg[ray] = nseg;
  if (a.end_code) a.end_code[ray] = code;
}

cudaError_t launch_raypath(const RayArgs& a, cudaStream_t st) {
  if (a.nb <= 0) return cudaSuccess;
  rb_raypath_kernel<<<a.nb, 32, 0, st>>>(a);
  return cudaGetLastError();
}

}  // namespace rb
