// Exponential integrals E1 and E2 in float64 for the b = 'disc' weighting
// W = 2 a E2(tau) of Brightness.single (brightness.py:96, which calls
// scipy.special.expn(2, tau)) and its derivative dE2/dx = -E1(x)
// (Abramowitz & Stegun 5.1.26), used by the forward scan and the adjoint.
//
//   x <= 1: power series, A&S 5.1.11 (E1) and 5.1.12 with n = 2 (E2);
//   x > 1:  continued fraction A&S 5.1.22, evaluated by the modified Lentz
//           method (Thompson & Barnett 1986);
//   x > 740: 0 (below the smallest double times e^-x).
#pragma once
#include <math_constants.h>

namespace rb {

// E_n(x), n >= 1, x > 1, by the continued fraction of A&S 5.1.22.
__device__ __forceinline__ double expint_cf(int n, double x) {
  const double tiny = 1e-300;
  double bb = x + n;
  double c = 1.0 / tiny;
  double d = 1.0 / bb;
  double h = d;
  for (int i = 1; i < 200; ++i) {
    const double an = -(double)i * (n - 1 + i);
    bb += 2.0;
    d = 1.0 / (an * d + bb);
    c = bb + an / c;
    const double del = c * d;
    h *= del;
    if (fabs(del - 1.0) < 1e-16) break;
  }
  return h * exp(-x);
}

__device__ __forceinline__ double expint2(double x) {
  if (x == 0.0) return 1.0;
  if (!(x > 0.0)) return CUDART_NAN;
  if (x > 740.0) return 0.0;
  if (x <= 1.0) {
    // E2(x) = 1 + x (ln x - 1 + gamma) - sum_{k>=2} (-x)^k / ((k-1) k!)
    const double euler = 0.57721566490153286061;
    double sum = 0.0;
    double fact = -x;  // (-x)^1 / 1!
    for (int kk = 2; kk < 60; ++kk) {
      fact *= -x / kk;                 // (-x)^k / k!
      const double term = fact / (kk - 1);
      sum += term;
      if (fabs(term) < 1e-18 * fabs(sum) + 1e-300) break;
    }
    return 1.0 + x * (log(x) - 1.0 + euler) - sum;
  }
  return expint_cf(2, x);
}

__device__ __forceinline__ double expint1(double x) {
  if (x == 0.0) return CUDART_INF;
  if (!(x > 0.0)) return CUDART_NAN;
  if (x > 740.0) return 0.0;
  if (x <= 1.0) {
    // E1(x) = -gamma - ln x - sum_{k>=1} (-x)^k / (k k!)
    const double euler = 0.57721566490153286061;
    double sum = 0.0;
    double fact = 1.0;
    for (int kk = 1; kk < 60; ++kk) {
      fact *= -x / kk;                 // (-x)^k / k!
      const double term = fact / kk;
      sum += term;
      if (fabs(term) < 1e-18 * fabs(sum) + 1e-300) break;
    }
    return -euler - log(x) - sum;
  }
  return expint_cf(1, x);
}

}  // namespace rb
