// exact.cuh — exact FP64 decisions by error-free transformations: the sign
// of a sum of doubles (Shewchuk's grow-expansion, "Adaptive Precision
// Floating-Point Arithmetic and Fast Robust Geometric Predicates", 1997) and
// ST_DWithin's distance test with a correctly rounded hypot.
#pragma once
#include "common.cuh"

namespace spj {
namespace exact {
namespace {

__device__ __forceinline__ void two_sum(double a, double b, double& s, double& e) {
  s = __dadd_rn(a, b);
  const double bb = __dsub_rn(s, a);
  e = __dadd_rn(__dsub_rn(a, __dsub_rn(s, bb)), __dsub_rn(b, bb));
}

__device__ __forceinline__ void two_prod(double a, double b, double& p, double& e) {
  p = __dmul_rn(a, b);
  e = __fma_rn(a, b, -p);
}

// Sign of the exact sum of n doubles (Shewchuk grow-expansion).
template <int N>
__device__ __forceinline__ int exact_sign(const double (&t)[N]) {
  double e[N];
  int len = 0;
  for (int i = 0; i < N; i++) {
    double q = t[i];
    int nl = 0;
    for (int j = 0; j < len; j++) {
      double s, h;
      two_sum(q, e[j], s, h);
      q = s;
      if (h != 0.0) e[nl++] = h;
    }
    if (q != 0.0) e[nl++] = q;
    len = nl;
  }
  if (len == 0) return 0;
  return e[len - 1] > 0 ? 1 : -1;
}

// Exact decision of RN(sqrt(dx^2 + dy^2)) <= d, i.e. a correctly rounded
// hypot compared with d (ties to even at the rounding midpoint).
__device__ __noinline__ bool dwithin_exact(double2 b, double2 p, double d) {
  const double dx = __dsub_rn(b.x, p.x), dy = __dsub_rn(b.y, p.y);
  if (isnan(dx) || isnan(dy) || isnan(d) || d < 0) return false;
  if (isinf(dx) || isinf(dy)) return isinf(d);
  if (isinf(d)) return true;
  const double up = next_up(d);
  const double ulp = __dsub_rn(up, d);
  // m = d + ulp/2 ; m^2 = d^2 + d*ulp + ulp^2/4 (the last two exact)
  double P1, e1, P2, e2, Q1, q1;
  two_prod(dx, dx, P1, e1);
  two_prod(dy, dy, P2, e2);
  two_prod(d, d, Q1, q1);
  const double Q2 = __dmul_rn(d, ulp);
  const double Q3 = __dmul_rn(__dmul_rn(ulp, ulp), 0.25);
  const double t[8] = {e1, e2, -q1, -Q3, -Q2, P1, P2, -Q1};
  const int sg = exact_sign(t);
  if (sg < 0) return true;
  if (sg > 0) return false;
  // exactly on the midpoint: rounds to the even neighbour
  const unsigned long long bits = (unsigned long long)__double_as_longlong(d);
  return (bits & 1ull) == 0;
}

}  // namespace
}  // namespace exact
}  // namespace spj
