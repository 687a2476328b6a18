// boys.cuh -- device Boys function F_j(T), j = 0..L, in two modes.
//
// Reference parity (MQ_MODE_REFERENCE) restates Boys/Boys1/Boys2/Boys3/BoysG
// (src/integrals/auxilary.f90:85-215,265-285):
//   T < 12          7-term Taylor of F_Q about Tk = NINT(10T)/10 from the
//                   Ftab table, then downward recursion to j = 0, where Q is
//                   the reference's order 3*(sum of the four sets' lmax)
//                   (int2e.f90:654-668) -- Q selects the table columns, so it
//                   must match for the table's bad entries to land the same;
//   12 <= T < 2Q+36 F0 = sqrt(pi)/2 T^-1/2 - e^-T g(T)/T with BoysG's
//                   polynomials, upward recursion;
//   T >= 2Q+36      F0 = sqrt(pi)/2 T^-1/2, upward recursion without e^-T;
// pi is the reference's float-valued constant.  BoysG is undefined for
// T >= 30 in the reference; g = 0.490 is used there (effect < 3e-15).
//
// Tight (MQ_MODE_TIGHT): 9-term Taylor series about the nearest grid point of
// an accurate table (T step 0.1 up to 36, |remainder| < 1e-17), with the
// coefficients F_{m+k}(Tk)/k! stored per order m so that each term is one
// fma: every F_j so for L <= 2, else F_L so and downward recursion; above 36
// F0 = sqrt(pi/T)/2 (erf(sqrt T) = 1 in FP64) and upward recursion.
//
// Table layout in device memory (one buffer, see set_system):
//   parity: Ft(0:120,0:22) column-major (2783 doubles), then Tk/10 (121)
//   tight : tab[Tk][m], 361 x 13 row-major (4693 doubles), then Tk/10 (361),
//           then F_{m+k}(Tk)/k! [m < 5][Tk][k < 9]
#pragma once
#include "internal.h"

namespace mq {

constexpr int BOYS_REF_GRID = FTAB_NT * FTAB_NM;      // offset of Tk/10 values
constexpr int BOYS_TIGHT_GRID = TIGHT_NT * TIGHT_NM;  // offset of Tk/10 values
constexpr int BOYS_TIGHT_SCALED = BOYS_TIGHT_GRID + TIGHT_NT;  // offset of the scaled Taylor coefficients

// e^-T is below 4.3e-18 * F0 for T >= 40; there the recursions drop it.
constexpr double BOYS_EXP_CUT = 40.0;

__device__ __forceinline__ double boysG(double T, double iT) {
  if (T < 15.0) return 0.4999489092 - 0.2473631686 * iT + 0.321180909 * iT * iT - 0.3811559346 * iT * iT * iT;
  if (T < 18.0) return 0.4998436875 - 0.24249438 * iT + 0.24642845 * iT * iT;
  if (T < 24.0) return 0.499093162 - 0.2152832 * iT;
  return 0.490;
}

template <int Q, int L>
__device__ __forceinline__ void boys_ref(double T, const double *__restrict__ tab, double (&F)[L + 1]) {
  static_assert(L <= Q && Q + 6 < FTAB_NM, "Boys order");
  if (T < 12.0) {
    const int tk = (int)(T * 10.0 + 0.5);  // NINT(T*10) for T >= 0
    const double d = __ldg(tab + BOYS_REF_GRID + tk) - T;
    const double *col = tab + tk;
    double f = __ldg(col + FTAB_NT * (Q + 6));
    f = __ldg(col + FTAB_NT * (Q + 5)) + f * (d * (1.0 / 6.0));
    f = __ldg(col + FTAB_NT * (Q + 4)) + f * (d * (1.0 / 5.0));
    f = __ldg(col + FTAB_NT * (Q + 3)) + f * (d * (1.0 / 4.0));
    f = __ldg(col + FTAB_NT * (Q + 2)) + f * (d * (1.0 / 3.0));
    f = __ldg(col + FTAB_NT * (Q + 1)) + f * (d * 0.5);
    f = __ldg(col + FTAB_NT * Q) + f * d;
    const double e = exp(-T), t2 = 2.0 * T;
    if (L == Q) F[L] = f;
#pragma unroll
    for (int j = Q - 1; j >= 0; --j) {
      f = (t2 * f + e) * (1.0 / (2 * j + 1));
      if (j <= L) F[j] = f;
    }
  } else {
    const double rT = rsqrt(T), iT = rT * rT, i2T = 0.5 * iT;
    const double c0 = 0.8862269377835134;  // 0.5*sqrt(3.1415927410125732), the reference's pi
    if (T < 2 * Q + 36) {
      const double e = T < BOYS_EXP_CUT ? exp(-T) : 0.0;
      F[0] = c0 * rT - e * boysG(T, iT) * iT;
#pragma unroll
      for (int j = 1; j <= L; ++j) F[j] = i2T * ((2 * j - 1) * F[j - 1] - e);
    } else {
      F[0] = c0 * rT;
#pragma unroll
      for (int j = 1; j <= L; ++j) F[j] = i2T * (2 * j - 1) * F[j - 1];
    }
  }
}

// F_m(T) = sum_k F_{m+k}(Tk) (Tk - T)^k / k! from the scaled coefficients
// (9 terms, |Tk - T| <= 0.05: remainder below 1e-17), one fma per term
template <int M>
__device__ __forceinline__ double boys_taylor(const double *__restrict__ tab, int tk, double d) {
  const double *c = tab + BOYS_TIGHT_SCALED + ((size_t)M * TIGHT_NT + tk) * 9;
  double f = __ldg(c + 8);
#pragma unroll
  for (int k = 7; k >= 0; --k) f = fma(f, d, __ldg(c + k));
  return f;
}

template <int L>
__device__ __forceinline__ void boys_tight(double T, const double *__restrict__ tab, double (&F)[L + 1]) {
  static_assert(L + 8 < TIGHT_NM && L < BOYS_SCALED_M, "Boys order");
  if (T < 36.0) {
    const int tk = __double2int_rn(T * 10.0);
    const double d = __ldg(tab + BOYS_TIGHT_GRID + tk) - T;
    if constexpr (L <= 2) {  // every order by its own series: no e^-T, no recursion
      F[0] = boys_taylor<0>(tab, tk, d);
      if constexpr (L >= 1) F[1] = boys_taylor<1>(tab, tk, d);
      if constexpr (L >= 2) F[2] = boys_taylor<2>(tab, tk, d);
    } else {  // the highest by its series, then downward recursion
      F[L] = boys_taylor<L>(tab, tk, d);
      const double e = exp(-T), t2 = 2.0 * T;
#pragma unroll
      for (int j = L - 1; j >= 0; --j) F[j] = (t2 * F[j + 1] + e) * (1.0 / (2 * j + 1));
    }
  } else {
    const double rT = rsqrt(T), i2T = 0.5 * rT * rT;
    F[0] = 0.8862269254527579 * rT;  // sqrt(pi)/2
#pragma unroll
    for (int j = 1; j <= L; ++j) F[j] = i2T * (2 * j - 1) * F[j - 1];
  }
}

template <int Q, int L>
__device__ __forceinline__ void boys(int mode, double T, const double *__restrict__ tab, double (&F)[L + 1]) {
  if (mode == MQ_MODE_REFERENCE) boys_ref<Q, L>(T, tab, F);
  else boys_tight<L>(T, tab, F);
}

}  // namespace mq
