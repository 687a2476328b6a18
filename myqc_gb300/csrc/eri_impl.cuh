// eri_impl.cuh -- the integral kernels' shared device code (included by eri.cu
// and eri_store.cu, which compile in parallel).
//   two-electron repulsion integrals over contracted s/sp shell
// quartets (McMurchie-Davidson), in FP64, or in FP32 for quartets whose
// Schwarz bound is below the context's threshold, with three epilogues:
//   EPI_XX      scatter each unique integral to its 8 places in the full
//               XX(i,j,g,h) array (replaces proc2e + fillsym,
//               src/integrals/int2e.f90:78-351,540-613);
//   EPI_SCHWARZ sqrt(max |(ab|ab)|) per shell pair (Schwarz bounds);
//   EPI_FOCK    digest each unique integral straight into J and K (direct SCF;
//               the reference digests the stored XX in RHFI2G/UHFI2G);
//   EPI_STORE   write each surviving quartet's integral block once, contiguous,
//               into the quartet store (qstore.cu), which the sparse Fock
//               digestion reads instead of the n^4 array.
//
// Integral formula (the reference's clmnew, int2e.f90:618-726):
//   (ab|cd) = sum_prim  2 pi^5/2 / (p q sqrt(p+q)) *
//             sum_{tuv} E^{ab}_{tuv} sum_{t'u'v'} (-1)^{t'+u'+v'} E^{cd}_{t'u'v'}
//             R_{t+t',u+u',v+v'}(alpha = pq/(p+q), PQ)
// with E the Hermite expansion coefficients (auxilary.f90:349-536), R the
// Hermite Coulomb integrals (RNLMj, auxilary.f90:22-80) built on the Boys
// values of boys.cuh, contraction coefficients times the primitive norms of
// gtoD (auxilary.f90:704-726), and the reference's primitive screen
// EIJ*EGH < 1e-14 (int2e.f90:257).
//
// Work decomposition: one thread per contracted shell quartet.  Shell pairs
// are kept in three classes (s,s), (sp,s), (sp,sp); a kernel instance serves
// one (bra class, ket class) combination, so every thread of a launch runs the
// same fully unrolled register code.  Quartets with more than 16 integrals
// ((sp sp|sp s): 64, (sp sp|sp sp): 256) are split over 4 or 16 threads by
// ket function c or ket pair (c, d), each thread forming the whole bra; the
// split index is constant per warp (warp w serves split w % nsplit for 32
// consecutive quartets), so no lane diverges.  The Schwarz launches split a
// diagonal quartet (P|P) the same way into one thread per diagonal integral
// (ab|ab).
#pragma once
#include <algorithm>
#include <type_traits>
#include <string>
#include <vector>

// the EPI_STORE epilogue returns before the element loop of the other epilogues
#pragma nv_diag_suppress 128
#include "boys.cuh"
#include "internal.h"

namespace mq {

enum { EPI_XX = 0, EPI_SCHWARZ = 1, EPI_FOCK = 2, EPI_STORE = 3 };

struct EriArgs {
  PairTable t;
  const double *boys;
  int mode;
  int n;
  int pOff, nP, qOff, nQ;
  int tri;       // bra and ket pairs from the same class: P >= Q
  int diag;      // Schwarz: quartet (P,P) only
  long long nq;  // quartets in this launch
  double thr;    // Schwarz threshold (0: off)
  double thr_hi; // > 0: only quartets whose bound is below it (the FP32 window of a mixed-precision pass)
  const float *boys_f;  // FP32 Boys table (tight layout) for the FP32 instances
  double *XX;
  unsigned long long *sch;  // Schwarz output (bit pattern of a positive double)
  const double *Da, *Db;
  double *J, *Ka, *Kb;
  int uhf;
  unsigned long long *counters;  // [0] quartets computed, [1] primitive quartets
  // batch (nmol > 0): the launch covers one class combination of every
  // molecule; mq_off is the prefix of the molecules' quartet counts, pstart /
  // pcount the molecules' pair ranges per class in the batch pair table
  int nmol, cP, cQ;
  const long long *mq_off;
  const int *pstart, *pcount;
  const MolDesc *mols;
  // Schwarz-compacted launch: the quartet indices that pass the screen, in
  // ascending order, *list_n of them (null: every index below nq, screened
  // inline); nq is then only the bound the grid is sized for
  const long long *list;
  const long long *list_n;
  // quartet store (EPI_STORE): the launch covers the staircase of one class
  // combination -- bra rank r holds the ket ranks s < len_r, quartet index
  // q in [st_off[r], st_off[r+1]) -- with ranks mapped to pairs by permP /
  // permQ; block q of the launch goes to store + q * (integrals per quartet)
  const long long *st_off;
  int st_n;
  const int *permP, *permQ;
  double *store;
  // persistent launch (queue non-null): the grid is sized to the resident
  // CTAs and each warp takes work units from *queue (zeroed first) while
  // they last; units = warp slots of the launch (quartets / 32 x split)
  unsigned long long *queue;
  long long units;
};

__host__ __device__ constexpr int fl(int f, int axis) { return f == axis + 1 ? 1 : 0; }  // f: 0 s, 1 px, 2 py, 3 pz
__host__ __device__ constexpr int fang(int f) { return f > 0 ? 1 : 0; }
__host__ __device__ constexpr int nfun(int L) { return L ? 4 : 1; }

// Is Hermite index (t,u,v) used by some bra pair (a,b) with a in [A0,A1), b in [B0,B1)?
__host__ __device__ constexpr bool bra_needs(int A0, int A1, int B0, int B1, int t, int u, int v) {
  for (int a = A0; a < A1; ++a)
    for (int b = B0; b < B1; ++b)
      if (t <= fl(a, 0) + fl(b, 0) && u <= fl(a, 1) + fl(b, 1) && v <= fl(a, 2) + fl(b, 2)) return true;
  return false;
}

// Hermite R_{tuv} (t+u+v <= L) from F_j already scaled by the prefactor.
template <int L, class RT>
__device__ __forceinline__ void hermite_R(const RT (&F)[L + 1], RT m2a, RT X, RT Y, RT Z,
                                          RT (&R)[L + 1][L + 1][L + 1]) {
  RT Rj[L + 1][L + 1][L + 1][L + 1];
  RT pw = RT(1);
#pragma unroll
  for (int j = 0; j <= L; ++j) {
    Rj[j][0][0][0] = pw * F[j];
    pw *= m2a;
  }
#pragma unroll
  for (int j = L - 1; j >= 0; --j) {
#pragma unroll
    for (int t = 0; t <= L; ++t)
#pragma unroll
      for (int u = 0; u <= L; ++u)
#pragma unroll
        for (int v = 0; v <= L; ++v) {
          if (t + u + v == 0 || t + u + v > L - j) continue;
          RT r;
          if (t > 0) {
            r = X * Rj[j + 1][t - 1][u][v];
            if (t > 1) r += RT(t - 1) * Rj[j + 1][t - 2][u][v];
          } else if (u > 0) {
            r = Y * Rj[j + 1][t][u - 1][v];
            if (u > 1) r += RT(u - 1) * Rj[j + 1][t][u - 2][v];
          } else {
            r = Z * Rj[j + 1][t][u][v - 1];
            if (v > 1) r += RT(v - 1) * Rj[j + 1][t][u][v - 2];
          }
          Rj[j][t][u][v] = r;
        }
  }
#pragma unroll
  for (int t = 0; t <= L; ++t)
#pragma unroll
    for (int u = 0; u <= L; ++u)
#pragma unroll
      for (int v = 0; v <= L; ++v)
        if (t + u + v <= L) R[t][u][v] = Rj[0][t][u][v];
}

// Per-axis Hermite coefficients of a primitive pair for l_a, l_b in {0,1}:
// e[la][lb][t], t <= la+lb (sign folded in for the ket when sgn = -1).
template <class RT>
__device__ __forceinline__ void pair_E(RT PA, RT PB, RT i2p, RT sgn, RT (&e)[2][2][3]) {
  e[0][0][0] = RT(1);
  e[1][0][0] = PA;
  e[1][0][1] = sgn * i2p;
  e[0][1][0] = PB;
  e[0][1][1] = sgn * i2p;
  e[1][1][0] = PA * PB + i2p;
  e[1][1][1] = sgn * (PA + PB) * i2p;
  e[1][1][2] = i2p * i2p;
}

// One primitive pair's data in the arithmetic type of the instance: FP64 from
// the pair table's arrays, FP32 from its packed copy (4 float4 per primitive
// pair: p 1/2p K Px | Py Pz PAx PAy | PAz PBx PBy PBz | c4).
template <class RT>
struct PrimPair {
  RT p, i2p, K, Px, Py, Pz, PAx, PAy, PAz, PBx, PBy, PBz, c[4];
};
__device__ __forceinline__ void load_pp(const PairTable &t, int ip, PrimPair<double> &d) {
  d.p = t.p[ip];
  d.i2p = t.inv2p[ip];
  d.K = t.K[ip];
  d.Px = t.Px[ip];
  d.Py = t.Py[ip];
  d.Pz = t.Pz[ip];
  d.PAx = t.PAx[ip];
  d.PAy = t.PAy[ip];
  d.PAz = t.PAz[ip];
  d.PBx = t.PBx[ip];
  d.PBy = t.PBy[ip];
  d.PBz = t.PBz[ip];
#pragma unroll
  for (int k = 0; k < 4; ++k) d.c[k] = t.c4[4 * ip + k];
}
__device__ __forceinline__ void load_pp(const PairTable &t, int ip, PrimPair<float> &d) {
  const float4 a = __ldg(t.pf + 4 * ip), b = __ldg(t.pf + 4 * ip + 1), c = __ldg(t.pf + 4 * ip + 2),
               e = __ldg(t.pf + 4 * ip + 3);
  d.p = a.x;
  d.i2p = a.y;
  d.K = a.z;
  d.Px = a.w;
  d.Py = b.x;
  d.Pz = b.y;
  d.PAx = b.z;
  d.PAy = b.w;
  d.PAz = c.x;
  d.PBx = c.y;
  d.PBy = c.z;
  d.PBz = c.w;
  d.c[0] = e.x;
  d.c[1] = e.y;
  d.c[2] = e.z;
  d.c[3] = e.w;
}
__device__ __forceinline__ double rsq(double x) { return rsqrt(x); }
__device__ __forceinline__ float rsq(float x) { return rsqrtf(x); }

// FP32 Boys values F_0..F_L from the tight table in single precision: 6-term
// Taylor of F_L about the nearest grid point (|d| <= 0.05: remainder below
// 1e-10 relative), downward recursion; above 36 the asymptotic F_0 and upward
// recursion.  Serves the FP32 instances, whose quartets are below a bound
// where single-precision relative errors stay far under the integral
// tolerance.
template <int L>
__device__ __forceinline__ void boys_f32(float T, const float *__restrict__ tab, float (&F)[L + 1]) {
  static_assert(L + 5 < TIGHT_NM, "Boys order");
  if (T < 36.0f) {
    const int tk = (int)(T * 10.0f + 0.5f);
    const float d = __ldg(tab + BOYS_TIGHT_GRID + tk) - T;
    const float *row = tab + tk * TIGHT_NM + L;
    float f = __ldg(row + 5);
    f = __ldg(row + 4) + f * (d * 0.2f);
    f = __ldg(row + 3) + f * (d * 0.25f);
    f = __ldg(row + 2) + f * (d * (1.0f / 3.0f));
    f = __ldg(row + 1) + f * (d * 0.5f);
    f = __ldg(row + 0) + f * d;
    F[L] = f;
    if (L > 0) {
      const float e = expf(-T), t2 = 2.0f * T;
#pragma unroll
      for (int j = L - 1; j >= 0; --j) F[j] = (t2 * F[j + 1] + e) * (1.0f / (2 * j + 1));
    }
  } else {
    const float rT = rsqrtf(T), i2T = 0.5f * rT * rT;
    F[0] = 0.886226925f * rT;  // sqrt(pi)/2
#pragma unroll
    for (int j = 1; j <= L; ++j) F[j] = i2T * float(2 * j - 1) * F[j - 1];
  }
}
template <int Q, int L>
__device__ __forceinline__ void boys_any(const EriArgs &g, double T, double (&F)[L + 1]) {
  boys<Q, L>(g.mode, T, g.boys, F);
}
template <int Q, int L>
__device__ __forceinline__ void boys_any(const EriArgs &g, float T, float (&F)[L + 1]) {
  boys_f32<L>(T, g.boys_f, F);
}

// One contracted quartet (P, Q), the bra functions a in [A0, A1), b in [B0, B1)
// and ket functions c in [C0, C1), d in [D0, D1) of it (a thread's share when a
// quartet is split over threads).  With the whole bra in one thread (ONFLY)
// the bra Hermite products are formed on the fly from the per-axis
// coefficients instead of being kept for every (a, b): a ket-split thread then
// forms each ket contraction W once and applies it to all 16 bra functions.
template <int LA, int LB, int LC, int LD, int A0, int A1, int B0, int B1, int C0, int C1, int D0, int D1, int EPI,
          class RT = double>
__device__ __forceinline__ void quartet(const EriArgs &g, int P, int Q, size_t n, double *XXout) {
  constexpr int LAB = LA + LB, LT = LA + LB + LC + LD;
  constexpr int QREF = 3 * LT;  // the reference's Boys order for s/sp sets
  constexpr bool ONFLY = (A1 - A0) * (B1 - B0) > 4;
  const PairTable &t = g.t;
  RT acc[A1 - A0][B1 - B0][C1 - C0][D1 - D0];
#pragma unroll
  for (int a = 0; a < A1 - A0; ++a)
#pragma unroll
    for (int b = 0; b < B1 - B0; ++b)
#pragma unroll
      for (int c = 0; c < C1 - C0; ++c)
#pragma unroll
        for (int d = 0; d < D1 - D0; ++d) acc[a][b][c][d] = RT(0);

  const int p0 = t.pp_off[P], p1 = t.pp_off[P + 1];
  const int q0 = t.pp_off[Q], q1 = t.pp_off[Q + 1];
  const bool parity = g.mode == MQ_MODE_REFERENCE;
  const RT pref0 = parity ? RT(2.0 * 17.493419544621675) : RT(2.0 * 17.493418327624862);  // 2 pi^2.5
  unsigned nprim = 0;
  // The surviving primitive quartets only, in one flat loop.  The primitive
  // pairs of a shell pair are ordered by K descending, so the ket primitives
  // that pass the reference's screen Kab*Kcd >= 1e-14 (int2e.f90:257) against
  // one bra primitive are a prefix of the ket list, and the bra primitives
  // with any partner a prefix of the bra list: the loop moves to the next bra
  // primitive at the first failing ket, and stops at the first bra primitive
  // without a partner.  A warp's trip count is the largest survivor count of
  // its lanes (which the binned launch order makes nearly equal).  The
  // Schwarz bounds take every primitive quartet: they must bound the exact
  // (ab|ab), and the screen can remove every primitive quartet of (ab|ab) for
  // a distant pair while (ab|cd) with a compact partner survives it.
  const RT screen = EPI == EPI_SCHWARZ ? RT(0) : RT(1.0e-14);
  RT p = RT(0), i2p = RT(0), Kab = RT(0), Px = RT(0), Py = RT(0), Pz = RT(0);
  RT ex[2][2][3], ey[2][2][3], ez[2][2][3];
  RT cab[4];
  // bra products E^{ab}_{tuv} * c_a c_b K_ab (kept per (a, b) unless ONFLY)
  RT eb[ONFLY ? 1 : A1 - A0][ONFLY ? 1 : B1 - B0][3][3][3];
  int ip = p0 - 1, iq = q1;
  for (;;) {
    PrimPair<RT> cd;
    bool next_bra = iq >= q1;
    if (!next_bra) {
      load_pp(t, iq, cd);
      next_bra = Kab * cd.K < screen;
    }
    if (next_bra) {
      if (++ip >= p1 || q0 >= q1) break;
      PrimPair<RT> ab;
      load_pp(t, ip, ab);
      load_pp(t, q0, cd);
      if (ab.K * cd.K < screen) break;  // nor any later bra primitive
      p = ab.p;
      i2p = ab.i2p;
      Kab = ab.K;
      Px = ab.Px;
      Py = ab.Py;
      Pz = ab.Pz;
      pair_E(ab.PAx, ab.PBx, i2p, RT(1), ex);
      pair_E(ab.PAy, ab.PBy, i2p, RT(1), ey);
      pair_E(ab.PAz, ab.PBz, i2p, RT(1), ez);
#pragma unroll
      for (int k = 0; k < 4; ++k) cab[k] = ab.c[k];
      if (!ONFLY) {
#pragma unroll
        for (int a = A0; a < A1; ++a)
#pragma unroll
          for (int b = B0; b < B1; ++b)
#pragma unroll
            for (int x = 0; x <= fl(a, 0) + fl(b, 0); ++x)
#pragma unroll
              for (int y = 0; y <= fl(a, 1) + fl(b, 1); ++y)
#pragma unroll
                for (int z = 0; z <= fl(a, 2) + fl(b, 2); ++z)
                  eb[ONFLY ? 0 : a - A0][ONFLY ? 0 : b - B0][x][y][z] = ex[fl(a, 0)][fl(b, 0)][x] *
                                                                       ey[fl(a, 1)][fl(b, 1)][y] *
                                                                       ez[fl(a, 2)][fl(b, 2)][z] *
                                                                       cab[2 * fang(a) + fang(b)];
      }
      iq = q0;
    }
    ++iq;
    ++nprim;
    {
      const RT q = cd.p, i2q = cd.i2p;
      const RT X = Px - cd.Px, Y = Py - cd.Py, Z = Pz - cd.Pz;
      const RT s = p + q;
      const RT rs = rsq(s);
      const RT ipq = RT(4) * i2p * i2q;  // 1/(pq)
      const RT alpha = (p * q) * (rs * rs);
      const RT T = alpha * (X * X + Y * Y + Z * Z);
      const RT pref = pref0 * rs * ipq;
      RT F[LT + 1];
      boys_any<QREF, LT>(g, T, F);
#pragma unroll
      for (int j = 0; j <= LT; ++j) F[j] *= pref;
      RT R[LT + 1][LT + 1][LT + 1];
      hermite_R<LT>(F, RT(-2) * alpha, X, Y, Z, R);
      RT fx[2][2][3], fy[2][2][3], fz[2][2][3];
      pair_E(cd.PAx, cd.PBx, i2q, RT(-1), fx);
      pair_E(cd.PAy, cd.PBy, i2q, RT(-1), fy);
      pair_E(cd.PAz, cd.PBz, i2q, RT(-1), fz);
      RT ccd[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) ccd[k] = cd.c[k];
#pragma unroll
      for (int c = C0; c < C1; ++c)
#pragma unroll
        for (int d = D0; d < D1; ++d) {
          const RT cf = ccd[2 * fang(c) + fang(d)];
          RT W[LAB + 1][LAB + 1][LAB + 1];
#pragma unroll
          for (int x = 0; x <= LAB; ++x)
#pragma unroll
            for (int y = 0; y <= LAB; ++y)
#pragma unroll
              for (int z = 0; z <= LAB; ++z) {
                if (x + y + z > LAB || !bra_needs(A0, A1, B0, B1, x, y, z)) continue;
                RT w = RT(0);
#pragma unroll
                for (int xx = 0; xx <= fl(c, 0) + fl(d, 0); ++xx)
#pragma unroll
                  for (int yy = 0; yy <= fl(c, 1) + fl(d, 1); ++yy)
#pragma unroll
                    for (int zz = 0; zz <= fl(c, 2) + fl(d, 2); ++zz)
                      w += (fx[fl(c, 0)][fl(d, 0)][xx] * fy[fl(c, 1)][fl(d, 1)][yy] * fz[fl(c, 2)][fl(d, 2)][zz]) *
                           R[x + xx][y + yy][z + zz];
                W[x][y][z] = w * cf;
              }
#pragma unroll
          for (int a = A0; a < A1; ++a)
#pragma unroll
            for (int b = B0; b < B1; ++b) {
              RT v = RT(0);
#pragma unroll
              for (int x = 0; x <= fl(a, 0) + fl(b, 0); ++x)
#pragma unroll
                for (int y = 0; y <= fl(a, 1) + fl(b, 1); ++y)
#pragma unroll
                  for (int z = 0; z <= fl(a, 2) + fl(b, 2); ++z) {
                    const RT e = ONFLY ? ex[fl(a, 0)][fl(b, 0)][x] * ey[fl(a, 1)][fl(b, 1)][y] *
                                             ez[fl(a, 2)][fl(b, 2)][z]
                                       : eb[ONFLY ? 0 : a - A0][ONFLY ? 0 : b - B0][x][y][z];
                    v += e * W[x][y][z];
                  }
              acc[a - A0][b - B0][c - C0][d - D0] += ONFLY ? v * cab[2 * fang(a) + fang(b)] : v;
            }
        }
    }
  }
  // ---------------- epilogues ----------------
  const int A = t.shA[P], B = t.shB[P], C = t.shA[Q], D = t.shB[Q];
  const int i0 = t.aoA[P], j0 = t.aoB[P], k0 = t.aoA[Q], l0 = t.aoB[Q];
  if (EPI == EPI_SCHWARZ) {
    double m = 0.0;
#pragma unroll
    for (int a = A0; a < A1; ++a)
#pragma unroll
      for (int b = B0; b < B1; ++b)
        if (a >= C0 && a < C1 && b >= D0 && b < D1) m = fmax(m, fabs((double)acc[a - A0][b - B0][a - C0][b - D0]));
    atomicMax(g.sch + P, (unsigned long long)__double_as_longlong(sqrt(m)));
    return;
  }
  if (g.counters && A0 == 0 && B0 == 0 && C0 == 0 && D0 == 0) {  // one atomic pair per warp, not per quartet
    const unsigned act = __activemask();
    const unsigned nq_w = __popc(act), np_w = __reduce_add_sync(act, nprim);
    if ((threadIdx.x & 31) == __ffs(act) - 1) {
      atomicAdd(g.counters, (unsigned long long)nq_w);
      atomicAdd(g.counters + 1, (unsigned long long)np_w);
    }
  }
  if constexpr (EPI == EPI_STORE) {  // the whole block (this thread's share), layout ((a NB + b) NC + c) ND + d
    constexpr int NB_ = nfun(LB), NC_ = nfun(LC), ND_ = nfun(LD);
#pragma unroll
    for (int a = A0; a < A1; ++a)
#pragma unroll
      for (int b = B0; b < B1; ++b)
#pragma unroll
        for (int c = C0; c < C1; ++c)
#pragma unroll
          for (int d = D0; d < D1; ++d)
            XXout[((a * NB_ + b) * NC_ + c) * ND_ + d] = (double)acc[a - A0][b - B0][c - C0][d - D0];
    return;
  }
#pragma unroll
  for (int a = A0; a < A1; ++a)
#pragma unroll
    for (int b = B0; b < B1; ++b)
#pragma unroll
      for (int c = C0; c < C1; ++c)
#pragma unroll
        for (int d = D0; d < D1; ++d) {
          const int i = i0 + a, j = j0 + b, k = k0 + c, l = l0 + d;
          if (A == B && i < j) continue;
          if (C == D && k < l) continue;
          if (P == Q && (size_t)i * n + j < (size_t)k * n + l) continue;
          const double x = (double)acc[a - A0][b - B0][c - C0][d - D0];
          if (EPI == EPI_XX) {
            double *XX = XXout;
            const size_t ij = (size_t)i + n * j, ji = (size_t)j + n * i, kl = (size_t)k + n * l,
                         lk = (size_t)l + n * k, n2 = n * n;
            XX[ij + n2 * kl] = x;
            XX[ji + n2 * kl] = x;
            XX[ij + n2 * lk] = x;
            XX[ji + n2 * lk] = x;
            XX[kl + n2 * ij] = x;
            XX[lk + n2 * ij] = x;
            XX[kl + n2 * ji] = x;
            XX[lk + n2 * ji] = x;
          } else {  // EPI_FOCK: half-sums, symmetrised afterwards
            double deg = 1.0;
            if (i == j) deg *= 0.5;
            if (k == l) deg *= 0.5;
            if (i == k && j == l) deg *= 0.5;
            const double x2 = 2.0 * deg * x, x4 = 2.0 * x2;
            const double *Da = g.Da;
            if (!g.uhf) {
              atomicAdd(g.J + i + n * j, x4 * Da[k + n * l]);
              atomicAdd(g.J + k + n * l, x4 * Da[i + n * j]);
              atomicAdd(g.Ka + i + n * k, x2 * Da[j + n * l]);
              atomicAdd(g.Ka + j + n * k, x2 * Da[i + n * l]);
              atomicAdd(g.Ka + i + n * l, x2 * Da[j + n * k]);
              atomicAdd(g.Ka + j + n * l, x2 * Da[i + n * k]);
            } else {
              const double *Db = g.Db;
              atomicAdd(g.J + i + n * j, x4 * (Da[k + n * l] + Db[k + n * l]));
              atomicAdd(g.J + k + n * l, x4 * (Da[i + n * j] + Db[i + n * j]));
              atomicAdd(g.Ka + i + n * k, x2 * Da[j + n * l]);
              atomicAdd(g.Ka + j + n * k, x2 * Da[i + n * l]);
              atomicAdd(g.Ka + i + n * l, x2 * Da[j + n * k]);
              atomicAdd(g.Ka + j + n * l, x2 * Da[i + n * k]);
              atomicAdd(g.Kb + i + n * k, x2 * Db[j + n * l]);
              atomicAdd(g.Kb + j + n * k, x2 * Db[i + n * l]);
              atomicAdd(g.Kb + i + n * l, x2 * Db[j + n * k]);
              atomicAdd(g.Kb + j + n * l, x2 * Db[i + n * k]);
            }
          }
        }
}

// decode (P, Q) of the launch's q-th quartet, and the molecule m (0 for one
// system); returns false past the end.  With a list (Schwarz-compacted or
// binned launch order) q is first replaced by its list entry, the quartet's
// index in the launch's own numbering (the quartet store's block index).
__device__ __forceinline__ bool decode(const EriArgs &g, long long &q, int &P, int &Q, int &m) {
  if (q >= g.nq) return false;
  const bool listed = g.list != nullptr;
  if (listed) {
    if (q >= *g.list_n) return false;
    q = g.list[q];
  }
  if (g.st_off) {  // largest r with st_off[r] <= q
    int lo = 0, hi = g.st_n - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (g.st_off[mid] <= q) lo = mid;
      else hi = mid - 1;
    }
    m = 0;
    P = g.permP[lo];
    Q = g.permQ[(int)(q - g.st_off[lo])];
    return true;
  }
  m = 0;
  int pOff = g.pOff, qOff = g.qOff, nQ = g.nQ;
  if (g.nmol) {  // largest m with mq_off[m] <= q
    int lo = 0, hi = g.nmol - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (g.mq_off[mid] <= q) lo = mid;
      else hi = mid - 1;
    }
    m = lo;
    q -= g.mq_off[m];
    pOff = g.pstart[3 * m + g.cP];
    qOff = g.pstart[3 * m + g.cQ];
    nQ = g.pcount[3 * m + g.cQ];
  }
  if (g.diag) {
    P = Q = pOff + (int)q;
    return true;
  }
  if (g.tri) {
    long long r = (long long)((sqrt(8.0 * (double)q + 1.0) - 1.0) * 0.5);
    while (r * (r + 1) / 2 > q) --r;
    while ((r + 1) * (r + 2) / 2 <= q) ++r;
    P = pOff + (int)r;
    Q = qOff + (int)(q - r * (r + 1) / 2);
  } else {
    P = pOff + (int)(q / nQ);
    Q = qOff + (int)(q % nQ);
  }
  if (!listed && g.thr > 0.0) {
    const double b = g.t.schwarz[P] * g.t.schwarz[Q];
    if (b < g.thr || (g.thr_hi > 0.0 && b >= g.thr_hi)) return false;
  }
  return true;
}

// Flattened index of the Hermite integral R_{tuv}, t + u + v <= L.
__host__ __device__ constexpr int ridx(int L, int t, int u, int v) {
  int k = 0;
  for (int a = 0; a < t; ++a) k += (L - a + 1) * (L - a + 2) / 2;
  for (int b = 0; b < u; ++b) k += L - t - b + 1;
  return k + v;
}
__host__ __device__ constexpr int nherm(int L) { return (L + 1) * (L + 2) * (L + 3) / 6; }

// The next surviving primitive quartet after (ip, iq) of a quartet whose
// primitive pairs are ordered by K descending (see quartet()): the next ket
// while it passes the screen against the bra, else the first ket of the next
// bra.  Returns false when none is left (ip is then p1).
__device__ __forceinline__ bool next_survivor(const PairTable &t, int p1, int q0, int q1, int &ip, int &iq,
                                              double &Kab) {
  if (++iq < q1 && Kab * t.K[iq] >= 1.0e-14) return true;
  if (++ip >= p1) return false;
  Kab = t.K[ip];
  iq = q0;
  if (Kab * t.K[q0] >= 1.0e-14) return true;
  ip = p1;
  return false;
}

// Quartet-store pass of the split classes ((sp sp|sp s): 4 warps, one ket
// function c each; (sp sp|sp sp): 16 warps, one ket pair (c, d) each), with
// the per-primitive-quartet work shared.  The CTA's warps serve the same 32
// quartets (lane = quartet), so every one of them needs the same Boys values
// and Hermite integrals R_tuv of each primitive quartet.  A lane's surviving
// primitive quartets are numbered k = 0 .. S-1 (bra outer, ket inner, the
// survivors of the K-ordered lists as quartet() visits them); in round r warp
// w forms the prefactor, Boys values and R recursion of survivor
// r * NSPLIT + w of its lane's quartet -- once instead of once per warp --
// and leaves R and the survivor's (bra, ket) primitive pair in shared memory;
// after a barrier every warp contracts all the round's survivors into its own
// outputs.  The round count is the warp's largest S (every warp of the CTA
// computes the same S per lane), so the barriers are reached by every thread,
// and a round has idle producers only at the end of a lane's list.
template <int LA, int LB, int LC, int LD, int NSPLIT, int C0, int C1, int D0, int D1>
__device__ __forceinline__ void quartet_store_shared(const EriArgs &g, bool valid, int P, int Q, double *XXout,
                                                     double *smR, int2 *smI) {
  constexpr int LAB = LA + LB, LT = LA + LB + LC + LD, NR = nherm(LT);
  constexpr int QREF = 3 * LT;
  constexpr int NA = nfun(LA), NB = nfun(LB), NC = nfun(LC), ND = nfun(LD);
  const PairTable &t = g.t;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  double acc[NA][NB][C1 - C0][D1 - D0];
#pragma unroll
  for (int a = 0; a < NA; ++a)
#pragma unroll
    for (int b = 0; b < NB; ++b)
#pragma unroll
      for (int c = 0; c < C1 - C0; ++c)
#pragma unroll
        for (int d = 0; d < D1 - D0; ++d) acc[a][b][c][d] = 0.0;
  const int p0 = valid ? t.pp_off[P] : 0, p1 = valid ? t.pp_off[P + 1] : 0;
  const int q0 = valid ? t.pp_off[Q] : 0, q1 = valid ? t.pp_off[Q + 1] : 0;
  // S: the survivors of this lane's quartet (the prefix lengths of the bra
  // primitives, each no longer than the previous)
  int S = 0;
  {
    int m = q1 - q0;
    for (int i = p0; i < p1 && m > 0; ++i) {
      const double Ki = t.K[i];
      while (m > 0 && Ki * t.K[q0 + m - 1] < 1.0e-14) --m;
      S += m;
    }
  }
  const int rounds = (__reduce_max_sync(0xffffffffu, S) + NSPLIT - 1) / NSPLIT;
  // this warp's producer position: survivor w, then NSPLIT further each round
  int ip = p0, iq = q0 - 1;
  double Kab = valid && p0 < p1 ? t.K[p0] : 0.0;
  bool live = S > 0;
  for (int k = 0; k <= w && live; ++k) live = next_survivor(t, p1, q0, q1, ip, iq, Kab);
  const bool parity = g.mode == MQ_MODE_REFERENCE;
  const double pref0 = parity ? 2.0 * 17.493419544621675 : 2.0 * 17.493418327624862;  // 2 pi^2.5
  unsigned nprim = 0;
  int cur_ip = -1;  // the bra primitive whose expansion the consumer holds
  double ex[2][2][3], ey[2][2][3], ez[2][2][3], cab[4];
  for (int r = 0; r < rounds; ++r) {
    // producer: survivor r * NSPLIT + w of this lane's quartet
    {
      int2 id = make_int2(-1, -1);
      if (live) {
        PrimPair<double> ab, cd;
        load_pp(t, ip, ab);
        load_pp(t, iq, cd);
        id = make_int2(ip, iq);
        ++nprim;
        const double q = cd.p, X = ab.Px - cd.Px, Y = ab.Py - cd.Py, Z = ab.Pz - cd.Pz;
        const double sum = ab.p + q, rs = rsqrt(sum);
        const double ipq = 4.0 * ab.i2p * cd.i2p;
        const double alpha = (ab.p * q) * (rs * rs);
        const double T = alpha * (X * X + Y * Y + Z * Z);
        const double pref = pref0 * rs * ipq;
        double F[LT + 1];
        boys<QREF, LT>(g.mode, T, g.boys, F);
#pragma unroll
        for (int j = 0; j <= LT; ++j) F[j] *= pref;
        double R[LT + 1][LT + 1][LT + 1];
        hermite_R<LT>(F, -2.0 * alpha, X, Y, Z, R);
        double *dst = smR + (size_t)(w * 32 + lane) * NR;
#pragma unroll
        for (int x = 0; x <= LT; ++x)
#pragma unroll
          for (int y = 0; y <= LT; ++y)
#pragma unroll
            for (int z = 0; z <= LT; ++z)
              if (x + y + z <= LT) dst[ridx(LT, x, y, z)] = R[x][y][z];
        for (int k = 0; k < NSPLIT && live; ++k) live = next_survivor(t, p1, q0, q1, ip, iq, Kab);
      }
      smI[w * 32 + lane] = id;
    }
    __syncthreads();
    // consumers: every survivor of the round into this warp's outputs
    for (int j = 0; j < NSPLIT; ++j) {
      const int2 id = smI[j * 32 + lane];
      if (id.x < 0) continue;
      if (id.x != cur_ip) {
        PrimPair<double> ab;
        load_pp(t, id.x, ab);
        pair_E(ab.PAx, ab.PBx, ab.i2p, 1.0, ex);
        pair_E(ab.PAy, ab.PBy, ab.i2p, 1.0, ey);
        pair_E(ab.PAz, ab.PBz, ab.i2p, 1.0, ez);
#pragma unroll
        for (int k = 0; k < 4; ++k) cab[k] = ab.c[k];
        cur_ip = id.x;
      }
      const double *Rs = smR + (size_t)(j * 32 + lane) * NR;
      PrimPair<double> cd;
      load_pp(t, id.y, cd);
      double fx[2][2][3], fy[2][2][3], fz[2][2][3];
      pair_E(cd.PAx, cd.PBx, cd.i2p, -1.0, fx);
      pair_E(cd.PAy, cd.PBy, cd.i2p, -1.0, fy);
      pair_E(cd.PAz, cd.PBz, cd.i2p, -1.0, fz);
#pragma unroll
      for (int c = C0; c < C1; ++c)
#pragma unroll
        for (int d = D0; d < D1; ++d) {
          const double cf = cd.c[2 * fang(c) + fang(d)];
          double W[LAB + 1][LAB + 1][LAB + 1];
#pragma unroll
          for (int x = 0; x <= LAB; ++x)
#pragma unroll
            for (int y = 0; y <= LAB; ++y)
#pragma unroll
              for (int z = 0; z <= LAB; ++z) {
                if (x + y + z > LAB) continue;
                double wv = 0.0;
#pragma unroll
                for (int xx = 0; xx <= fl(c, 0) + fl(d, 0); ++xx)
#pragma unroll
                  for (int yy = 0; yy <= fl(c, 1) + fl(d, 1); ++yy)
#pragma unroll
                    for (int zz = 0; zz <= fl(c, 2) + fl(d, 2); ++zz)
                      wv += (fx[fl(c, 0)][fl(d, 0)][xx] * fy[fl(c, 1)][fl(d, 1)][yy] * fz[fl(c, 2)][fl(d, 2)][zz]) *
                            Rs[ridx(LT, x + xx, y + yy, z + zz)];
                W[x][y][z] = wv * cf;
              }
#pragma unroll
          for (int a = 0; a < NA; ++a)
#pragma unroll
            for (int b = 0; b < NB; ++b) {
              double v = 0.0;
#pragma unroll
              for (int x = 0; x <= fl(a, 0) + fl(b, 0); ++x)
#pragma unroll
                for (int y = 0; y <= fl(a, 1) + fl(b, 1); ++y)
#pragma unroll
                  for (int z = 0; z <= fl(a, 2) + fl(b, 2); ++z)
                    v += ex[fl(a, 0)][fl(b, 0)][x] * ey[fl(a, 1)][fl(b, 1)][y] * ez[fl(a, 2)][fl(b, 2)][z] *
                         W[x][y][z];
              acc[a][b][c - C0][d - D0] += v * cab[2 * fang(a) + fang(b)];
            }
        }
    }
    __syncthreads();
  }
  if (g.counters) {  // quartets by warp 0, the primitive quartets each warp formed
    const unsigned np_w = __reduce_add_sync(0xffffffffu, nprim);
    const unsigned nq_w = __popc(__ballot_sync(0xffffffffu, valid));
    if (lane == 0) {
      if (w == 0) atomicAdd(g.counters, (unsigned long long)nq_w);
      atomicAdd(g.counters + 1, (unsigned long long)np_w);
    }
  }
  if (!valid) return;
#pragma unroll
  for (int a = 0; a < NA; ++a)
#pragma unroll
    for (int b = 0; b < NB; ++b)
#pragma unroll
      for (int c = C0; c < C1; ++c)
#pragma unroll
        for (int d = D0; d < D1; ++d) XXout[((a * NB + b) * NC + c) * ND + d] = acc[a][b][c - C0][d - D0];
}

// Store pass of a split class: one CTA of NSPLIT warps per 32 quartets.
template <int LA, int LB, int LC, int LD>
__global__ void __launch_bounds__(512) eri_store_shared_kernel(EriArgs g) {
  constexpr int NOUT = nfun(LA) * nfun(LB) * nfun(LC) * nfun(LD);
  constexpr int NSPLIT = NOUT <= 64 ? 4 : 16;
  constexpr int NR = nherm(LA + LB + LC + LD);
  extern __shared__ double sm_shared[];  // R of the round's survivors [NSPLIT][32][NR], then their (bra, ket) pairs
  double *smR = sm_shared;
  int2 *smI = reinterpret_cast<int2 *>(sm_shared + NSPLIT * 32 * NR);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  long long q = (long long)blockIdx.x * 32 + lane;
  int P = 0, Q = 0, m = 0;
  const bool valid = decode(g, q, P, Q, m);
  double *out = valid ? g.store + q * NOUT : nullptr;
  if constexpr (NSPLIT == 4) {
    switch (w) {
      case 0: quartet_store_shared<LA, LB, LC, LD, 4, 0, 1, 0, 1>(g, valid, P, Q, out, smR, smI); break;
      case 1: quartet_store_shared<LA, LB, LC, LD, 4, 1, 2, 0, 1>(g, valid, P, Q, out, smR, smI); break;
      case 2: quartet_store_shared<LA, LB, LC, LD, 4, 2, 3, 0, 1>(g, valid, P, Q, out, smR, smI); break;
      default: quartet_store_shared<LA, LB, LC, LD, 4, 3, 4, 0, 1>(g, valid, P, Q, out, smR, smI); break;
    }
  } else {
#define MQ_SH16(s)                                                                                             \
  case s:                                                                                                      \
    quartet_store_shared<LA, LB, LC, LD, 16, (s) / 4, (s) / 4 + 1, (s) % 4, (s) % 4 + 1>(g, valid, P, Q, out, smR, \
                                                                                       smI);                   \
    break;
    switch (w) {
      MQ_SH16(0) MQ_SH16(1) MQ_SH16(2) MQ_SH16(3) MQ_SH16(4) MQ_SH16(5) MQ_SH16(6) MQ_SH16(7) MQ_SH16(8)
      MQ_SH16(9) MQ_SH16(10) MQ_SH16(11) MQ_SH16(12) MQ_SH16(13) MQ_SH16(14)
      default: quartet_store_shared<LA, LB, LC, LD, 16, 3, 4, 3, 4>(g, valid, P, Q, out, smR, smI); break;
    }
#undef MQ_SH16
  }
}

// Schwarz bounds need only the diagonal integrals (ab|ab) of a shell pair: one
// thread per pair and diagonal function pair S = (a, b), a single integral each
template <int LA, int LB, int S>
__device__ __forceinline__ void schwarz_diag(const EriArgs &g, int P, size_t n, double *XX) {
  constexpr int NB = nfun(LB), a = S / NB, b = S % NB;
  if constexpr (a < nfun(LA))
    quartet<LA, LB, LA, LB, a, a + 1, b, b + 1, a, a + 1, b, b + 1, EPI_SCHWARZ, double>(g, P, P, n, XX);
}

template <int LA, int LB, int LC, int LD, int EPI, class RT>
__device__ __forceinline__ void eri_unit(const EriArgs &g, long long warp, int lane);

template <int LA, int LB, int LC, int LD, int EPI, class RT = double>
__global__ void __launch_bounds__(256) eri_kernel(EriArgs g) {
  constexpr int NA = nfun(LA), NB = nfun(LB);
  constexpr int NOUT = NA * NB * nfun(LC) * nfun(LD);
  if constexpr (EPI == EPI_SCHWARZ) {  // diagonal classes only (LC = LA, LD = LB)
    constexpr int NDIAG = NA * NB;
    const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int split = (int)(warp % NDIAG);
    long long q = (warp / NDIAG) * 32 + (threadIdx.x & 31);
    int P, Q, m;
    if (!decode(g, q, P, Q, m)) return;
    const size_t n = (size_t)g.n;
    switch (split) {
#define MQ_DIAG(s) \
  case s: schwarz_diag<LA, LB, s>(g, P, n, g.XX); break;
      MQ_DIAG(0) MQ_DIAG(1) MQ_DIAG(2) MQ_DIAG(3) MQ_DIAG(4) MQ_DIAG(5) MQ_DIAG(6) MQ_DIAG(7)
      MQ_DIAG(8) MQ_DIAG(9) MQ_DIAG(10) MQ_DIAG(11) MQ_DIAG(12) MQ_DIAG(13) MQ_DIAG(14)
      default: schwarz_diag<LA, LB, 15>(g, P, n, g.XX); break;
#undef MQ_DIAG
    }
    return;
  }
  constexpr int NSPLIT = NOUT <= 16 ? 1 : (NOUT <= 64 ? 4 : 16);
  const int lane = threadIdx.x & 31;
  if (g.queue) {  // persistent: each warp takes work units from the launch's queue until it is empty
    for (;;) {
      unsigned long long unit = 0;
      if (lane == 0) unit = atomicAdd(g.queue, 1ull);
      unit = __shfl_sync(0xffffffffu, unit, 0);
      if (unit >= (unsigned long long)g.units) break;
      eri_unit<LA, LB, LC, LD, EPI, RT>(g, (long long)unit, lane);
    }
    return;
  }
  eri_unit<LA, LB, LC, LD, EPI, RT>(g, ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane);
}

// One work unit of an integral launch: warp unit w serves split w % NSPLIT of
// the 32 consecutive quartets (w / NSPLIT) * 32 .. + 31 of the launch order.
template <int LA, int LB, int LC, int LD, int EPI, class RT>
__device__ __forceinline__ void eri_unit(const EriArgs &g, long long warp, int lane) {
  constexpr int NA = nfun(LA), NB = nfun(LB);
  constexpr int NOUT = NA * NB * nfun(LC) * nfun(LD);
  constexpr int NSPLIT = NOUT <= 16 ? 1 : (NOUT <= 64 ? 4 : 16);
  const int split = (int)(warp % NSPLIT);
  long long q = (warp / NSPLIT) * 32 + lane;
  int P, Q, m;
  if (!decode(g, q, P, Q, m)) return;
  size_t n = (size_t)g.n;
  double *XX = g.XX;
  if (g.nmol) {
    n = (size_t)g.mols[m].n;
    XX += g.mols[m].xx;
  }
  if constexpr (EPI == EPI_STORE) XX = g.store + q * NOUT;
  constexpr int NC = nfun(LC), ND = nfun(LD);
  if (NSPLIT == 1) {
    quartet<LA, LB, LC, LD, 0, NA, 0, NB, 0, NC, 0, ND, EPI, RT>(g, P, Q, n, XX);
  } else if (NSPLIT == 4) {  // (sp sp|sp s): one ket function c per thread, the whole bra
    switch (split) {
      case 0: quartet<LA, LB, LC, LD, 0, NA, 0, NB, 0, 1, 0, ND, EPI, RT>(g, P, Q, n, XX); break;
      case 1: quartet<LA, LB, LC, LD, 0, NA, 0, NB, 1, 2, 0, ND, EPI, RT>(g, P, Q, n, XX); break;
      case 2: quartet<LA, LB, LC, LD, 0, NA, 0, NB, 2, 3, 0, ND, EPI, RT>(g, P, Q, n, XX); break;
      default: quartet<LA, LB, LC, LD, 0, NA, 0, NB, 3, 4, 0, ND, EPI, RT>(g, P, Q, n, XX); break;
    }
  } else {  // (sp sp|sp sp): one ket pair (c, d) per thread, the whole bra
#define MQ_SPLIT16(s) \
  case s: quartet<LA, LB, LC, LD, 0, NA, 0, NB, (s) / 4, (s) / 4 + 1, (s) % 4, (s) % 4 + 1, EPI, RT>(g, P, Q, n, XX); break;
    switch (split) {
      MQ_SPLIT16(0) MQ_SPLIT16(1) MQ_SPLIT16(2) MQ_SPLIT16(3) MQ_SPLIT16(4) MQ_SPLIT16(5) MQ_SPLIT16(6)
      MQ_SPLIT16(7) MQ_SPLIT16(8) MQ_SPLIT16(9) MQ_SPLIT16(10) MQ_SPLIT16(11) MQ_SPLIT16(12) MQ_SPLIT16(13)
      MQ_SPLIT16(14) default: quartet<LA, LB, LC, LD, 0, NA, 0, NB, 3, 4, 3, 4, EPI, RT>(g, P, Q, n, XX); break;
    }
#undef MQ_SPLIT16
  }
}

static inline int nsplit_of(int cP, int cQ) {
  int nout = (cP == 0 ? 1 : cP == 1 ? 4 : 16) * (cQ == 0 ? 1 : cQ == 1 ? 4 : 16);
  return nout <= 16 ? 1 : (nout <= 64 ? 4 : 16);
}

// The launch order of an integral launch sorted by surviving primitive
// quartets (eri_store.cu): h.list / h.list_n are set.
int bin_quartets(mq_ctx *c, EriArgs &h, int slot);
// the batch's integral launch of one class combination, in its autotuned shape (eri_store.cu)
int eri_batch_launch(mq_ctx *c, const EriArgs &h, int cP, int cQ);

// One class combination's integral launch; `block` is the CTA size of the
// thread-per-quartet kernel (64, 128 or 256; the autotuner's choice)
template <int EPI, class RT = double>
static int launch_class(mq_ctx *c, EriArgs g, int cP, int cQ, int block = 128, bool persistent = false) {
  // Schwarz: one warp slot per diagonal function pair (ab|ab) of the class
  const int nsplit = EPI == EPI_SCHWARZ ? (cP == 0 ? 1 : cP == 1 ? 4 : 16) : nsplit_of(cP, cQ);
  const long long warps = (g.nq + 31) / 32 * nsplit;
  const long long threads = warps * 32;
  if (block != 64 && block != 128 && block != 256) return set_err(c, MQ_EINVAL, "integral launch: bad CTA size");
  long long grid = (threads + block - 1) / block;
  if (grid == 0) return MQ_OK;
  if (persistent && EPI != EPI_SCHWARZ) {
    // a work queue: as many CTAs as can be resident (more only find it empty)
    unsigned long long *queue = (unsigned long long *)buf(c, "eri_queue", 256);
    if (!queue) return MQ_ENOMEM;
    MQ_CUDA(c, cudaMemsetAsync(queue, 0, sizeof(unsigned long long), c->stream));
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
    grid = std::min<long long>(grid, (long long)sms * (2048 / block));
    g.queue = queue;
    g.units = warps;
  } else {
    g.queue = nullptr;
  }
  if (grid > 2147483647LL) return set_err(c, MQ_EINVAL, "integral launch too large");
  dim3 gd((unsigned)grid);
  if constexpr (EPI == EPI_STORE && std::is_same<RT, double>::value) {
    if (nsplit > 1) {  // the split classes: per-primitive work shared by the CTA's warps
      const long long ctas = (g.nq + 31) / 32;
      if (ctas > 2147483647LL) return set_err(c, MQ_EINVAL, "integral launch too large");
      if (cP == 2 && cQ == 1) {
        const size_t sm = sizeof(double) * 4 * 32 * nherm(3) + sizeof(int2) * 4 * 32;
        MQ_CUDA(c, cudaFuncSetAttribute(eri_store_shared_kernel<1, 1, 1, 0>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        eri_store_shared_kernel<1, 1, 1, 0><<<(unsigned)ctas, 128, sm, c->stream>>>(g);
      } else {
        const size_t sm = sizeof(double) * 16 * 32 * nherm(4) + sizeof(int2) * 16 * 32;
        MQ_CUDA(c, cudaFuncSetAttribute(eri_store_shared_kernel<1, 1, 1, 1>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        eri_store_shared_kernel<1, 1, 1, 1><<<(unsigned)ctas, 512, sm, c->stream>>>(g);
      }
      c->stats.launches += 1;
      MQ_CUDA(c, cudaGetLastError());
      return sync_check(c, "eri_store");
    }
  }
#define MQ_LAUNCH(a, b, cc, d) eri_kernel<a, b, cc, d, EPI, RT><<<gd, block, 0, c->stream>>>(g)
  if (cP == 0 && cQ == 0) MQ_LAUNCH(0, 0, 0, 0);
  else if (cP == 1 && cQ == 0) MQ_LAUNCH(1, 0, 0, 0);
  else if (cP == 1 && cQ == 1) MQ_LAUNCH(1, 0, 1, 0);
  else if (cP == 2 && cQ == 0) MQ_LAUNCH(1, 1, 0, 0);
  else if (cP == 2 && cQ == 1) MQ_LAUNCH(1, 1, 1, 0);
  else MQ_LAUNCH(1, 1, 1, 1);
#undef MQ_LAUNCH
  c->stats.launches += 1;
  MQ_CUDA(c, cudaGetLastError());
  return sync_check(c, EPI == EPI_SCHWARZ ? "eri_schwarz"
                       : (EPI == EPI_XX ? "eri_xx" : (EPI == EPI_STORE ? "eri_store" : "eri_fock")));
}

static EriArgs base_args(mq_ctx *c) {
  EriArgs g{};
  g.t = c->pt;
  g.boys = c->d_boys;
  g.mode = c->mode;
  g.n = c->nao;
  return g;
}

}  // namespace mq
