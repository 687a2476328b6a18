// qstore.cu -- the quartet store and the sparse FP64 RHF Fock digestion over it.
//
// The reference keeps all n^4 integrals (XX, filled 8-fold by fillsym,
// src/integrals/int2e.f90:540-613) and RHFI2G digests every one of them in
// each SCF iteration (src/I2G/RHFI2G.f90:80-90).  Most of them are zero by the
// Schwarz screen, and each unique value is stored eight times.  Here every
// contracted shell quartet (AB|CD) with bound_AB bound_CD >= threshold is
// computed once and its block of NA NB NC ND integrals (layout
// ((a NB + b) NC + c) ND + d) is written once, contiguous, into the store.
//
// Layout: the pairs of each class ((s,s), (sp,s), (sp,sp)) are ranked by
// Schwarz bound, descending.  For a class combination (bra class cP >= ket
// class cQ) the surviving kets of bra rank r are then the ket ranks
// s < len_r -- a staircase: len_r = m_r = #{s : b_P(r) b_Q(s) >= thr}, or
// min(m_r, r + 1) within one class (each unordered quartet once).  Quartet
// (r, s) sits at off[r] + s, so any block is found from its two ranks, and the
// bra ranks that reach ket rank s form the range r < R_s (m_r falls with r).
//
// Digestion of the canonical quartets, as the direct build does (element
// filter i >= j for A = B, k >= l for C = D, ij >= kl for P = Q; weight w
// halved for i = j, for k = l and for (i,j) = (k,l)):
//   Jh[i,j] += 4 w x D[k,l]    Jh[k,l] += 4 w x D[i,j]
//   Kh[i,k] += 2 w x D[j,l]    Kh[i,l] += 2 w x D[j,k]
//   Kh[j,k] += 2 w x D[i,l]    Kh[j,l] += 2 w x D[i,k]
//   G = (Jh + Jh^T)/2 - (Kh + Kh^T)/4                       (RHF, D total)
// which is the reference's G_ij = sum_kl D_kl [(ij|kl) - (ik|jl)/4 - (il|jk)/4],
// with six FP64 multiply-adds per unique integral that passes the screen.
// The constant factors 4 and 2 are applied once, in the assembly.
//
// Row pass: one CTA per bra pair P = (A,B) and one thread per shell s.
// Thread s walks the kets Q of P's staircase rows in which s is the first
// shell C (adding Kh[i,k], Kh[j,k] and the row part of Jh[i,j]) or the second
// shell D (Kh[i,l], Kh[j,l]).  It alone owns the columns of s in P's partial
// rows Kh[A u B, :], so nothing is shared and nothing is atomic.  Column
// pass: one CTA per ket pair Q, Jh[k,l] over the bra pairs that reach Q.
// Assembly sums each shell's partial rows over the pairs that contain it in a
// fixed order.  The result is deterministic.
#include <algorithm>
#include <cstring>
#include <vector>

#include "internal.h"

namespace mq {

// functions of the first (A) and second (B) shell of a pair class:
// class 0 (s,s), 1 (sp,s), 2 (sp,sp)
__host__ __device__ constexpr int nfa(int cls) { return cls >= 1 ? 4 : 1; }
__host__ __device__ constexpr int nfb(int cls) { return cls == 2 ? 4 : 1; }
__host__ __device__ constexpr int combo_index(int cP, int cQ) { return cP * (cP + 1) / 2 + cQ; }

constexpr int QS_THREADS = 256;      // row pass: AO columns (x shares) per CTA
constexpr int QS_COL_THREADS = 256;  // column pass
constexpr int QS_SHARES[3] = {1, 2, 4};  // row-pass CTAs per bra pair, by bra class
constexpr int QS_MAX_SHARES = 4;

// rank of each pair of one class by Schwarz bound, descending (ties: pair
// index); the bounds are >= 0, so their bit patterns order like the values
__global__ void qs_rank_kernel(const double *__restrict__ sch, int off, int cnt, int *__restrict__ perm) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= cnt) return;
  const long long mine = __double_as_longlong(sch[off + p]);
  int r = 0;
  for (int q = 0; q < cnt; ++q) {
    const long long o = __double_as_longlong(sch[off + q]);
    r += (o > mine) || (o == mine && q < p);
  }
  perm[off + r] = off + p;
}

// Everything the digestion kernels read.
struct QsArgs {
  const double *X;
  const int *perm;
  const int *shA, *shB, *aoA, *aoB;
  int cls_off[4];
  long long base[6];
  const long long *off[6];
  const int *len[6];
  const int *rcol[6];
  const int *thr_shell;
  int nthr, nsp_pad;
  const int *lst_off;
  const int4 *lst;
  const int4 *rinfo;  // by class offset + rank: pair, A | B << 16, i0 | j0 << 16
  const int *thr_ao;
  int nshare[3];  // row-pass shares (CTAs per bra pair) by bra class
  const int2 *ksh;
  const int *ksh_off;
  const int *shell_ao0;
  int nshell, n, npairs;
  const double *D;
  double *Kpart;  // [pair][8 rows][n]
  double *Jrow;   // [pair][16]
  double *Jcol;   // [pair][16]
  double *Jh, *Kh;
  // screened increments: the kets (and, in the column pass, the bras) of a
  // quartet with sch[P] sch[Q] < kscreen are skipped (0: none); the store's
  // ranks ascend as the bounds fall, so each walk stops at the first one
  const double *sch;
  double kscreen;
};

// canonical-element weight of (i,j,k,l) in a degenerate block (0: not
// canonical; else 1/2 for each of i = j, k = l, (i,j) = (k,l)), from integer
// tests and one table entry
__device__ __forceinline__ double canon_weight(int A, int B, int C, int Dsh, int P, int Q, int i, int j, int k, int l,
                                               int n) {
  const bool zero = (A == B && i < j) || (C == Dsh && k < l) || (P == Q && i * n + j < k * n + l);
  const int h = (i == j) + (k == l) + (i == k && j == l);
  return zero ? 0.0 : (h == 0 ? 1.0 : (h == 1 ? 0.5 : (h == 2 ? 0.25 : 0.125)));
}

// The contribution of one ket block to a row-pass thread's column f.  DEGEN:
// the block has A = B, C = D or P = Q, and its elements carry the canonical
// weights (an integer test per element; the general blocks need none).
template <int NA, int NB, int NC, int ND, int ROLE, bool DEGEN>
__device__ __forceinline__ void row_block(const double *__restrict__ Xb, const double *__restrict__ D, size_t n,
                                          int A, int B, int C, int Dsh, int P, int Q, int i0, int j0, int k0, int l0,
                                          int f, double (&KA)[4], double (&KB)[4], double (&Jr)[4][4]) {
  if (ROLE == 0) {  // column k = k0 + f: Kh[i,k] += x D[j,l], Kh[j,k] += x D[i,l], Jh[i,j] += x D[k,l]
#pragma unroll 1
    for (int d = 0; d < ND; ++d) {
      double Dbd[NB], Dad[NA];
#pragma unroll
      for (int b = 0; b < NB; ++b) Dbd[b] = D[(j0 + b) + n * (l0 + d)];
#pragma unroll
      for (int a = 0; a < NA; ++a) Dad[a] = D[(i0 + a) + n * (l0 + d)];
      const double Dcd = D[(k0 + f) + n * (l0 + d)];
#pragma unroll
      for (int a = 0; a < NA; ++a)
#pragma unroll
        for (int b = 0; b < NB; ++b) {
          double x = Xb[((a * NB + b) * NC + f) * ND + d];
          if (DEGEN) x *= canon_weight(A, B, C, Dsh, P, Q, i0 + a, j0 + b, k0 + f, l0 + d, (int)n);
          KA[a] = fma(x, Dbd[b], KA[a]);
          KB[b] = fma(x, Dad[a], KB[b]);
          Jr[a][b] = fma(x, Dcd, Jr[a][b]);
        }
    }
  } else {  // column l = l0 + f: Kh[i,l] += x D[j,k], Kh[j,l] += x D[i,k]
#pragma unroll 1
    for (int c = 0; c < NC; ++c) {
      double Dbc[NB], Dac[NA];
#pragma unroll
      for (int b = 0; b < NB; ++b) Dbc[b] = D[(j0 + b) + n * (k0 + c)];
#pragma unroll
      for (int a = 0; a < NA; ++a) Dac[a] = D[(i0 + a) + n * (k0 + c)];
#pragma unroll
      for (int a = 0; a < NA; ++a)
#pragma unroll
        for (int b = 0; b < NB; ++b) {
          double x = Xb[((a * NB + b) * NC + c) * ND + f];
          if (DEGEN) x *= canon_weight(A, B, C, Dsh, P, Q, i0 + a, j0 + b, k0 + c, l0 + f, (int)n);
          KA[a] = fma(x, Dbc[b], KA[a]);
          KB[b] = fma(x, Dac[a], KB[b]);
        }
    }
  }
}

// One role of a row-pass thread, which owns AO column f of shell s: the kets
// Q of class CQ whose ROLE-th shell (0: first, 1: second) is s -- ranks from
// lst[lo, hi), ascending, every S-th from lo + k (the column's S threads
// share the list) -- up to the staircase length of bra rank r.
template <int CP, int CQ, int ROLE>
__device__ __forceinline__ void row_role(const QsArgs &g, int r, int P, int A, int B, int i0, int j0, int f, int lo,
                                         int hi, int k, int S, double (&KA)[4], double (&KB)[4], double (&Jr)[4][4]) {
  constexpr int NA = nfa(CP), NB = nfb(CP), NC = nfa(CQ), ND = nfb(CQ);
  constexpr int NOUT = NA * NB * NC * ND;
  constexpr int K = combo_index(CP, CQ);
  const int lenr = g.len[K][r];
  const double *Xc = g.X + g.base[K] + (size_t)g.off[K][r] * NOUT;
  const size_t n = g.n;
  const double *D = g.D;
  const double kq = g.kscreen > 0.0 ? g.kscreen / g.sch[P] : 0.0;  // smallest ket bound kept
#pragma unroll 1
  for (int e = lo + k; e < hi; e += S) {
    const int4 q = g.lst[e];  // rank, pair, shells C | D << 16, AOs k0 | l0 << 16
    if (q.x >= lenr) break;   // ranks ascend: the rest lie beyond the staircase
    if (kq > 0.0 && g.sch[q.y] < kq) break;  // and their bounds fall: the rest are screened out too
    const int Q = q.y, C = q.z & 0xffff, Dsh = q.z >> 16, k0 = q.w & 0xffff, l0 = q.w >> 16;
    const double *Xb = Xc + (size_t)q.x * NOUT;
    if ((A == B) || (C == Dsh) || (P == Q))
      row_block<NA, NB, NC, ND, ROLE, true>(Xb, D, n, A, B, C, Dsh, P, Q, i0, j0, k0, l0, f, KA, KB, Jr);
    else
      row_block<NA, NB, NC, ND, ROLE, false>(Xb, D, n, A, B, C, Dsh, P, Q, i0, j0, k0, l0, f, KA, KB, Jr);
  }
}

template <int CQ, int ROLE>
__device__ __forceinline__ void list_range(const QsArgs &g, int s, int &lo, int &hi) {
  const int *o = g.lst_off + (size_t)(CQ * 2 + ROLE) * (g.nshell + 1);
  lo = o[s];
  hi = o[s + 1];
}

// All roles of the row-pass thread of column slot t (shell s), list share k of S.
template <int CP>
__device__ __forceinline__ void row_column(const QsArgs &g, int r, int P, int A, int B, int i0, int j0, int t, int k,
                                           int S, double (&KA)[4], double (&KB)[4], double (&Jr)[4][4]) {
  const int s = g.thr_shell[t];
  if (s < 0) return;
  const int f = g.thr_ao[t] - g.shell_ao0[s];
  int lo, hi;
  if (t < g.nsp_pad) {  // sp-shell AOs (uniform per warp)
    if constexpr (CP >= 1) {
      list_range<1, 0>(g, s, lo, hi);
      row_role<CP, 1, 0>(g, r, P, A, B, i0, j0, f, lo, hi, k, S, KA, KB, Jr);
    }
    if constexpr (CP >= 2) {
      list_range<2, 0>(g, s, lo, hi);
      row_role<CP, 2, 0>(g, r, P, A, B, i0, j0, f, lo, hi, k, S, KA, KB, Jr);
      list_range<2, 1>(g, s, lo, hi);
      row_role<CP, 2, 1>(g, r, P, A, B, i0, j0, f, lo, hi, k, S, KA, KB, Jr);
    }
  } else {
    list_range<0, 0>(g, s, lo, hi);
    row_role<CP, 0, 0>(g, r, P, A, B, i0, j0, 0, lo, hi, k, S, KA, KB, Jr);
    list_range<0, 1>(g, s, lo, hi);
    row_role<CP, 0, 1>(g, r, P, A, B, i0, j0, 0, lo, hi, k, S, KA, KB, Jr);
    if constexpr (CP >= 1) {
      list_range<1, 1>(g, s, lo, hi);
      row_role<CP, 1, 1>(g, r, P, A, B, i0, j0, 0, lo, hi, k, S, KA, KB, Jr);
    }
  }
}

// Row pass for the bra pairs of class CP: CTA (bra rank, share k of S), thread
// = one AO column (the four AOs of each sp shell first, padded to whole
// warps, then the s shells: warps never mix the two code paths).  Share k
// takes every S-th ket of each list; its partial rows and row part of Jh go to
// its own slice (the assembly adds the S slices in order), so the result does
// not depend on timing.
template <int CP>
__global__ void __launch_bounds__(QS_THREADS) qs_row_kernel(QsArgs g) {
  constexpr int NA = nfa(CP), NB = nfb(CP);
  __shared__ double red[QS_THREADS / 32][NA * NB];
  const int r = blockIdx.x, k = blockIdx.y, S = gridDim.y;
  const int P = g.perm[g.cls_off[CP] + r];
  const int A = g.shA[P], B = g.shB[P], i0 = g.aoA[P], j0 = g.aoB[P];
  const size_t n = g.n;
  double Jr[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) Jr[a][b] = 0.0;
  double *kp0 = g.Kpart + ((size_t)k * g.npairs + P) * 8 * n;
  for (int t = threadIdx.x; t < g.nthr; t += blockDim.x) {
    double KA[4] = {0.0, 0.0, 0.0, 0.0}, KB[4] = {0.0, 0.0, 0.0, 0.0};
    row_column<CP>(g, r, P, A, B, i0, j0, t, k, S, KA, KB, Jr);
    if (g.thr_shell[t] < 0) continue;
    double *kp = kp0 + g.thr_ao[t];  // this column of P's partial rows: A's rows, then B's
#pragma unroll
    for (int a = 0; a < NA; ++a) kp[(size_t)a * n] = KA[a];
#pragma unroll
    for (int b = 0; b < NB; ++b) kp[(size_t)(NA + b) * n] = KB[b];
  }
  // row part of Jh over P's block: warp sums, then the warps in order
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int a = 0; a < NA; ++a)
#pragma unroll
    for (int b = 0; b < NB; ++b) {
      double v = Jr[a][b];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0) red[w][a * NB + b] = v;
    }
  __syncthreads();
  if (threadIdx.x < NA * NB) {
    double v = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) v += red[q][threadIdx.x];
    g.Jrow[((size_t)k * g.npairs + P) * 16 + threadIdx.x] = v;
  }
}

// Column part of Jh for ket pair Q (class CQ) from the bra pairs of class CP
// whose staircase reaches ket rank s.
template <int CP, int CQ>
__device__ __forceinline__ void col_combo(const QsArgs &g, int s, int Q, int C, int Dsh, int k0, int l0,
                                          double (&Jc)[4][4]) {
  constexpr int NA = nfa(CP), NB = nfb(CP), NC = nfa(CQ), ND = nfb(CQ);
  constexpr int NOUT = NA * NB * NC * ND;
  constexpr int K = combo_index(CP, CQ);
  const int r0 = CP == CQ ? s : 0, r1 = g.rcol[K][s];
  const size_t n = g.n;
  const double *D = g.D;
  const double kp = g.kscreen > 0.0 ? g.kscreen / g.sch[Q] : 0.0;  // smallest bra bound kept
  for (int r = r0 + (int)threadIdx.x; r < r1; r += blockDim.x) {
    const int4 pi = g.rinfo[g.cls_off[CP] + r];  // pair, A | B << 16, i0 | j0 << 16
    const int P = pi.x, A = pi.y & 0xffff, B = pi.y >> 16, i0 = pi.z & 0xffff, j0 = pi.z >> 16;
    if (kp > 0.0 && g.sch[P] < kp) break;  // bra ranks ascend as their bounds fall
    if (s >= g.len[K][r]) continue;  // a row another partition holds
    const double *Xb = g.X + g.base[K] + ((size_t)g.off[K][r] + s) * NOUT;
    const bool degen = (A == B) || (C == Dsh) || (P == Q);
    double Dab[NA][NB];
#pragma unroll
    for (int a = 0; a < NA; ++a)
#pragma unroll
      for (int b = 0; b < NB; ++b) Dab[a][b] = D[(i0 + a) + n * (j0 + b)];
#pragma unroll
    for (int a = 0; a < NA; ++a)
#pragma unroll
      for (int b = 0; b < NB; ++b)
#pragma unroll
        for (int c = 0; c < NC; ++c)
#pragma unroll
          for (int d = 0; d < ND; ++d) {
            double x = Xb[((a * NB + b) * NC + c) * ND + d];
            if (degen) x *= canon_weight(A, B, C, Dsh, P, Q, i0 + a, j0 + b, k0 + c, l0 + d, (int)n);
            Jc[c][d] = fma(x, Dab[a][b], Jc[c][d]);
          }
  }
}

template <int CQ>
__global__ void __launch_bounds__(QS_COL_THREADS) qs_col_kernel(QsArgs g) {
  constexpr int NC = nfa(CQ), ND = nfb(CQ);
  __shared__ double red[QS_COL_THREADS / 32][NC * ND];
  const int s = blockIdx.x;
  const int Q = g.perm[g.cls_off[CQ] + s];
  const int C = g.shA[Q], Dsh = g.shB[Q], k0 = g.aoA[Q], l0 = g.aoB[Q];
  double Jc[4][4];
#pragma unroll
  for (int c = 0; c < 4; ++c)
#pragma unroll
    for (int d = 0; d < 4; ++d) Jc[c][d] = 0.0;
  col_combo<CQ, CQ>(g, s, Q, C, Dsh, k0, l0, Jc);
  if constexpr (CQ <= 1) col_combo<CQ + 1, CQ>(g, s, Q, C, Dsh, k0, l0, Jc);
  if constexpr (CQ == 0) col_combo<2, CQ>(g, s, Q, C, Dsh, k0, l0, Jc);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int c = 0; c < NC; ++c)
#pragma unroll
    for (int d = 0; d < ND; ++d) {
      double v = Jc[c][d];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0) red[w][c * ND + d] = v;
    }
  __syncthreads();
  if (threadIdx.x < NC * ND) {
    double v = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) v += red[k][threadIdx.x];
    g.Jcol[(size_t)Q * 16 + threadIdx.x] = v;
  }
}

// Kh rows of shell S: 2 x the sum of its partial rows over the pairs that
// contain it (list order: pair index, A role before B role)
__global__ void qs_khat_kernel(QsArgs g) {
  const int S = blockIdx.x;
  const int a0 = g.shell_ao0[S];
  const int ns = (S + 1 < g.nshell ? g.shell_ao0[S + 1] : g.n) - a0;
  const size_t n = g.n;
  const int e0 = g.ksh_off[S], e1 = g.ksh_off[S + 1];
  for (int idx = blockIdx.y * blockDim.x + threadIdx.x; idx < ns * g.n; idx += gridDim.y * blockDim.x) {
    const int a = idx / g.n, col = idx % g.n;
    double v = 0.0;
    for (int e = e0; e < e1; ++e) {
      const int2 pr = g.ksh[e];
      const int cls = pr.x >= g.cls_off[2] ? 2 : (pr.x >= g.cls_off[1] ? 1 : 0);
      for (int k = 0; k < g.nshare[cls]; ++k)
        v += g.Kpart[((size_t)k * g.npairs + pr.x) * 8 * n + (size_t)(pr.y + a) * n + col];
    }
    g.Kh[(a0 + a) + n * col] = 2.0 * v;
  }
}

// Jh over each pair's block: 4 x (row part + column part)
__global__ void qs_jhat_kernel(QsArgs g) {
  const int P = blockIdx.x * blockDim.x + threadIdx.x;
  if (P >= g.npairs) return;
  const int cls = P >= g.cls_off[2] ? 2 : (P >= g.cls_off[1] ? 1 : 0);
  const int NA = nfa(cls), NB = nfb(cls), i0 = g.aoA[P], j0 = g.aoB[P];
  const size_t n = g.n;
  for (int a = 0; a < NA; ++a)
    for (int b = 0; b < NB; ++b) {
      double v = 0.0;
      for (int k = 0; k < g.nshare[cls]; ++k) v += g.Jrow[((size_t)k * g.npairs + P) * 16 + a * NB + b];
      g.Jh[(i0 + a) + n * (j0 + b)] = 4.0 * (v + g.Jcol[(size_t)P * 16 + a * NB + b]);
    }
}

// G = Gprev + (Jh + Jh^T)/2 - f (Kh + Kh^T)/2   (Gprev null: zero)
__global__ void qs_combine_kernel(const double *__restrict__ Jh, const double *__restrict__ Kh, int n, double f,
                                  const double *__restrict__ Gprev, double *__restrict__ G) {
  const size_t N = n, idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= N * N) return;
  const size_t t = (idx % N) * N + idx / N;
  const double g = 0.5 * (Jh[idx] + Jh[t]) - f * 0.5 * (Kh[idx] + Kh[t]);
  G[idx] = Gprev ? Gprev[idx] + g : g;
}

// The store's blocks written into the full n^4 array, each canonical element
// to its 8 places (the zeroed array then equals the full pass's)
template <int CP, int CQ>
__global__ void qs_expand_kernel(const double *__restrict__ X, long long total, const long long *__restrict__ off,
                                 int nP, const int *__restrict__ permP, const int *__restrict__ permQ,
                                 const int *__restrict__ shA, const int *__restrict__ shB, const int *__restrict__ aoA,
                                 const int *__restrict__ aoB, int n, double *__restrict__ XX) {
  constexpr int NA = nfa(CP), NB = nfb(CP), NC = nfa(CQ), ND = nfb(CQ), NOUT = NA * NB * NC * ND;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= total * NOUT) return;
  const long long q = idx / NOUT;
  const int e = (int)(idx % NOUT);
  int lo = 0, hi = nP - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (off[mid] <= q) lo = mid;
    else hi = mid - 1;
  }
  const int P = permP[lo], Q = permQ[(int)(q - off[lo])];
  const int a = e / (NB * NC * ND), b = (e / (NC * ND)) % NB, c = (e / ND) % NC, d = e % ND;
  const int A = shA[P], B = shB[P], C = shA[Q], D = shB[Q];
  const int i = aoA[P] + a, j = aoB[P] + b, k = aoA[Q] + c, l = aoB[Q] + d;
  const size_t N = n;
  if (A == B && i < j) return;
  if (C == D && k < l) return;
  if (P == Q && (size_t)i * N + j < (size_t)k * N + l) return;
  const double x = X[idx];
  const size_t ij = i + N * j, ji = j + N * i, kl = k + N * l, lk = l + N * k, n2 = N * N;
  XX[ij + n2 * kl] = x;
  XX[ji + n2 * kl] = x;
  XX[ij + n2 * lk] = x;
  XX[ji + n2 * lk] = x;
  XX[kl + n2 * ij] = x;
  XX[lk + n2 * ij] = x;
  XX[kl + n2 * ji] = x;
  XX[lk + n2 * ji] = x;
}

// ---------------------------------------------------------------------------
// host side

// device tables, packed into one context buffer
struct Blob {
  std::vector<char> bytes;
  template <class T>
  size_t add(const T *p, size_t count) {
    size_t o = (bytes.size() + 255) / 256 * 256;
    bytes.resize(o + count * sizeof(T));
    if (count) memcpy(bytes.data() + o, p, count * sizeof(T));
    return o;
  }
};

int qstore_integrals(mq_ctx *c);

// The staircase, digestion tables and store allocation of the current system
// and threshold (rebuilt when either changes), then the integral blocks.
int qstore_build(mq_ctx *c) {
  QStore &qs = c->qs;
  qs.valid = 0;
  const double thr = c->schwarz_thr;
  if (!(thr >= 0.0)) return set_err(c, MQ_EINVAL, "the quartet store needs a Schwarz threshold >= 0");
  MQ_TRY(ensure_schwarz(c));
  if (qs.tables_valid && qs.thr == thr) return qstore_integrals(c);
  const int np = c->pt.npairs, nsh = c->nshell, n = c->nao;
  const int *co = c->hp_class_off;
  if ((int)c->hp_shA.size() != np) return set_err(c, MQ_ESTATE, "pair table host copy missing");
  int *d_perm = (int *)buf(c, "qstore_perm", sizeof(int) * std::max(np, 1));
  if (!d_perm) return MQ_ENOMEM;
  for (int cl = 0; cl < 3; ++cl) {
    const int cnt = co[cl + 1] - co[cl];
    if (cnt > 0) qs_rank_kernel<<<(cnt + 127) / 128, 128, 0, c->stream>>>(c->pt.schwarz, co[cl], cnt, d_perm);
  }
  c->stats.launches += 3;
  MQ_CUDA(c, cudaGetLastError());
  std::vector<int> perm(np);
  std::vector<double> sch(np);
  MQ_CUDA(c, cudaMemcpyAsync(perm.data(), d_perm, sizeof(int) * np, cudaMemcpyDeviceToHost, c->stream));
  MQ_CUDA(c, cudaMemcpyAsync(sch.data(), c->pt.schwarz, sizeof(double) * np, cudaMemcpyDeviceToHost, c->stream));
  MQ_CUDA(c, cudaStreamSynchronize(c->stream));
  qs.perm = d_perm;
  for (int cl = 0; cl < 3; ++cl) {
    qs.ncls[cl] = co[cl + 1] - co[cl];
    qs.cls_off[cl] = co[cl];
  }
  Blob blob;
  size_t o_off[6], o_len[6], o_rcol[6];
  long long base = 0;
  double quartets = 0, unique = 0;
  for (int cP = 0; cP < 3; ++cP)
    for (int cQ = 0; cQ <= cP; ++cQ) {
      const int k = combo_index(cP, cQ);
      QCombo &cb = qs.combo[k];
      cb = QCombo{};
      cb.cP = cP;
      cb.cQ = cQ;
      cb.tri = cP == cQ;
      cb.nout = nfa(cP) * nfb(cP) * nfa(cQ) * nfb(cQ);
      cb.nP = qs.ncls[cP];
      cb.nQ = qs.ncls[cQ];
      std::vector<double> bP(cb.nP), bQ(cb.nQ);
      for (int r = 0; r < cb.nP; ++r) bP[r] = sch[perm[co[cP] + r]];
      for (int s = 0; s < cb.nQ; ++s) bQ[s] = sch[perm[co[cQ] + s]];
      std::vector<long long> off(cb.nP + 1, 0);
      std::vector<int> len(cb.nP), m(cb.nP), rcol(cb.nQ);
      for (int r = 0; r < cb.nP; ++r) {
        int lo = 0, hi = cb.nQ;  // first s with bP[r] bQ[s] < thr
        while (lo < hi) {
          const int mid = (lo + hi) / 2;
          if (bP[r] * bQ[mid] >= thr) lo = mid + 1;
          else hi = mid;
        }
        m[r] = lo;
        len[r] = cb.tri ? std::min(lo, r + 1) : lo;
        // a partition of the quartets over processes: this one keeps the
        // rows whose bra pair index falls to it
        if (c->nparts > 1 && perm[co[cP] + r] % c->nparts != c->part) len[r] = 0;
        off[r + 1] = off[r] + len[r];
      }
      for (int s = 0; s < cb.nQ; ++s) {  // first r with m_r <= s
        int lo = 0, hi = cb.nP;
        while (lo < hi) {
          const int mid = (lo + hi) / 2;
          if (m[mid] > s) lo = mid + 1;
          else hi = mid;
        }
        rcol[s] = lo;
      }
      cb.total = off[cb.nP];
      cb.base = base;
      base += cb.total * cb.nout;
      quartets += (double)cb.total;
      // canonical unique integrals of the combination: degenerate blocks
      // (A = B, C = D, P = Q) hold fewer than NA NB NC ND
      {
        const int fa = nfa(cP), fb = nfb(cP), fc = nfa(cQ), fd = nfb(cQ);
        auto diag = [&](int cls, int rank) {
          const int p = perm[co[cls] + rank];
          return c->hp_shA[p] == c->hp_shB[p];
        };
        std::vector<int> dq(cb.nQ + 1, 0);  // diagonal kets among ranks < s
        for (int s = 0; s < cb.nQ; ++s) dq[s + 1] = dq[s] + (diag(cQ, s) ? 1 : 0);
        const double ub_full = (double)fa * fb, ub_diag = fa * (fa + 1) / 2.0;
        const double uk_full = (double)fc * fd, uk_diag = fc * (fc + 1) / 2.0;
        for (int r = 0; r < cb.nP; ++r) {
          const bool bd = diag(cP, r);
          const double ub = bd ? ub_diag : ub_full;
          const int L = len[r];
          const int nd = dq[L];  // diagonal kets in the row
          double u = ub * (nd * uk_diag + (L - nd) * uk_full);
          if (cb.tri && L > r) {  // the quartet (P,P): pair functions ij >= kl
            const double kk = bd ? uk_diag : uk_full;
            u -= ub * kk;
            u += ub * (ub + 1) / 2.0;
          }
          unique += u;
        }
      }
      o_off[k] = blob.add(off.data(), off.size());
      o_len[k] = blob.add(len.data(), len.size());
      o_rcol[k] = blob.add(rcol.data(), rcol.size());
    }
  // row-pass threads, one per AO column: the four AOs of each sp shell
  // (padded to a warp multiple), then the s shells' AOs (padded)
  std::vector<int> thr_shell, thr_ao;
  for (int s = 0; s < nsh; ++s)
    if (c->shells[s].type == 1)
      for (int f = 0; f < 4; ++f) {
        thr_shell.push_back(s);
        thr_ao.push_back(c->shells[s].ao0 + f);
      }
  while (thr_shell.size() % 32) {
    thr_shell.push_back(-1);
    thr_ao.push_back(0);
  }
  const int nsp_pad = (int)thr_shell.size();
  for (int s = 0; s < nsh; ++s)
    if (c->shells[s].type == 0) {
      thr_shell.push_back(s);
      thr_ao.push_back(c->shells[s].ao0);
    }
  while (thr_shell.size() % 32) {
    thr_shell.push_back(-1);
    thr_ao.push_back(0);
  }
  if (nsh > 0xffff || n > 0xffff) return set_err(c, MQ_EINVAL, "quartet store: more than 65535 shells or AOs");
  // per (ket class, role, shell): the pairs whose role-th shell is s, by
  // ascending rank, packed (rank, pair, C | D << 16, k0 | l0 << 16)
  std::vector<int> lst_off(6 * (nsh + 1), 0);
  std::vector<int4> lst;
  {
    std::vector<std::vector<int4>> l(6 * nsh);
    for (int cl = 0; cl < 3; ++cl)
      for (int t = 0; t < qs.ncls[cl]; ++t) {
        const int p = perm[co[cl] + t];
        const int4 e = make_int4(t, p, c->hp_shA[p] | (c->hp_shB[p] << 16), c->hp_aoA[p] | (c->hp_aoB[p] << 16));
        l[(cl * 2 + 0) * nsh + c->hp_shA[p]].push_back(e);
        l[(cl * 2 + 1) * nsh + c->hp_shB[p]].push_back(e);
      }
    for (int g = 0; g < 6; ++g)
      for (int s = 0; s < nsh; ++s) {
        lst_off[g * (nsh + 1) + s] = (int)lst.size();
        for (const int4 &e : l[g * nsh + s]) lst.push_back(e);
        lst_off[g * (nsh + 1) + s + 1] = (int)lst.size();
      }
  }
  // per shell: (pair, row offset of the shell in the pair's partial K rows)
  std::vector<int> ksh_off(nsh + 1, 0);
  std::vector<int2> ksh;
  {
    std::vector<std::vector<int2>> l(nsh);
    for (int p = 0; p < np; ++p) {
      const int cls = p >= co[2] ? 2 : (p >= co[1] ? 1 : 0);
      l[c->hp_shA[p]].push_back(make_int2(p, 0));
      l[c->hp_shB[p]].push_back(make_int2(p, nfa(cls)));
    }
    for (int s = 0; s < nsh; ++s) {
      ksh_off[s] = (int)ksh.size();
      for (const int2 &e : l[s]) ksh.push_back(e);
      ksh_off[s + 1] = (int)ksh.size();
    }
  }
  std::vector<int> ao0(nsh);
  for (int s = 0; s < nsh; ++s) ao0[s] = c->shells[s].ao0;
  for (int s = 1; s < nsh; ++s)
    if (ao0[s] <= ao0[s - 1]) return set_err(c, MQ_EINVAL, "shell AOs out of order");
  std::vector<int4> rinfo(np);
  for (int k = 0; k < np; ++k) {
    const int p = perm[k];
    rinfo[k] = make_int4(p, c->hp_shA[p] | (c->hp_shB[p] << 16), c->hp_aoA[p] | (c->hp_aoB[p] << 16), 0);
  }
  const size_t o_ri = blob.add(rinfo.data(), rinfo.size());
  const size_t o_thr = blob.add(thr_shell.data(), thr_shell.size());
  const size_t o_tao = blob.add(thr_ao.data(), thr_ao.size());
  const size_t o_lo = blob.add(lst_off.data(), lst_off.size());
  const size_t o_l = blob.add(lst.data(), lst.size());
  const size_t o_ko = blob.add(ksh_off.data(), ksh_off.size());
  const size_t o_k = blob.add(ksh.data(), ksh.size());
  const size_t o_ao = blob.add(ao0.data(), ao0.size());
  // AO -> shell, and (S1, S2) -> the pair holding both, with its class, rank
  // within the class and orientation (for lookups of single integrals)
  std::vector<int> ao_shell(n, 0);
  for (int sh = 0; sh < nsh; ++sh) {
    const int a1 = sh + 1 < nsh ? ao0[sh + 1] : n;
    for (int a = ao0[sh]; a < a1; ++a) ao_shell[a] = sh;
  }
  std::vector<int4> pinfo((size_t)nsh * nsh, make_int4(0, 0, 0, 0));
  for (int cl = 0; cl < 3; ++cl)
    for (int t = 0; t < qs.ncls[cl]; ++t) {
      const int p = perm[co[cl] + t], A = c->hp_shA[p], B = c->hp_shB[p];
      pinfo[(size_t)A * nsh + B] = make_int4(p, cl, t, A == B ? 2 : 0);
      pinfo[(size_t)B * nsh + A] = make_int4(p, cl, t, A == B ? 2 : 1);
    }
  std::vector<double> qmax(nsh, 0.0);
  for (int p = 0; p < np; ++p) {
    qmax[c->hp_shA[p]] = std::max(qmax[c->hp_shA[p]], sch[p]);
    qmax[c->hp_shB[p]] = std::max(qmax[c->hp_shB[p]], sch[p]);
  }
  // per shell S: every shell D ordered by the bound of the pair (D, S),
  // descending -- the shells D of the live quartets (D S|U V) of any pair
  // (U, V) are a prefix of S's list
  std::vector<int> ptn((size_t)nsh * nsh);
  for (int S2 = 0; S2 < nsh; ++S2) {
    int *row = ptn.data() + (size_t)S2 * nsh;
    for (int D1 = 0; D1 < nsh; ++D1) row[D1] = D1;
    std::stable_sort(row, row + nsh, [&](int a, int b) {
      return sch[pinfo[(size_t)a * nsh + S2].x] > sch[pinfo[(size_t)b * nsh + S2].x];
    });
  }
  const size_t o_ptn = blob.add(ptn.data(), ptn.size());
  const size_t o_qm = blob.add(qmax.data(), qmax.size());
  const size_t o_aos = blob.add(ao_shell.data(), ao_shell.size());
  const size_t o_pi = blob.add(pinfo.data(), pinfo.size());
  char *d = (char *)buf(c, "qstore_tab", blob.bytes.size() + 256);
  if (!d) return MQ_ENOMEM;
  MQ_CUDA(c, cudaMemcpyAsync(d, blob.bytes.data(), blob.bytes.size(), cudaMemcpyHostToDevice, c->stream));
  for (int k = 0; k < 6; ++k) {
    qs.combo[k].off = (long long *)(d + o_off[k]);
    qs.combo[k].len = (int *)(d + o_len[k]);
    qs.combo[k].rcol = (int *)(d + o_rcol[k]);
  }
  qs.nthr = (int)thr_shell.size();
  qs.nsp_pad = nsp_pad;
  qs.thr_shell = (int *)(d + o_thr);
  qs.lst_off = (int *)(d + o_lo);
  qs.lst = (int4 *)(d + o_l);
  qs.thr_ao = (int *)(d + o_tao);
  qs.rinfo = (int4 *)(d + o_ri);
  qs.ksh_off = (int *)(d + o_ko);
  qs.ksh = (int2 *)(d + o_k);
  qs.shell_ao0 = (int *)(d + o_ao);
  qs.ao_shell = (int *)(d + o_aos);
  qs.shell_qmax = (double *)(d + o_qm);
  qs.pinfo = (int4 *)(d + o_pi);
  qs.partners = (int *)(d + o_ptn);
  qs.X_elems = (size_t)base;
  qs.X = (double *)buf(c, "qstore_X", sizeof(double) * std::max<size_t>(qs.X_elems, 1));
  if (!qs.X) return MQ_ENOMEM;
  qs.quartets = quartets;
  qs.unique = unique;
  qs.thr = thr;
  (void)n;
  // (a copy from pageable host memory returns once the data is staged, so
  // the blob may go; the integral launches queue behind it)
  qs.tables_valid = 1;
  return qstore_integrals(c);
}

// the integral blocks of the store (tables built), timed on their own
int qstore_integrals(mq_ctx *c) {
  c->t_eri_kernel.collect_sync();
  c->t_eri_kernel.total = 0;
  c->t_eri_kernel.start(c->stream);
  MQ_TRY(eri_store_quartets(c));
  c->t_eri_kernel.stop(c->stream);
  c->qs.valid = 1;
  return MQ_OK;
}

int fock_direct_store_rhf(mq_ctx *c, const double *d_D, double *d_G) {
  MQ_TRY(qstore_build(c));
  return qstore_fock_rhf(c, d_D, d_G);
}

static QsArgs qs_args(mq_ctx *c) {
  const QStore &qs = c->qs;
  QsArgs g{};
  g.X = qs.X;
  g.perm = qs.perm;
  g.shA = c->pt.shA;
  g.shB = c->pt.shB;
  g.aoA = c->pt.aoA;
  g.aoB = c->pt.aoB;
  for (int k = 0; k < 4; ++k) g.cls_off[k] = c->hp_class_off[k];
  for (int k = 0; k < 6; ++k) {
    g.base[k] = qs.combo[k].base;
    g.off[k] = qs.combo[k].off;
    g.len[k] = qs.combo[k].len;
    g.rcol[k] = qs.combo[k].rcol;
  }
  g.thr_shell = qs.thr_shell;
  g.nthr = qs.nthr;
  g.nsp_pad = qs.nsp_pad;
  g.lst_off = qs.lst_off;
  g.lst = qs.lst;
  g.thr_ao = qs.thr_ao;
  g.rinfo = qs.rinfo;
  g.ksh = qs.ksh;
  g.ksh_off = qs.ksh_off;
  g.shell_ao0 = qs.shell_ao0;
  g.nshell = c->nshell;
  g.n = c->nao;
  g.npairs = c->pt.npairs;
  return g;
}

int qstore_fock_rhf(mq_ctx *c, const double *d_D, double *d_G, const double *d_Gprev, double kscreen) {
  const QStore &qs = c->qs;
  if (!qs.valid) return set_err(c, MQ_ESTATE, "no quartet store");
  const int n = c->nao, np = c->pt.npairs;
  const size_t N = n, n2 = N * N;
  const size_t SH = QS_MAX_SHARES;
  double *w = (double *)buf(c, "qstore_fock",
                            sizeof(double) * (SH * np * 8 * N + SH * np * 16 + (size_t)np * 16 + 2 * n2));
  if (!w) return MQ_ENOMEM;
  QsArgs g = qs_args(c);
  g.D = d_D;
  g.sch = c->pt.schwarz;
  g.kscreen = kscreen;
  g.Kpart = w;
  g.Jrow = w + SH * np * 8 * N;
  g.Jcol = g.Jrow + SH * np * 16;
  g.Jh = g.Jcol + (size_t)np * 16;
  g.Kh = g.Jh + n2;
  // pairs that are no bra (or no ket) of any stored quartet still get their
  // partial rows and J parts written (as zeros) by their own CTAs
  MQ_CUDA(c, cudaMemsetAsync(g.Jh, 0, sizeof(double) * n2, c->stream));
  // shares per bra pair: the (sp,sp) and (sp,s) bras have the longest rows
  g.nshare[0] = QS_SHARES[0];
  g.nshare[1] = QS_SHARES[1];
  g.nshare[2] = QS_SHARES[2];
  const int rt = std::min(QS_THREADS, qs.nthr);
  if (qs.ncls[0]) qs_row_kernel<0><<<dim3(qs.ncls[0], g.nshare[0]), rt, 0, c->stream>>>(g);
  if (qs.ncls[1]) qs_row_kernel<1><<<dim3(qs.ncls[1], g.nshare[1]), rt, 0, c->stream>>>(g);
  if (qs.ncls[2]) qs_row_kernel<2><<<dim3(qs.ncls[2], g.nshare[2]), rt, 0, c->stream>>>(g);
  if (qs.ncls[0]) qs_col_kernel<0><<<qs.ncls[0], QS_COL_THREADS, 0, c->stream>>>(g);
  if (qs.ncls[1]) qs_col_kernel<1><<<qs.ncls[1], QS_COL_THREADS, 0, c->stream>>>(g);
  if (qs.ncls[2]) qs_col_kernel<2><<<qs.ncls[2], QS_COL_THREADS, 0, c->stream>>>(g);
  qs_khat_kernel<<<dim3(c->nshell, (4 * n + QS_COL_THREADS - 1) / QS_COL_THREADS), QS_COL_THREADS, 0, c->stream>>>(g);
  qs_jhat_kernel<<<(np + 127) / 128, 128, 0, c->stream>>>(g);
  qs_combine_kernel<<<(unsigned)((n2 + 255) / 256), 256, 0, c->stream>>>(g.Jh, g.Kh, n, 0.5, d_Gprev, d_G);
  c->stats.launches += 9;
  MQ_CUDA(c, cudaGetLastError());
  return sync_check(c, "qstore_fock");
}

int qstore_expand(mq_ctx *c, double *d_XX) {
  const QStore &qs = c->qs;
  if (!qs.valid) return set_err(c, MQ_ESTATE, "no quartet store");
  const size_t n = c->nao;
  MQ_CUDA(c, cudaMemsetAsync(d_XX, 0, n * n * n * n * sizeof(double), c->stream));
  for (int cP = 0; cP < 3; ++cP)
    for (int cQ = 0; cQ <= cP; ++cQ) {
      const QCombo &cb = qs.combo[combo_index(cP, cQ)];
      if (!cb.total) continue;
      const long long items = cb.total * cb.nout;
      const unsigned grid = (unsigned)((items + 255) / 256);
      const int *pP = qs.perm + qs.cls_off[cP], *pQ = qs.perm + qs.cls_off[cQ];
#define MQ_EXP(a, b)                                                                                              \
  qs_expand_kernel<a, b><<<grid, 256, 0, c->stream>>>(qs.X + cb.base, cb.total, cb.off, cb.nP, pP, pQ, c->pt.shA, \
                                                      c->pt.shB, c->pt.aoA, c->pt.aoB, (int)n, d_XX)
      if (cP == 0) MQ_EXP(0, 0);
      else if (cP == 1 && cQ == 0) MQ_EXP(1, 0);
      else if (cP == 1) MQ_EXP(1, 1);
      else if (cQ == 0) MQ_EXP(2, 0);
      else if (cQ == 1) MQ_EXP(2, 1);
      else MQ_EXP(2, 2);
#undef MQ_EXP
      c->stats.launches += 1;
    }
  MQ_CUDA(c, cudaGetLastError());
  return MQ_OK;
}

}  // namespace mq
