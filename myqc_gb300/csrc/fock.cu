// fock.cu -- two-electron Fock matrix from the device-resident full XX.
//
// Replaces RHFI2G (src/I2G/RHFI2G.f90:80-90) and UHFI2G (src/I2G/UHFI2G.f90:80-93).
// For symmetric densities the reference's
//   G_ij = sum_kl D_kl [(ij|kl) - 1/4 (ik|jl) - 1/4 (il|jk)]
// is J - K/2 with J_ij = sum_kl (ij|kl) D_kl and K_ij = sum_kl (ik|jl) D_kl; UHF
// uses G^a = J[Da+Db] - K[Da], G^b = J[Da+Db] - K[Db].
//
// One streaming pass over XX.  The slab S = XX(:,:,i,j) (n^2 contiguous
// doubles, (kl|ij) for all k,l) gives J_ij = <S, Dt> and adds S . D(:,j) to
// column i of K.  A CTA owns one i and a chunk of j: J_ij is complete inside
// the CTA, and the chunk's partial K column goes to a scratch slice; a second
// kernel sums the slices in a fixed order.  No atomics, deterministic.
#include <algorithm>
#include <type_traits>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>

#include "df32.cuh"
#include "internal.h"

namespace mq {

constexpr int FOCK_THREADS = 256;

// Arithmetic of the digestion.  ArithF64 is plain FP64, the reference's
// arithmetic (the default).  ArithDF32 keeps each integral as a float pair and
// the row sums as double-float on the FP32 pipes (opt-in, mq_set_fock_precision):
// about 2^-48 relative per product, below 1e-12 relative on G.  Either way
// the sums over slabs and the assembly are FP64.
struct ArithDF32 {
  typedef float2 Den;  // a density element as the kernels read it
  typedef float2 Acc;
  __device__ static Acc zero() { return make_float2(0.f, 0.f); }
  __device__ static float2 load(const double *p) { return split_f64(__ldcs(p)); }
  __device__ static float2 cvt(double x) { return split_f64(x); }
  __device__ static void fma(Acc &s, float2 x, Den d) { dfma(s, x, d); }
  __device__ static double val(Acc s) { return (double)s.x + (double)s.y; }
};
struct ArithF64 {
  typedef double Den;
  typedef double Acc;
  __device__ static Acc zero() { return 0.0; }
  __device__ static double load(const double *p) { return __ldcs(p); }
  __device__ static double cvt(double x) { return x; }
  __device__ static void fma(Acc &s, double x, Den d) { s = ::fma(x, d, s); }
  __device__ static double val(Acc s) { return s; }
};

// ArithF32: single-precision products and row sums, for the increments
// G[D_k - D_{k-1}] of an SCF whose density has almost stopped changing (the
// error scales with the increment).  An integral becomes a float by
// truncating its significand (integer operations; relative error < 2^-23,
// values below 2^-126 flush to 0).
struct ArithF32 {
  typedef float Den;
  typedef float Acc;
  __device__ static Acc zero() { return 0.f; }
  __device__ static float cvt(double x) {
    const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
    const unsigned sign = hi & 0x80000000u;
    const unsigned E = (hi >> 20) & 0x7ffu;
    const unsigned hb = sign | (((hi & 0x7fffffffu) - 0x38000000u) << 3) | (lo >> 29);
    return __uint_as_float(E > 896u ? hb : sign);
  }
  __device__ static float load(const double *p) { return cvt(__ldcs(p)); }
  __device__ static void fma(Acc &s, float x, Den d) { s = fmaf(x, d, s); }
  __device__ static double val(Acc s) { return (double)s; }
};

// FP32 density increments: DJ = triangle-weighted total (Da + Db) - (Dpa + Dpb),
// DKa = Da - Dpa, DKb = Db - Dpb (UHF), differences formed in FP64
__global__ void delta_density_f32_kernel(const double *__restrict__ Da, const double *__restrict__ Db,
                                         const double *__restrict__ Dpa, const double *__restrict__ Dpb, size_t n2,
                                         int tri_n, float *__restrict__ DJ, float *__restrict__ DKa,
                                         float *__restrict__ DKb) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n2) return;
  const double a = Da[i] - Dpa[i];
  const double b = Db ? Db[i] - Dpb[i] : 0.0;
  const size_t k = i % (size_t)tri_n, l = i / (size_t)tri_n;
  const double wj = l < k ? 2.0 : (l == k ? 1.0 : 0.0);
  DJ[i] = (float)(wj * (a + b));
  DKa[i] = (float)a;
  if (Db) DKb[i] = (float)b;
}

// FP64 density prepared for J: the lower-triangle weights of the total density
// (2 D(k,l) for l < k, D(k,k), 0 above) for a system of order tri_n
__global__ void prep_density_f64_kernel(const double *__restrict__ Da, const double *__restrict__ Db, size_t n2,
                                        double *__restrict__ DJ, int tri_n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n2) return;
  const size_t k = i % (size_t)tri_n, l = i / (size_t)tri_n;
  const double w = l < k ? 2.0 : (l == k ? 1.0 : 0.0);
  DJ[i] = w * (Da[i] + (Db ? Db[i] : 0.0));
}

// density hi/lo pairs: DJ from Da (+ Db), DKa from Da, DKb from Db (UHF).
// With tri_n > 0 (the order n of one system) DJ holds the lower-triangle
// weights for J over half of a symmetric slab: 2 D(k,l) for l < k, D(k,k) on
// the diagonal, 0 above; DKa must then be a separate array.
__global__ void split_density_kernel(const double *__restrict__ Da, const double *__restrict__ Db, size_t n2,
                                     float2 *__restrict__ DJ, float2 *__restrict__ DKa, float2 *__restrict__ DKb,
                                     int tri_n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n2) return;
  const double a = Da[i];
  const double b = Db ? Db[i] : 0.0;
  double wj = 1.0;
  if (tri_n > 0) {
    const size_t k = i % (size_t)tri_n, l = i / (size_t)tri_n;
    wj = l < k ? 2.0 : (l == k ? 1.0 : 0.0);
  }
  DJ[i] = split_f64(wj * (a + b));
  if (tri_n > 0 || Db) DKa[i] = split_f64(a);
  if (Db) DKb[i] = split_f64(b);
}

int split_density(mq_ctx *c, const double *Da, const double *Db, size_t n2, float2 *DJ, float2 *DKa, float2 *DKb,
                  int tri_n) {
  if (n2 == 0) return MQ_OK;
  split_density_kernel<<<(unsigned)((n2 + 255) / 256), 256, 0, c->stream>>>(Da, Db, n2, DJ, DKa, DKb, tri_n);
  c->stats.launches += 1;
  MQ_CUDA(c, cudaGetLastError());
  return MQ_OK;
}

template <class P, bool UHF>
__global__ void __launch_bounds__(FOCK_THREADS) fock_slab_kernel(const double *__restrict__ XX,
                                                                 const typename P::Den *__restrict__ DJ,
                                                                 const typename P::Den *__restrict__ DKa,
                                                                 const typename P::Den *__restrict__ DKb, int n,
                                                                 int jchunk, double *__restrict__ J,
                                                                 double *__restrict__ Kpa, double *__restrict__ Kpb) {
  const int i = blockIdx.x, chunk = blockIdx.y;
  const int j0 = chunk * jchunk, j1 = min(n, j0 + jchunk);
  const size_t N = n, n2 = N * N;
  __shared__ double red[FOCK_THREADS / 32];
  // each thread owns rows k = tid, tid + 256, ... (at most 4 rows: n <= 1024)
  double ka[4] = {0, 0, 0, 0}, kb[4] = {0, 0, 0, 0};
  for (int j = j0; j < j1; ++j) {
    const double *S = XX + n2 * ((size_t)i + N * j);
    double jsum = 0.0;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int k = threadIdx.x + r * FOCK_THREADS;
      if (k >= n) break;
      typename P::Acc sa = P::zero(), sb = sa, sj = sa;
#pragma unroll 4
      for (int l = 0; l < n; ++l) {
        const auto x = P::load(S + k + N * l);  // streamed once: do not keep in L2
        P::fma(sj, x, DJ[k + N * l]);
        P::fma(sa, x, DKa[l + N * j]);
        if (UHF) P::fma(sb, x, DKb[l + N * j]);
      }
      jsum += P::val(sj);
      ka[r] += P::val(sa);
      if (UHF) kb[r] += P::val(sb);
    }
    // block reduction of J_ij
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) jsum += __shfl_xor_sync(0xffffffffu, jsum, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = jsum;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (int w = 0; w < FOCK_THREADS / 32; ++w) t += red[w];
      J[i + N * j] = t;
    }
    __syncthreads();
  }
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int k = threadIdx.x + r * FOCK_THREADS;
    if (k >= n) break;
    Kpa[n2 * chunk + k + N * i] = ka[r];
    if (UHF) Kpb[n2 * chunk + k + N * i] = kb[r];
  }
}

// G = J - f*K_total with K_total the sum of the chunk slices (fixed order),
// symmetrised as (K_ij + K_ji)/2.  J_ij and J_ji come from identical slabs in
// the same order and are equal bit for bit; K_ij and K_ji come from different
// slabs and differ by rounding, which the eigensolver must not see as an
// off-diagonal residue it cannot rotate away.
__global__ void fock_combine_kernel(const double *__restrict__ J, const double *__restrict__ Kp, int nchunk, int n,
                                    double f, double *__restrict__ G) {
  const size_t N = n, n2 = N * N;
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n2) return;
  const size_t tdx = (idx % N) * N + idx / N;
  double k = 0.0, kt = 0.0;
  for (int c = 0; c < nchunk; ++c) {
    k += Kp[n2 * c + idx];
    kt += Kp[n2 * c + tdx];
  }
  G[idx] = J[idx] - f * (0.5 * (k + kt));
}

// ---- pair-slab digestion: only the slabs with i <= j ------------------------
// Slab (i,j) and slab (j,i) hold the same n^2 values ((kl|ij) = (kl|ji)), so
// one read of S = XX(:,:,i,j), i <= j, serves
//   J_ij = J_ji = <S, Dt>,   K[:,i] += S . D(:,j),   K[:,j] += S . D(:,i) (i < j)
// and half of XX is never read.  A CTA owns one i and a run of up to JC
// consecutive j >= i (a tile): the l loop loads the density row element once
// and applies it to all JC slabs, whose XX streams are in flight together.
// K[:,i] accumulates over the tile in registers and goes to a per-tile slice;
// the contribution of slab (i,j) to K[:,j] goes to Q[:, i, j].  An assembly
// kernel then sums, in a fixed order, the row-j tile slices and Q[:, i<j, j]:
// deterministic, no atomics.  Thread t of T = blockDim.x owns rows k = t + T r,
// r < R.
constexpr int PAIR_MAX_THREADS = 256;
// A tile is (i, j0, j1, molecule); the molecule's descriptor gives its order
// and where its XX, matrices and Q live, so one launch serves one system or a
// whole batch.  Tiles of molecules whose `active` flag is 0 do nothing.
template <class P, int R, int JC, bool UHF>
__global__ void __launch_bounds__(PAIR_MAX_THREADS) fock_pair_kernel(
    const double *__restrict__ XX, const typename P::Den *__restrict__ DJ, const typename P::Den *__restrict__ DKa,
    const typename P::Den *__restrict__ DKb, const int4 *__restrict__ tiles, const MolDesc *__restrict__ mols,
    const int *__restrict__ active, int kp_stride, int tri, const unsigned char *__restrict__ live,
    double *__restrict__ J, double *__restrict__ Kpa, double *__restrict__ Kpb, double *__restrict__ Qa,
    double *__restrict__ Qb) {
  typedef typename P::Den Den;
  extern __shared__ __align__(16) unsigned char dsh_raw[];
  Den *dsh = (Den *)dsh_raw;  // D(:,i) then D(:,j) for the tile's j (alpha; beta after)
  const int4 tile = tiles[blockIdx.x];
  if (active && !active[tile.w]) return;
  const MolDesc md = mols[tile.w];
  const int i = tile.x, j0 = tile.y, nj = tile.z - tile.y, n = md.n;
  const size_t N = n, n2 = N * N;
  XX += md.xx;
  DJ += md.mat;
  DKa += md.mat;
  if (UHF) DKb += md.mat;
  J += md.mat;
  Qa += md.q;
  if (UHF) Qb += md.q;
  const int tid = threadIdx.x, T = blockDim.x;
  Den *dia = dsh, *dja = dsh + n;
  Den *dib = dsh + (size_t)(1 + JC) * n, *djb = dib + n;
  for (int l = tid; l < n; l += T) {
    dia[l] = DKa[l + N * i];
    if (UHF) dib[l] = DKb[l + N * i];
  }
  for (int jj = 0; jj < nj; ++jj)
    for (int l = tid; l < n; l += T) {
      dja[jj * n + l] = DKa[l + N * (j0 + jj)];
      if (UHF) djb[jj * n + l] = DKb[l + N * (j0 + jj)];
    }
  __syncthreads();

  const typename P::Acc z = P::zero();
  const Den dz = Den();
  typename P::Acc aj[JC][R], aqa[JC][R], aqb[UHF ? JC : 1][R], aka[R], akb[R];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    aka[r] = z;
    akb[r] = z;
#pragma unroll
    for (int jj = 0; jj < JC; ++jj) {
      aj[jj][r] = z;
      aqa[jj][r] = z;
      if (UHF) aqb[jj][r] = z;
    }
  }
  // slabs known to be zero (every quartet screened out) are not read
  // live slabs of the tile as a bit mask (kept in a register)
  unsigned lvm = 0;
#pragma unroll
  for (int jj = 0; jj < JC; ++jj)
    if (jj < nj && (!live || live[i + N * (j0 + jj)])) lvm |= 1u << jj;
  const double *S0 = XX + n2 * ((size_t)i + N * j0);
  // FP64 (the reference's arithmetic, the plain path) and the largest orders
  // (R = 4) interleave loads and arithmetic; the FP32-pipe arithmetics batch
  // the loads of several columns (below).
  constexpr bool BATCH = !std::is_same<P, ArithF64>::value && R <= 2;
  if constexpr (!BATCH) {
#pragma unroll 2
    for (int l = 0; lvm && l < n; ++l) {
      const Den di_a = dia[l];
      const Den di_b = UHF ? dib[l] : dz;
      Den dj[R];
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int k = tid + r * T;
        dj[r] = k < n ? DJ[k + N * l] : dz;
      }
#pragma unroll
      for (int jj = 0; jj < JC; ++jj) {
        if (lvm >> jj & 1u) {
          const Den dja_l = dja[jj * n + l];
          const Den djb_l = UHF ? djb[jj * n + l] : dz;
          const double *S = S0 + n2 * N * jj + N * l;
#pragma unroll
          for (int r = 0; r < R; ++r) {
            const int k = tid + r * T;
            if (k < n) {
              const auto x = P::load(S + k);  // streamed once: keep it out of L2
              // triangle weights are 0 for l > k: skip once l passes the warp's last row
              if (!tri || l <= (tid | 31) + r * T) P::fma(aj[jj][r], x, dj[r]);
              P::fma(aka[r], x, dja_l);
              P::fma(aqa[jj][r], x, di_a);
              if (UHF) {
                P::fma(akb[r], x, djb_l);
                P::fma(aqb[jj][r], x, di_b);
              }
            }
          }
        }
      }
    }
  } else {
    // Batched loads: the operands of UB consecutive columns l -- XX(k, l, i, j)
    // of the tile's live slabs and DJ(k, l) for the thread's rows k -- are all
    // requested before any is used, so each thread keeps UB (JC + 1) R loads in
    // flight instead of the few that the interleaved loop above exposes.
    constexpr int UB = JC * R >= 4 ? 2 : (JC * R >= 2 ? 4 : 8);
    for (int l0 = 0; lvm && l0 < n; l0 += UB) {
      double xv[UB][JC][R];
      Den dv[UB][R];
#pragma unroll
      for (int u = 0; u < UB; ++u) {
        const int l = l0 + u;
#pragma unroll
        for (int r = 0; r < R; ++r) {
          const int k = tid + r * T;
          const bool ok = k < n && l < n;
          dv[u][r] = ok ? DJ[k + N * l] : dz;
#pragma unroll
          for (int jj = 0; jj < JC; ++jj)
            xv[u][jj][r] = ok && (lvm >> jj & 1u) ? __ldcs(S0 + n2 * N * jj + N * l + k) : 0.0;
        }
      }
#pragma unroll
      for (int u = 0; u < UB; ++u) {
        const int l = l0 + u;
        if (l >= n) break;
        const Den di_a = dia[l];
        const Den di_b = UHF ? dib[l] : dz;
#pragma unroll
        for (int jj = 0; jj < JC; ++jj) {
          if (lvm >> jj & 1u) {
            const Den dja_l = dja[jj * n + l];
            const Den djb_l = UHF ? djb[jj * n + l] : dz;
#pragma unroll
            for (int r = 0; r < R; ++r) {
              const int k = tid + r * T;
              if (k < n) {
                const auto x = P::cvt(xv[u][jj][r]);
                if (!tri || l <= (tid | 31) + r * T) P::fma(aj[jj][r], x, dv[u][r]);
                P::fma(aka[r], x, dja_l);
                P::fma(aqa[jj][r], x, di_a);
                if (UHF) {
                  P::fma(akb[r], x, djb_l);
                  P::fma(aqb[jj][r], x, di_b);
                }
              }
            }
          }
        }
      }
    }
  }

  // epilogue: J_ij by block reduction, Q(:, i, j) for j > i, the tile's K(:, i) slice
  __shared__ double red[PAIR_MAX_THREADS / 32][JC];
#pragma unroll
  for (int jj = 0; jj < JC; ++jj) {
    double v = 0.0;
#pragma unroll
    for (int r = 0; r < R; ++r) v += P::val(aj[jj][r]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((tid & 31) == 0) red[tid >> 5][jj] = v;
  }
  __syncthreads();
  if (tid < nj) {
    double t = 0.0;
    for (int w = 0; w < T / 32; ++w) t += red[w][tid];
    const int j = j0 + tid;
    J[i + N * j] = t;
    J[j + N * i] = t;
  }
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int k = tid + r * T;
    if (k >= n) continue;
    Kpa[(size_t)kp_stride * blockIdx.x + k] = P::val(aka[r]);
    if (UHF) Kpb[(size_t)kp_stride * blockIdx.x + k] = P::val(akb[r]);
#pragma unroll
    for (int jj = 0; jj < JC; ++jj) {
      const int j = j0 + jj;
      if (jj < nj && j > i) {
        Qa[k + N * i + n2 * j] = P::val(aqa[jj][r]);
        if (UHF) Qb[k + N * i + n2 * j] = P::val(aqb[jj][r]);
      }
    }
  }
}

// K(k, j) = sum over row j's tiles of their slices + sum_{i<j} Q(k, i, j);
// blockIdx.y is the molecule
__global__ void fock_pair_assemble_kernel(const double *__restrict__ Kp, const double *__restrict__ Q,
                                          const int *__restrict__ row_first, const MolDesc *__restrict__ mols,
                                          const int *__restrict__ active, int kp_stride, double *__restrict__ K) {
  const int m = blockIdx.y;
  if (active && !active[m]) return;
  const MolDesc md = mols[m];
  const size_t N = md.n, n2 = N * N;
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n2) return;
  const int k = (int)(idx % N), j = (int)(idx / N);
  const int *rf = row_first + md.row_first;
  Q += md.q;
  double s = 0.0;
  for (int b = rf[j]; b < rf[j + 1]; ++b) s += Kp[(size_t)kp_stride * b + k];
  for (int i = 0; i < j; ++i) s += Q[k + N * i + n2 * j];
  K[md.mat + idx] = s;
}

// G = J - f (K + K^T)/2 per molecule (blockIdx.y), plus Gbase when given
// (single system: an increment added to the previous G)
__global__ void fock_pair_combine_kernel(const double *__restrict__ J, const double *__restrict__ K,
                                         const MolDesc *__restrict__ mols, const int *__restrict__ active, double f,
                                         const double *__restrict__ Gbase, double *__restrict__ G) {
  const int m = blockIdx.y;
  if (active && !active[m]) return;
  const MolDesc md = mols[m];
  const size_t N = md.n, n2 = N * N;
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n2) return;
  const size_t tdx = (idx % N) * N + idx / N;
  const double g = J[md.mat + idx] - f * (0.5 * (K[md.mat + idx] + K[md.mat + tdx]));
  G[md.mat + idx] = Gbase ? Gbase[md.mat + idx] + g : g;
}

template <class P, int R, int JC>
static int launch_pair(mq_ctx *c, const PairLaunch &L, int threads, bool uhf) {
  const size_t smem = sizeof(typename P::Den) * (size_t)(1 + JC) * L.nmax * (uhf ? 2 : 1);  // density columns
  if (smem > 227u * 1024) return set_err(c, MQ_EINVAL, "Fock digestion: shared memory");
  typedef typename P::Den Den;
  const Den *DJ = (const Den *)L.DJ, *DKa = (const Den *)L.DKa, *DKb = (const Den *)L.DKb;
  if (uhf) {
    auto k = fock_pair_kernel<P, R, JC, true>;
    MQ_CUDA(c, cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k<<<L.ntiles, threads, smem, c->stream>>>(L.XX, DJ, DKa, DKb, L.tiles, L.mols, L.active, L.nmax, L.tri, L.live,
                                              L.J, L.Kpa, L.Kpb, L.Qa, L.Qb);
  } else {
    auto k = fock_pair_kernel<P, R, JC, false>;
    MQ_CUDA(c, cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k<<<L.ntiles, threads, smem, c->stream>>>(L.XX, DJ, DKa, nullptr, L.tiles, L.mols, L.active, L.nmax, L.tri,
                                              L.live, L.J, L.Kpa, nullptr, L.Qa, nullptr);
  }
  return MQ_OK;
}

template <class P, int R>
static int launch_pair_jc(mq_ctx *c, int jc, const PairLaunch &L, int threads, bool uhf) {
  switch (jc) {
    case 1: return launch_pair<P, R, 1>(c, L, threads, uhf);
    case 2: return launch_pair<P, R, 2>(c, L, threads, uhf);
    default: return launch_pair<P, R, 4>(c, L, threads, uhf);
  }
}

template <class P>
static int launch_pair_r(mq_ctx *c, int Rp, int jc, const PairLaunch &L, int threads, bool uhf) {
  switch (Rp) {
    case 1: return launch_pair_jc<P, 1>(c, jc, L, threads, uhf);
    case 2: return launch_pair_jc<P, 2>(c, jc, L, threads, uhf);
    default: return launch_pair_jc<P, 4>(c, jc, L, threads, uhf);
  }
}

void pair_tiles_host(int n, int JC, int mol, std::vector<int4> &tl, std::vector<int> &rf) {
  for (int i = 0; i < n; ++i) {
    rf.push_back((int)tl.size());
    for (int j = i; j < n; j += JC) tl.push_back(make_int4(i, j, std::min(n, j + JC), mol));
  }
  rf.push_back((int)tl.size());
}

// Tile table of the single system for JC slabs per tile: (i, j0, j1, 0) over
// row i's j in [i, n), row_first[i] = first tile of row i, and the one
// molecule descriptor.  Cached per (n, JC).
static int pair_tiles(mq_ctx *c, int n, int JC, PairLaunch &L) {
  const size_t N = n;
  FockTiles &ft = c->fock_tiles[JC];
  if (ft.n != n) {
    std::vector<int4> tl;
    std::vector<int> rf;
    pair_tiles_host(n, JC, 0, tl, rf);
    MolDesc md{};
    md.n = n;
    const std::string name = "fock_tiles" + std::to_string(JC);
    char *d = (char *)buf(c, name.c_str(), sizeof(int4) * tl.size() + sizeof(int) * (N + 1) + sizeof(MolDesc) + 16);
    if (!d) return MQ_ENOMEM;
    const size_t o1 = sizeof(int4) * tl.size(), o2 = (o1 + sizeof(int) * (N + 1) + 15) / 16 * 16;
    MQ_CUDA(c, cudaMemcpyAsync(d, tl.data(), o1, cudaMemcpyHostToDevice, c->stream));
    MQ_CUDA(c, cudaMemcpyAsync(d + o1, rf.data(), sizeof(int) * (N + 1), cudaMemcpyHostToDevice, c->stream));
    MQ_CUDA(c, cudaMemcpyAsync(d + o2, &md, sizeof(MolDesc), cudaMemcpyHostToDevice, c->stream));
    MQ_CUDA(c, cudaStreamSynchronize(c->stream));  // the host vectors go out of scope
    ft.n = n;
    ft.ntiles = (int)tl.size();
    ft.d = d;
    ft.rf_off = o1;
    ft.mol_off = o2;
  }
  L.tiles = (const int4 *)ft.d;
  L.row_first = (const int *)(ft.d + ft.rf_off);
  L.mols = (const MolDesc *)(ft.d + ft.mol_off);
  L.ntiles = ft.ntiles;
  L.nmol = 1;
  L.nmax = n;
  L.active = nullptr;
  return MQ_OK;
}

// One digestion of split densities with JC slabs per tile, then assembly of K
// and G = J - f (K + K^T)/2, for all molecules of L.
int pair_digest(mq_ctx *c, int JC, bool uhf, const PairLaunch &L, double *d_Ga, double *d_Gb, bool timed) {
  const int n = L.nmax;
  const int T = std::min(PAIR_MAX_THREADS, (n + 31) / 32 * 32);
  const int R0 = (n + T - 1) / T;
  const int Rp = R0 <= 1 ? 1 : R0 <= 2 ? 2 : 4;
  if (timed) c->t_fock_kernel.start(c->stream);
  if (L.arith == FOCK_ARITH_DF32) MQ_TRY(launch_pair_r<ArithDF32>(c, Rp, JC, L, T, uhf));
  else if (L.arith == FOCK_ARITH_F32) MQ_TRY(launch_pair_r<ArithF32>(c, Rp, JC, L, T, uhf));
  else MQ_TRY(launch_pair_r<ArithF64>(c, Rp, JC, L, T, uhf));
  if (timed) {
    c->t_fock_kernel.stop(c->stream);
    c->stats.fock_kernel_launches += 1;
  }
  MQ_CUDA(c, cudaGetLastError());
  const int tb = 256;
  const dim3 gb((unsigned)(((size_t)n * n + tb - 1) / tb), (unsigned)L.nmol);
  fock_pair_assemble_kernel<<<gb, tb, 0, c->stream>>>(L.Kpa, L.Qa, L.row_first, L.mols, L.active, L.nmax, L.Ka);
  if (uhf)
    fock_pair_assemble_kernel<<<gb, tb, 0, c->stream>>>(L.Kpb, L.Qb, L.row_first, L.mols, L.active, L.nmax, L.Kb);
  const size_t n2 = (size_t)n * n;
  fock_pair_combine_kernel<<<gb, tb, 0, c->stream>>>(L.J, L.Ka, L.mols, L.active, uhf ? 1.0 : 0.5, L.Gbase, d_Ga);
  if (uhf)
    fock_pair_combine_kernel<<<gb, tb, 0, c->stream>>>(L.J, L.Kb, L.mols, L.active, 1.0,
                                                       L.Gbase ? L.Gbase + n2 : nullptr, d_Gb);
  c->stats.launches += uhf ? 5 : 3;
  MQ_CUDA(c, cudaGetLastError());
  return MQ_OK;
}

// Scratch of the single system: J | K slices | Q | K.
static int pair_build(mq_ctx *c, int arith, int JC, bool uhf, const void *DJ, const void *DKa, const void *DKb,
                      double *d_Ga, double *d_Gb, bool timed = false, const double *Gbase = nullptr) {
  const int n = c->nao;
  const size_t N = n, n2 = N * N;
  PairLaunch L{};
  MQ_TRY(pair_tiles(c, n, JC, L));
  const int ns = uhf ? 2 : 1;
  const size_t nt = L.ntiles;
  double *J = (double *)buf(c, "fock_partials", sizeof(double) * (n2 + ns * (N * nt + N * n2 + n2)));
  if (!J) return MQ_ENOMEM;
  L.XX = c->d_XX;
  L.tri = 1;
  L.live = c->slab_live_valid ? c->d_slab_live : nullptr;
  L.arith = arith;
  L.Gbase = Gbase;
  L.DJ = DJ;
  L.DKa = DKa;
  L.DKb = DKb;
  L.J = J;
  L.Kpa = J + n2;
  L.Kpb = uhf ? L.Kpa + N * nt : nullptr;
  L.Qa = J + n2 + ns * N * nt;
  L.Qb = uhf ? L.Qa + N * n2 : nullptr;
  L.Ka = J + n2 + ns * (N * nt + N * n2);
  L.Kb = uhf ? L.Ka + n2 : nullptr;
  return pair_digest(c, JC, uhf, L, d_Ga, d_Gb, timed);
}

// Autotuner for the tile length JC: on the first build for a given (n, RHF or
// UHF, arithmetic) each candidate digests the caller's densities twice under
// CUDA events and the fastest is kept for the context's later builds.  Every
// candidate computes the same G (the tile length only changes the summation
// grouping, ~1e-13 relative), and the call's result comes from the chosen one.
// MYQC_FOCK_JC=1|2|4 in the environment pins the choice instead.
static int pair_choose_jc(mq_ctx *c, int arith, bool uhf, const void *DJ, const void *DKa, const void *DKb,
                          double *d_Ga, double *d_Gb) {
  const int n = c->nao;
  int &slot = c->fock_jc[uhf ? 1 : 0][arith];
  int &slot_n = c->fock_jc_n[uhf ? 1 : 0][arith];
  if (slot_n == n && slot > 0) return slot;
  if (const char *e = getenv("MYQC_FOCK_JC")) {
    const int v = atoi(e);
    slot = v >= 4 ? 4 : v >= 2 ? 2 : 1;
    slot_n = n;
    return slot;
  }
  const int cand[3] = {1, 2, 4};
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  float best = 1e30f;
  int best_jc = 2;
  for (int jc : cand) {
    if (pair_build(c, arith, jc, uhf, DJ, DKa, DKb, d_Ga, d_Gb) != MQ_OK) continue;  // warm-up, tile table
    cudaEventRecord(a, c->stream);
    bool ok = true;
    for (int r = 0; r < 2 && ok; ++r) ok = pair_build(c, arith, jc, uhf, DJ, DKa, DKb, d_Ga, d_Gb) == MQ_OK;
    cudaEventRecord(b, c->stream);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    if (ok && ms < best) {
      best = ms;
      best_jc = jc;
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  c->stats.tune_fock_ms = best / 2;
  slot = best_jc;
  slot_n = n;
  return slot;
}

// Density operands for the digestion, in the context's arithmetic: DJ the
// triangle-weighted total density, DKa / DKb the spin densities (FP64: the
// caller's arrays themselves; double-float: split copies).
int fock_densities(mq_ctx *c, int n, const double *d_Da, const double *d_Db, const void **DJ, const void **DKa,
                   const void **DKb) {
  const size_t n2 = (size_t)n * n;
  const bool uhf = d_Db != nullptr;
  if (c->fock_df32) {
    float2 *d = (float2 *)buf(c, "fock_dsplit", sizeof(float2) * n2 * (uhf ? 3 : 2));
    if (!d) return MQ_ENOMEM;
    MQ_TRY(split_density(c, d_Da, d_Db, n2, d, d + n2, uhf ? d + 2 * n2 : nullptr, n));
    *DJ = d;
    *DKa = d + n2;
    *DKb = uhf ? d + 2 * n2 : nullptr;
  } else {
    double *d = (double *)buf(c, "fock_dsplit", sizeof(double) * n2);
    if (!d) return MQ_ENOMEM;
    prep_density_f64_kernel<<<(unsigned)((n2 + 255) / 256), 256, 0, c->stream>>>(d_Da, d_Db, n2, d, n);
    c->stats.launches += 1;
    MQ_CUDA(c, cudaGetLastError());
    *DJ = d;
    *DKa = d_Da;
    *DKb = d_Db;
  }
  return MQ_OK;
}

int fock_stored_device(mq_ctx *c, const double *d_Da, const double *d_Db, double *d_Ga, double *d_Gb) {
  const int n = c->nao;
  const bool uhf = d_Db != nullptr;
  if (c->qs.valid && !uhf && !c->fock_df32) {  // RHF, FP64: digest the quartet store itself
    c->t_fock_kernel.collect();
    c->t_fock_kernel.start(c->stream);
    const int rc = qstore_fock_rhf(c, d_Da, d_Ga);
    c->t_fock_kernel.stop(c->stream);
    c->stats.fock_kernel_launches += 1;
    return rc;
  }
  MQ_TRY(ensure_xx_full(c));
  MQ_TRY(join_side(c));
  if (n > 4 * PAIR_MAX_THREADS) return set_err(c, MQ_EINVAL, "stored Fock build supports n <= 1024");
  const void *DJ, *DKa, *DKb;
  MQ_TRY(fock_densities(c, n, d_Da, d_Db, &DJ, &DKa, &DKb));
  const int arith = c->fock_df32 ? FOCK_ARITH_DF32 : FOCK_ARITH_F64;
  const int JC = pair_choose_jc(c, arith, uhf, DJ, DKa, DKb, d_Ga, d_Gb);
  c->stats.fock_jc = JC;
  c->t_fock_kernel.collect();  // a previous build's timing not yet collected by its caller
  return pair_build(c, arith, JC, uhf, DJ, DKa, DKb, d_Ga, d_Gb, true);
}

// G = Gprev + G[D - Dprev], the increment digested in FP32 (J and K linear in
// D).  On the first call for an order n the autotuner's candidate builds write
// the bare increment to G before the final build overwrites it, so G must not
// alias Gprev.
int fock_stored_increment(mq_ctx *c, const double *d_Da, const double *d_Db, const double *d_Dpa,
                          const double *d_Dpb, const double *d_Gpa, const double *d_Gpb, double *d_Ga, double *d_Gb) {
  const int n = c->nao;
  MQ_TRY(ensure_xx_full(c));
  MQ_TRY(join_side(c));
  if (n > 4 * PAIR_MAX_THREADS) return set_err(c, MQ_EINVAL, "stored Fock build supports n <= 1024");
  const bool uhf = d_Db != nullptr;
  if (uhf && d_Gpb != d_Gpa + (size_t)n * n) return set_err(c, MQ_EINVAL, "increment: beta G must follow alpha G");
  if (d_Ga == d_Gpa) return set_err(c, MQ_EINVAL, "increment: G must not alias the previous G");
  const size_t n2 = (size_t)n * n;
  float *d = (float *)buf(c, "fock_dinc", sizeof(float) * n2 * (uhf ? 3 : 2));
  if (!d) return MQ_ENOMEM;
  delta_density_f32_kernel<<<(unsigned)((n2 + 255) / 256), 256, 0, c->stream>>>(
      d_Da, d_Db, d_Dpa, d_Dpb, n2, n, d, d + n2, uhf ? d + 2 * n2 : nullptr);
  c->stats.launches += 1;
  MQ_CUDA(c, cudaGetLastError());
  const void *DJ = d, *DKa = d + n2, *DKb = uhf ? d + 2 * n2 : nullptr;
  const int JC = pair_choose_jc(c, FOCK_ARITH_F32, uhf, DJ, DKa, DKb, d_Ga, d_Gb);
  c->t_fock_kernel.collect();
  return pair_build(c, FOCK_ARITH_F32, JC, uhf, DJ, DKa, DKb, d_Ga, d_Gb, true, d_Gpa);
}

// ---------------------------------------------------------------------------
// Allocation-free RHF Fock build (mq_fock_rhf_noalloc).
//
// For callers that may not allocate device memory themselves -- a Fortran or
// C host whose device arrays are owned by an OpenACC / OpenMP-offload runtime
// or by a preallocated pool, or code that must not call cudaMalloc while it
// runs -- a slab digestion (FP64, full slabs) and the combine kernel run on
// caller-owned device buffers, with their scratch (J and the per-chunk K
// columns) in the fixed array below instead of a context buffer.  The array is part of the
// loaded library: every GPU that loads libmyqc holds its 16 MiB until the
// process exits.  Host code cannot use the array's name as a device address;
// the first call on each device looks the address up with
// cudaGetSymbolAddress (with that device current) and keeps it.
constexpr size_t NOALLOC_SCRATCH_DOUBLES = (size_t)2 << 20;  // 16 MiB
static __device__ __align__(256) double g_fock_noalloc_scratch[NOALLOC_SCRATCH_DOUBLES];
constexpr int NOALLOC_MAX_DEVICES = 64;
static double *g_fock_noalloc_addr[NOALLOC_MAX_DEVICES];
static std::mutex g_fock_noalloc_mu;

static int noalloc_fail(char *msg, int len, int code, const char *what) {
  if (msg && len > 0) {
    strncpy(msg, what, len - 1);
    msg[len - 1] = 0;
  }
  return code;
}

}  // namespace mq

extern "C" int mq_fock_rhf_noalloc(int n, const double *d_XX, const double *d_D, double *d_G, void *stream,
                                   char *msg, int msglen) {
  using namespace mq;
  if (n <= 0 || !d_XX || !d_D || !d_G) return noalloc_fail(msg, msglen, MQ_EINVAL, "null pointer or n <= 0");
  if (n > 4 * FOCK_THREADS) return noalloc_fail(msg, msglen, MQ_EINVAL, "n > 1024 is not supported");
  const size_t n2 = (size_t)n * n;
  // J and at least one K slice must fit the fixed scratch: 2 n^2 <= 2 Mi
  // doubles, which n <= 1024 always meets
  if (2 * n2 > NOALLOC_SCRATCH_DOUBLES)
    return noalloc_fail(msg, msglen, MQ_EINVAL, "scratch too small: 2 n^2 must not exceed 2097152 doubles");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NOALLOC_MAX_DEVICES)
    return noalloc_fail(msg, msglen, MQ_ECUDA, "cudaGetDevice failed");
  double *scr = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_fock_noalloc_mu);
    if (!g_fock_noalloc_addr[dev]) {
      void *p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_fock_noalloc_scratch);
      if (e != cudaSuccess || !p) return noalloc_fail(msg, msglen, MQ_ECUDA, cudaGetErrorString(e));
      g_fock_noalloc_addr[dev] = (double *)p;
    }
    scr = g_fock_noalloc_addr[dev];
  }
  int sms = 148;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int nmax = (int)(NOALLOC_SCRATCH_DOUBLES / n2) - 1;  // K slices that fit beside J
  int nchunk = std::max(1, std::min({n, (4 * sms + n - 1) / n, nmax}));
  const int jchunk = (n + nchunk - 1) / nchunk;
  nchunk = (n + jchunk - 1) / jchunk;
  // every J and K-slice element is written by the first kernel before the
  // second reads it, so nothing needs clearing between calls (FP64 throughout)
  double *J = scr, *Kp = scr + n2;
  cudaStream_t s = (cudaStream_t)stream;
  fock_slab_kernel<ArithF64, false><<<dim3(n, nchunk), FOCK_THREADS, 0, s>>>(d_XX, d_D, d_D, nullptr, n, jchunk, J, Kp,
                                                                             nullptr);
  fock_combine_kernel<<<(unsigned)((n2 + 255) / 256), 256, 0, s>>>(J, Kp, nchunk, n, 0.5, d_G);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return noalloc_fail(msg, msglen, MQ_ECUDA, cudaGetErrorString(e));
  return MQ_OK;
}
