// purify.cu -- SCF density step without a diagonalisation.
//
// The reference obtains each new density from the lowest nocc eigenvectors of
// F C = S C e (DSYGV, src/scf/scf.f90:813-848, then dens.f90:115-124).  The
// density depends on F only through the spectral projector P onto those
// eigenvectors (in the orthogonal basis F' = X^T F X, X = S^-1/2):
// D = occf * X P X.  Trace-correcting purification (Niklasson, Phys. Rev. B 66,
// 155115 (2002), "TC2") builds P from F' with matrix products only:
//   X_0 = (hi I - F') / (hi - lo)   (Gershgorin bounds: spectrum mapped into [0,1],
//                                    occupied levels nearest 1)
//   X_{k+1} = X_k^2        if |tr X_k^2 - nocc| < |tr(2X_k - X_k^2) - nocc|
//           = 2X_k - X_k^2 otherwise
// until the idempotency error tr(X - X^2) vanishes; convergence is quadratic
// once the occupied and virtual eigenvalues have separated.  Each step is one
// FP64 GEMM (cuBLAS) and one fused select/update kernel; no host round trip
// except a convergence poll every few steps.  The SCF fixed point does not
// change: at a gapped spectrum P is exactly the aufbau projector.  Without a
// gap (degenerate frontier levels) the error stalls and the caller falls back
// to the eigensolver for that iteration.
#include <algorithm>
#include <cmath>
#include <string>
#include <type_traits>
#include <vector>

#include "df32.cuh"
#include "gridsync.cuh"
#include "internal.h"

namespace mq {

constexpr int PUR_THREADS = 1024;

__device__ __forceinline__ double block_sum(double v, double *red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();  // red may still be read from a previous call
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
  return t;
}

__device__ __forceinline__ double block_min(double v, double *red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = red[0];
  for (int w = 1; w < (int)(blockDim.x >> 5); ++w) t = fmin(t, red[w]);
  return t;
}

// Gershgorin bounds in three launches (one warp per row, a one-CTA min/max,
// an elementwise build) rather than on one SM: row r of the symmetric part
// (F + F^T)/2 gives [d - off, d + off] with off = sum_{j != r} |f_rj|, or with
// sym = 0 the row's absolute sum sum_j |s_rj| in rowhi (Newton-Schulz scale).
__global__ void gersh_rows_kernel(const double *__restrict__ F, int n, int sym, double *__restrict__ rowlo,
                                  double *__restrict__ rowhi) {
  const int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (r >= n) return;
  const size_t N = n;
  double off = 0.0;
  for (int j = lane; j < n; j += 32) {
    if (sym) {
      if (j != r) off += fabs(0.5 * (F[r + N * j] + F[j + N * r]));
    } else {
      off += fabs(F[r + N * j]);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) off += __shfl_xor_sync(0xffffffffu, off, o);
  if (lane == 0) {
    const double d = sym ? F[r + N * r] : 0.0;
    rowlo[r] = d - off;
    rowhi[r] = d + off;
  }
}

// lohi[0] = min rowlo, lohi[1] = max rowhi (one CTA, fixed order per thread)
__global__ void __launch_bounds__(PUR_THREADS) gersh_final_kernel(const double *__restrict__ rowlo,
                                                                  const double *__restrict__ rowhi, int n,
                                                                  double *__restrict__ lohi) {
  __shared__ double red[PUR_THREADS / 32];
  double lo = INFINITY, nhi = INFINITY;
  for (int r = threadIdx.x; r < n; r += blockDim.x) {
    lo = fmin(lo, rowlo[r]);
    nhi = fmin(nhi, -rowhi[r]);
  }
  lo = block_min(lo, red);
  nhi = block_min(nhi, red);
  if (threadIdx.x == 0) {
    lohi[0] = lo;
    lohi[1] = -nhi;
  }
}

// X_0 = (hi I - (F + F^T)/2) / (hi - lo)
__global__ void purify_build_kernel(const double *__restrict__ F, int n, const double *__restrict__ lohi,
                                    double *__restrict__ X) {
  const size_t N = n, idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= N * N) return;
  const double lo = lohi[0], hi = lohi[1];
  const size_t r = idx % N, col = idx / N;
  const double f = 0.5 * (F[idx] + F[col + N * r]);
  X[idx] = ((r == col ? hi : 0.0) - f) / fmax(hi - lo, 1e-300);
}

static int gershgorin(mq_ctx *c, const double *F, int n, int sym, double *lohi) {
  double *rows = (double *)buf(c, "gersh_rows", 2 * (size_t)n * sizeof(double));
  if (!rows) return MQ_ENOMEM;
  gersh_rows_kernel<<<(n * 32 + 255) / 256, 256, 0, c->stream>>>(F, n, sym, rows, rows + n);
  gersh_final_kernel<<<1, PUR_THREADS, 0, c->stream>>>(rows, rows + n, n, lohi);
  c->stats.launches += 2;
  return MQ_OK;
}

// Xn = select(X, T = X X), T given by its lower triangle (DSYRK; X is
// symmetric so X X = X X^T): every CTA reads the two diagonals to make the
// same choice; CTA 0 records the idempotency error tr X - tr T of step k.
__global__ void purify_step_kernel(const double *__restrict__ X, const double *__restrict__ T, int n, double nocc,
                                   double *__restrict__ Xn, double *__restrict__ err, int k) {
  __shared__ double red[32];
  const size_t N = n, n2 = N * N;
  double tx = 0.0, tt = 0.0;
  for (int r = threadIdx.x; r < n; r += blockDim.x) {
    tx += X[r + N * r];
    tt += T[r + N * r];
  }
  tx = block_sum(tx, red);
  tt = block_sum(tt, red);
  const bool square = fabs(tt - nocc) < fabs(2.0 * tx - tt - nocc);
  if (blockIdx.x == 0 && threadIdx.x == 0) err[k] = tx - tt;
  for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n2; idx += (size_t)gridDim.x * blockDim.x) {
    const size_t r = idx % N, col = idx / N;
    const double t = r >= col ? T[idx] : T[col + N * r];  // the lower triangle holds X X
    Xn[idx] = square ? t : 2.0 * X[idx] - t;
  }
}

__global__ void identity_kernel(double *__restrict__ A, int n) {
  const size_t N = n, idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx < N * N) A[idx] = (idx % N == idx / N) ? 1.0 : 0.0;
}

// ---- All TC2 steps in one cooperative launch (n <= PUR_PERSIST_MAX).
// CTA b owns the lower-triangle 16x16 tiles b, b + grid, ... of X^2.  X is
// symmetric, so (X^2)_ij = sum_k X_ki X_kj: the tile's 16 + 16 columns are
// staged in shared memory and each thread forms one element.  F64 = true
// (the default): FP64 products and sums.  F64 = false (contexts whose Fock
// digestion is double-float, mq_set_fock_precision(MQ_FOCK_DF32)): the columns
// as double-float pairs and the products and sums in double-float on the FP32
// pipes, which issue many times faster than FP64 on this GPU.  X itself, the
// selection and the traces are FP64 either way.  The selection
// needs tr X and tr X^2 of the matrix being squared; tr X^2 = ||X||_F^2, so
// both come from per-tile partial sums that the previous step wrote with X
// itself (double-buffered by step parity), and a step is: read the partials,
// decide, square, write the next X and its partials, one grid barrier.  Every
// CTA sums the partials in the same order, so all make the same choices and
// stop together: at step j + 2 after the first step j whose idempotency error
// tr(X_j - X_j^2) is below SETTLED, as the polled loop does.
constexpr int PUR_TILE = 16;
constexpr int PUR_PERSIST_MAX = 640;  // 2 x 16 staged columns of n doubles fit in shared memory
constexpr int PUR_MAX_STEPS = 120;
constexpr double PUR_SETTLED = 1e-9;

__device__ __forceinline__ void tile_of(int t, int &I, int &J) {
  I = (int)((sqrt(8.0 * t + 1.0) - 1.0) * 0.5);
  while (I * (I + 1) / 2 > t) --I;
  while ((I + 1) * (I + 2) / 2 <= t) ++I;
  J = t - I * (I + 1) / 2;
}

// partial sums of one tile of X (lower triangle): [0] diagonal, [1] squares
// weighted by 2 off the diagonal tiles; written to part[2 * tile + 0/1]
__device__ __forceinline__ void tile_partials(double tr, double sq, double *red, double *part, int tile) {
  tr = block_sum(tr, red);
  sq = block_sum(sq, red);
  if (threadIdx.x == 0) {
    part[2 * tile] = tr;
    part[2 * tile + 1] = sq;
  }
}

template <bool F64>
__global__ void __launch_bounds__(256) purify_persist_kernel(int n, double nocc, double *X0,
                                                             double *X1, double *part,
                                                             double *__restrict__ err, int *__restrict__ info,
                                                             GridSync gs) {
  // [2][16][ld] doubles or double-float pairs (8 bytes either way), ld = n | 1:
  // a warp's 16 columns hit 16 bank pairs
  typedef typename std::conditional<F64, double, float2>::type Col;
  extern __shared__ __align__(16) unsigned char cols_raw[];
  Col *cols = (Col *)cols_raw;
  __shared__ double red[32];
  const int nt = (n + PUR_TILE - 1) / PUR_TILE, ntiles = nt * (nt + 1) / 2;
  const int tid = threadIdx.x, ti = tid % PUR_TILE, tj = tid / PUR_TILE;
  const int ld = n | 1;
  const unsigned nb = gridDim.x;
  const size_t N = n;
  // partials of X_0
  for (int tile = blockIdx.x; tile < ntiles; tile += nb) {
    int I, J;
    tile_of(tile, I, J);
    const int i = I * PUR_TILE + ti, j = J * PUR_TILE + tj;
    double tr = 0.0, sq = 0.0;
    if (i < n && j < n) {
      const double x = X0[i + N * j];
      tr = (i == j) ? x : 0.0;
      sq = (I == J ? 1.0 : 2.0) * x * x;
    }
    tile_partials(tr, sq, red, part, tile);
  }
  if (!grid_barrier(gs, nb)) return;
  int settled_at = -1, k = 0;
  for (; k < PUR_MAX_STEPS; ++k) {
    const double *pk = part + (size_t)2 * ntiles * (k & 1);
    double tr = 0.0, sq = 0.0;
    for (int t = tid; t < ntiles; t += blockDim.x) {
      tr += pk[2 * t];
      sq += pk[2 * t + 1];
    }
    const double tx = block_sum(tr, red), tt = block_sum(sq, red);
    const double e = tx - tt;
    if (blockIdx.x == 0 && tid == 0) err[k] = e;
    if (settled_at < 0 && fabs(e) < PUR_SETTLED) settled_at = k;
    if (settled_at >= 0 && k >= settled_at + 2) break;
    const bool square = fabs(tt - nocc) < fabs(2.0 * tx - tt - nocc);
    const double *X = (k & 1) ? X1 : X0;
    double *Y = (k & 1) ? X0 : X1;
    double *pn = part + (size_t)2 * ntiles * ((k + 1) & 1);
    for (int tile = blockIdx.x; tile < ntiles; tile += nb) {
      int I, J;
      tile_of(tile, I, J);
      __syncthreads();  // the previous tile's columns are no longer read
      // 32 columns of n values, warp w staging columns w, w + 8, ..: lane e
      // loads rows e, e + 32, .. (8 loads in flight per batch), no division
      for (int cc = tid >> 5; cc < 2 * PUR_TILE; cc += blockDim.x >> 5) {
        const int col = cc < PUR_TILE ? I * PUR_TILE + cc : J * PUR_TILE + cc - PUR_TILE;
        Col *dst = cols + (size_t)cc * ld;
        const double *src = X + N * col;
        for (int r0 = tid & 31; r0 < n; r0 += 8 * 32) {
          double v[8];
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            const int r = r0 + 32 * u;
            v[u] = (col < n && r < n) ? src[r] : 0.0;
          }
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            const int r = r0 + 32 * u;
            if (r < n) {
              if constexpr (F64) dst[r] = v[u];
              else dst[r] = split_f64(v[u]);
            }
          }
        }
      }
      __syncthreads();
      const int i = I * PUR_TILE + ti, j = J * PUR_TILE + tj;
      const double xij = (i < n && j < n) ? X[i + N * j] : 0.0;
      const Col *ci = cols + (size_t)ti * ld, *cj = cols + (size_t)(PUR_TILE + tj) * ld;
      double t;
      if constexpr (F64) {  // (X^2)_ij in FP64, four interleaved sums
        double t0 = 0.0, t1 = 0.0, t2 = 0.0, t3 = 0.0;
        int r = 0;
        for (; r + 3 < n; r += 4) {
          t0 = fma(ci[r], cj[r], t0);
          t1 = fma(ci[r + 1], cj[r + 1], t1);
          t2 = fma(ci[r + 2], cj[r + 2], t2);
          t3 = fma(ci[r + 3], cj[r + 3], t3);
        }
        for (; r < n; ++r) t0 = fma(ci[r], cj[r], t0);
        t = (t0 + t1) + (t2 + t3);
      } else {
        // (X^2)_ij in double-float on the FP32 pipes (about 2^-48 relative per
        // product), four interleaved sums
        float2 t0 = make_float2(0.f, 0.f), t1 = t0, t2 = t0, t3 = t0;
        int r = 0;
        for (; r + 3 < n; r += 4) {
          dfma(t0, ci[r], cj[r]);
          dfma(t1, ci[r + 1], cj[r + 1]);
          dfma(t2, ci[r + 2], cj[r + 2]);
          dfma(t3, ci[r + 3], cj[r + 3]);
        }
        for (; r < n; ++r) dfma(t0, ci[r], cj[r]);
        t = (df_val(t0) + df_val(t1)) + (df_val(t2) + df_val(t3));
      }
      double ptr = 0.0, psq = 0.0;
      if (i < n && j < n) {
        const double y = square ? t : 2.0 * xij - t;
        Y[i + N * j] = y;
        if (I != J) Y[j + N * i] = y;
        ptr = (i == j) ? y : 0.0;
        psq = (I == J ? 1.0 : 2.0) * y * y;
      }
      tile_partials(ptr, psq, red, pn, tile);
    }
    if (!grid_barrier(gs, nb)) return;
  }
  if (blockIdx.x == 0 && tid == 0) {
    info[0] = k;                 // steps taken; the result is X_k
    info[1] = settled_at >= 0;   // converged
  }
}

static int purify_persistent(mq_ctx *c, int n, int nocc, double *d_P, double *d_W, double *d_err, int *steps) {
  const size_t n2 = (size_t)n * n;
  const int nt = (n + PUR_TILE - 1) / PUR_TILE, ntiles = nt * (nt + 1) / 2;
  const size_t smem = (size_t)2 * PUR_TILE * (n | 1) * sizeof(double);
  const void *kfn = c->fock_df32 ? (const void *)purify_persist_kernel<false> : (const void *)purify_persist_kernel<true>;
  char *ws = (char *)buf(c, "purify_persist", 256 + 64 + sizeof(double) * 4 * ntiles);
  if (!ws) return MQ_ENOMEM;
  GridSync gs{(unsigned *)ws, (unsigned *)(ws + 64), (int *)(ws + 128)};
  int *info = (int *)(ws + 192);
  double *part = (double *)(ws + 320);
  MQ_CUDA(c, cudaMemsetAsync(ws, 0, 320, c->stream));
  MQ_CUDA(c, cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int sms = 0, per_sm = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
  MQ_CUDA(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kfn, 256, smem));
  if (per_sm < 1) return set_err(c, MQ_EINVAL, "purification kernel does not fit on an SM");
  // one tile per CTA where the tiles allow; every CTA must be resident
  int grid = std::min(ntiles, sms * per_sm);
  double *X0 = d_P, *X1 = d_W;
  double noccd = (double)nocc;
  void *args[] = {&n, &noccd, &X0, &X1, &part, &d_err, &info, &gs};
  MQ_CUDA(c, cudaLaunchCooperativeKernel(kfn, dim3(grid), dim3(256), args, smem,
                                         c->stream));
  c->stats.launches += 1;
  int h[2] = {0, 0}, berr[4] = {0, 0, 0, 0};
  MQ_CUDA(c, cudaMemcpyAsync(h, info, 2 * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  MQ_CUDA(c, cudaMemcpyAsync(berr, gs.err, sizeof(berr), cudaMemcpyDeviceToHost, c->stream));
  MQ_CUDA(c, cudaStreamSynchronize(c->stream));
  if (berr[0])
    return set_err(c, MQ_ETIMEOUT, "purification grid barrier timed out (" + std::to_string(berr[1]) +
                                       " arrivals counted of " + std::to_string(grid) + ", CTA " +
                                       std::to_string(berr[2]) + ", barrier " + std::to_string(berr[3]) + ")");
  *steps = h[0];
  if (!h[1]) return set_err(c, MQ_ENOCONV, "purification did not converge (no gap at the Fermi level?)");
  if (h[0] & 1) MQ_CUDA(c, cudaMemcpyAsync(d_P, d_W, n2 * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
  return MQ_OK;
}

int purify_projector(mq_ctx *c, int n, int nocc, const double *d_Fp, double *d_P, double *d_T, double *d_W,
                     double *d_err, int *steps) {
  const size_t n2 = (size_t)n * n;
  const unsigned gb = (unsigned)((n2 + 255) / 256);
  *steps = 0;
  if (nocc <= 0) {
    MQ_CUDA(c, cudaMemsetAsync(d_P, 0, n2 * sizeof(double), c->stream));
    return MQ_OK;
  }
  if (nocc >= n) {
    identity_kernel<<<gb, 256, 0, c->stream>>>(d_P, n);
    c->stats.launches += 1;
    MQ_CUDA(c, cudaGetLastError());
    return MQ_OK;
  }
  constexpr int MAX_STEPS = PUR_MAX_STEPS, POLL = 4;
  constexpr double SETTLED = PUR_SETTLED;  // idempotency error after which two more steps reach FP64 round-off
  double *X = d_P, *Xn = d_W;
  MQ_TRY(gershgorin(c, d_Fp, n, 1, d_err + PUR_MAX_STEPS));  // [lo, hi] after the step errors
  purify_build_kernel<<<gb, 256, 0, c->stream>>>(d_Fp, n, d_err + PUR_MAX_STEPS, X);
  c->stats.launches += 1;
  // the one-launch form waits at grid-wide barriers, so it runs only when
  // nothing else is in flight beside it (no slicing of the transform's
  // operands on the side stream); otherwise one product and one update
  // launch per step
  if (c->side_pending && cudaEventQuery(c->ev_side) == cudaSuccess) MQ_TRY(join_side(c));  // it has finished
  if (n <= PUR_PERSIST_MAX && !c->side_pending) {
    c->stats.purify_persistent += 1;
    return purify_persistent(c, n, nocc, d_P, d_W, d_err, steps);
  }
  c->stats.purify_stepwise += 1;
  std::vector<double> e(MAX_STEPS);
  int k = 0, settled_at = -1;
  while (k < MAX_STEPS) {
    MQ_TRY(syrk_lower(c, n, n, 1.0, X, n, 0.0, d_T, n));
    purify_step_kernel<<<std::min(gb, 1024u), 256, 0, c->stream>>>(X, d_T, n, (double)nocc, Xn, d_err, k);
    c->stats.launches += 1;
    std::swap(X, Xn);
    ++k;
    if (settled_at >= 0 && k >= settled_at + 2) break;
    if (settled_at < 0 && k % POLL == 0) {
      MQ_CUDA(c, cudaMemcpyAsync(e.data(), d_err, k * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
      MQ_CUDA(c, cudaStreamSynchronize(c->stream));
      for (int j = 0; j < k; ++j)
        if (std::fabs(e[j]) < SETTLED) {  // X_j nearly idempotent: X_{j+2} is at round-off
          settled_at = j;
          break;
        }
      if (settled_at >= 0 && k >= settled_at + 2) break;
    }
  }
  *steps = k;
  if (settled_at < 0) return set_err(c, MQ_ENOCONV, "purification did not converge (no gap at the Fermi level?)");
  if (X != d_P) MQ_CUDA(c, cudaMemcpyAsync(d_P, X, n2 * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
  return MQ_OK;
}

// ---- S^-1/2 by the coupled Newton-Schulz iteration (Higham, "Functions of
// Matrices", 2008, eq. 6.35): with Y_0 = S / c, Z_0 = I and
//   T_k = (3 I - Z_k Y_k) / 2,  Y_{k+1} = Y_k T_k,  Z_{k+1} = T_k Z_k,
// Y -> (S/c)^(1/2) and Z -> (S/c)^(-1/2) quadratically once the spectrum of
// Z Y is near 1; c >= lambda_max(S) (Gershgorin) keeps every eigenvalue of
// S/c in (0, 1].  X = Z / sqrt(c).  Three FP64 GEMMs per step, no eigensolver.

// T = 1.5 I - 0.5 A (A = Z Y); err[k] = ||I - A||_F^2 (block 0)
__global__ void ns_step_kernel(const double *__restrict__ A, int n, double *__restrict__ T, double *__restrict__ err,
                               int k) {
  __shared__ double red[32];
  const size_t N = n, n2 = N * N;
  double e = 0.0;
  for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n2; idx += (size_t)gridDim.x * blockDim.x) {
    const double d = (idx % (N + 1) == 0) ? 1.0 - A[idx] : -A[idx];
    e += d * d;
    T[idx] = 0.5 * d + ((idx % (N + 1) == 0) ? 1.0 : 0.0);
  }
  e = block_sum(e, red);
  if (threadIdx.x == 0) atomicAdd(err + k, e);
}

// Y = S / c with c = lohi[1] the largest row absolute sum of S (>= lambda_max);
// Z = I; scal[0] = c
__global__ void ns_build_kernel(const double *__restrict__ S, int n, const double *__restrict__ lohi,
                                double *__restrict__ Y, double *__restrict__ Z, double *__restrict__ scal) {
  const size_t N = n, idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= N * N) return;
  const double c = lohi[1];
  Y[idx] = S[idx] / c;
  Z[idx] = (idx % (N + 1) == 0) ? 1.0 : 0.0;
  if (idx == 0) scal[0] = c;
}

__global__ void scale_kernel(const double *__restrict__ A, size_t n2, const double *__restrict__ c,
                             double *__restrict__ out) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n2) out[i] = A[i] * rsqrt(c[0]);
}

int inv_sqrt_ns(mq_ctx *c, int n, const double *d_S, double *d_X, double *w, double *d_err, int *steps) {
  const size_t n2 = (size_t)n * n;
  double *Y = w, *Z = w + n2, *T = w + 2 * n2, *A = w + 3 * n2, *Y2 = w + 4 * n2;
  constexpr int MAX_STEPS = 100, POLL = 4;
  const unsigned gb = (unsigned)std::min<size_t>((n2 + 255) / 256, 1024);
  MQ_CUDA(c, cudaMemsetAsync(d_err, 0, (MAX_STEPS + 1) * sizeof(double), c->stream));
  double *lohi = (double *)buf(c, "ns_lohi", 2 * sizeof(double));
  if (!lohi) return MQ_ENOMEM;
  MQ_TRY(gershgorin(c, d_S, n, 0, lohi));
  ns_build_kernel<<<(unsigned)((n2 + 255) / 256), 256, 0, c->stream>>>(d_S, n, lohi, Y, Z, d_err + MAX_STEPS);
  c->stats.launches += 1;
  std::vector<double> e(MAX_STEPS);
  int k = 0, done_at = -1;
  while (k < MAX_STEPS) {
    MQ_TRY(gemm(c, 'N', 'N', n, n, n, 1.0, Z, n, Y, n, 0.0, A, n));
    ns_step_kernel<<<gb, 256, 0, c->stream>>>(A, n, T, d_err, k);
    c->stats.launches += 1;
    MQ_TRY(gemm(c, 'N', 'N', n, n, n, 1.0, Y, n, T, n, 0.0, Y2, n));
    MQ_TRY(gemm(c, 'N', 'N', n, n, n, 1.0, T, n, Z, n, 0.0, A, n));
    std::swap(Y, Y2);
    std::swap(Z, A);  // A is scratch again
    ++k;
    if (done_at >= 0 && k >= done_at + 2) break;
    if (done_at < 0 && k % POLL == 0) {
      MQ_CUDA(c, cudaMemcpyAsync(e.data(), d_err, k * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
      MQ_CUDA(c, cudaStreamSynchronize(c->stream));
      for (int j = 0; j < k; ++j)
        if (e[j] < 1e-16 * n) {  // ||I - Z_j Y_j|| ~ 1e-8: two more steps reach round-off
          done_at = j;
          break;
        }
      if (done_at >= 0 && k >= done_at + 2) break;
    }
  }
  *steps = k;
  if (done_at < 0) return set_err(c, MQ_ENOCONV, "Newton-Schulz S^-1/2 did not converge");
  scale_kernel<<<(unsigned)((n2 + 255) / 256), 256, 0, c->stream>>>(Z, n2, d_err + MAX_STEPS, d_X);
  c->stats.launches += 1;
  MQ_CUDA(c, cudaGetLastError());
  return MQ_OK;
}

}  // namespace mq
