// dgemm.cu -- every FP64 GEMM of the library: C = alpha op(A) op(B) + beta C,
// column-major, as BLAS DGEMM, optionally strided-batched (blockIdx.z).
//
// FP64 throughput per SM is low on this GPU (2 fma per clock per SM), so a
// tile that keeps the FP64 pipe fed is enough: 32x32 output tiles, each CTA
// staging 32x16 slices of op(A) and op(B) in shared memory and forming a 2x2
// block per thread (4 fma per 4 shared loads).  A product of order ~200 is
// bound by how many SMs share it, so the K range is split until tiles x
// splits covers the SMs; the partial tiles go to a workspace and a second
// kernel adds them in split order (deterministic) and applies alpha and beta.
// Large products (the FP64 four-index transform's n^3 x n steps) have tiles
// enough without a split.
#include <algorithm>

#include "internal.h"

namespace mq {

constexpr int GB_M = 32, GB_N = 32, GB_K = 16, GB_THREADS = 256;

template <bool TA, bool TB>
__global__ void __launch_bounds__(GB_THREADS) dgemm_small_kernel(int m, int n, int k, int kchunk, double alpha,
                                                                 const double *__restrict__ A, int lda, long long sA,
                                                                 const double *__restrict__ B, int ldb, long long sB,
                                                                 double beta, double *__restrict__ C, int ldc,
                                                                 long long sC, double *__restrict__ W) {
  __shared__ double As[GB_K][GB_M + 1];  // As[kk][i] = op(A)(i, kb + kk)
  __shared__ double Bs[GB_K][GB_N + 1];  // Bs[kk][j] = op(B)(kb + kk, j)
  const int tiles_m = (m + GB_M - 1) / GB_M;
  const int bm = blockIdx.x % tiles_m, bn = blockIdx.x / tiles_m, s = blockIdx.y;
  A += sA * blockIdx.z;  // the batch's operands
  B += sB * blockIdx.z;
  C += sC * blockIdx.z;
  const int k0 = s * kchunk, k1 = min(k, k0 + kchunk);
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  double acc00 = 0.0, acc01 = 0.0, acc10 = 0.0, acc11 = 0.0;
  for (int kb = k0; kb < k1; kb += GB_K) {
    for (int e = threadIdx.x; e < GB_M * GB_K; e += GB_THREADS) {
      int i, kk;
      if (TA) {
        kk = e % GB_K;
        i = e / GB_K;
      } else {
        i = e % GB_M;
        kk = e / GB_M;
      }
      const int gi = bm * GB_M + i, gk = kb + kk;
      double v = 0.0;
      if (gi < m && gk < k1) v = TA ? A[gk + (size_t)lda * gi] : A[gi + (size_t)lda * gk];
      As[kk][i] = v;
    }
    for (int e = threadIdx.x; e < GB_N * GB_K; e += GB_THREADS) {
      int j, kk;
      if (TB) {
        j = e % GB_N;
        kk = e / GB_N;
      } else {
        kk = e % GB_K;
        j = e / GB_K;
      }
      const int gj = bn * GB_N + j, gk = kb + kk;
      double v = 0.0;
      if (gj < n && gk < k1) v = TB ? B[gj + (size_t)ldb * gk] : B[gk + (size_t)ldb * gj];
      Bs[kk][j] = v;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < GB_K; ++kk) {
      const double a0 = As[kk][tx], a1 = As[kk][tx + 16];
      const double b0 = Bs[kk][ty], b1 = Bs[kk][ty + 16];
      acc00 = fma(a0, b0, acc00);
      acc01 = fma(a0, b1, acc01);
      acc10 = fma(a1, b0, acc10);
      acc11 = fma(a1, b1, acc11);
    }
    __syncthreads();
  }
  const double acc[2][2] = {{acc00, acc01}, {acc10, acc11}};
#pragma unroll
  for (int a = 0; a < 2; ++a)
#pragma unroll
    for (int b = 0; b < 2; ++b) {
      const int gi = bm * GB_M + tx + 16 * a, gj = bn * GB_N + ty + 16 * b;
      if (gi >= m || gj >= n) continue;
      if (W) {
        W[(size_t)s * m * n + gi + (size_t)m * gj] = acc[a][b];
      } else {
        double *cp = C + gi + (size_t)ldc * gj;
        *cp = beta == 0.0 ? alpha * acc[a][b] : fma(alpha, acc[a][b], beta * *cp);
      }
    }
}

// C = alpha sum_s W[s] + beta C, splits added in order
__global__ void dgemm_reduce_kernel(int m, int n, int splits, double alpha, const double *__restrict__ W,
                                    double beta, double *__restrict__ C, int ldc) {
  const size_t mn = (size_t)m * n;
  for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < mn; idx += (size_t)gridDim.x * blockDim.x) {
    double t = W[idx];
    for (int s = 1; s < splits; ++s) t += W[s * mn + idx];
    const size_t i = idx % m, j = idx / m;
    double *cp = C + i + (size_t)ldc * j;
    *cp = beta == 0.0 ? alpha * t : fma(alpha, t, beta * *cp);
  }
}

bool dgemm_small_fits(int m, int n, int k) {
  return m > 0 && n > 0 && k > 0 && (long long)m * n <= (1 << 20) && (long long)m * n * k <= (1ll << 31);
}

int dgemm_small(mq_ctx *c, char ta, char tb, int m, int n, int k, double alpha, const double *A, int lda,
                const double *B, int ldb, double beta, double *C, int ldc) {
  return dgemm_batched(c, ta, tb, m, n, k, alpha, A, lda, 0, B, ldb, 0, beta, C, ldc, 0, 1);
}

int dgemm_batched(mq_ctx *c, char ta, char tb, int m, int n, int k, double alpha, const double *A, int lda,
                  long long sA, const double *B, int ldb, long long sB, double beta, double *C, int ldc,
                  long long sC, int batch) {
  if (m <= 0 || n <= 0 || batch <= 0) return MQ_OK;
  if (batch > 65535) return set_err(c, MQ_EINVAL, "dgemm: more than 65535 batched products");
  const bool TA = ta == 'T' || ta == 't', TB = tb == 'T' || tb == 't';
  int sms = 148;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
  const long long tiles_ll = (long long)((m + GB_M - 1) / GB_M) * ((n + GB_N - 1) / GB_N);
  if (tiles_ll > 2147483647LL) return set_err(c, MQ_EINVAL, "dgemm: too many output tiles");
  const int tiles = (int)tiles_ll;
  const int kblocks = std::max(1, (k + GB_K - 1) / GB_K);
  // K split only for a single product whose tiles do not cover the SMs
  int splits = batch > 1 ? 1 : std::max(1, std::min(kblocks, (int)((sms + tiles / 2) / std::max(tiles, 1))));
  const int kchunk = (kblocks + splits - 1) / splits * GB_K;
  splits = std::max(1, (k + kchunk - 1) / kchunk);
  double *W = nullptr;
  if (splits > 1) {
    // products queued on the aux stream (an eigensolve overlapping the SCF)
    // keep their own partial sums
    W = (double *)buf(c, c->aux && c->stream == c->aux ? "dgemm_split_aux" : "dgemm_split",
                      (size_t)splits * m * n * sizeof(double));
    if (!W) return MQ_ENOMEM;
  }
  const dim3 grid(tiles, splits, batch);
  if (TA && TB)
    dgemm_small_kernel<true, true><<<grid, GB_THREADS, 0, c->stream>>>(m, n, k, kchunk, alpha, A, lda, sA, B, ldb, sB,
                                                                       beta, C, ldc, sC, W);
  else if (TA)
    dgemm_small_kernel<true, false><<<grid, GB_THREADS, 0, c->stream>>>(m, n, k, kchunk, alpha, A, lda, sA, B, ldb,
                                                                        sB, beta, C, ldc, sC, W);
  else if (TB)
    dgemm_small_kernel<false, true><<<grid, GB_THREADS, 0, c->stream>>>(m, n, k, kchunk, alpha, A, lda, sA, B, ldb,
                                                                        sB, beta, C, ldc, sC, W);
  else
    dgemm_small_kernel<false, false><<<grid, GB_THREADS, 0, c->stream>>>(m, n, k, kchunk, alpha, A, lda, sA, B, ldb,
                                                                         sB, beta, C, ldc, sC, W);
  c->stats.launches += 1;
  if (splits > 1) {
    const size_t mn = (size_t)m * n;
    dgemm_reduce_kernel<<<(unsigned)std::min<size_t>((mn + 255) / 256, 1024), 256, 0, c->stream>>>(
        m, n, splits, alpha, W, beta, C, ldc);
    c->stats.launches += 1;
  }
  MQ_CUDA(c, cudaGetLastError());
  return MQ_OK;
}

}  // namespace mq
