// linalg.cu -- FP64 dense kernels for the SCF: batched cyclic Jacobi
// eigensolver (replaces LAPACK DSYEV/DSYGV's eigen step, src/scf/scf.f90:692,
// 478, 848), density matrix (src/dens/dens.f90:115-124, 213-228), and GEMM
// wrappers (plain library GEMMs go to cuBLAS).
//
// Jacobi: one CTA per matrix.  Each sweep runs the n'-1 rounds of a
// round-robin tournament (n' = n rounded up to even); a round rotates n'/2
// disjoint index pairs at once: rotation angles, then rows, then columns of
// A and V, with a block barrier between phases.  The matrix and the
// eigenvectors live in shared memory when 2 n^2 doubles fit, else in a
// global workspace.  Converges when the off-diagonal Frobenius norm falls
// below tol * ||A||_F; the result is sorted ascending.
#include <cublas_v2.h>

#include "internal.h"

namespace mq {

constexpr int JAC_THREADS = 512;

__device__ __forceinline__ void rr_pair(int np, int r, int k, int &p, int &q) {
  // circle method: player 0 fixed, players 1..np-1 rotate
  const int m = np - 1;
  if (k == 0) {
    p = 0;
    q = 1 + (r % m);
  } else {
    p = 1 + (r + k) % m;
    q = 1 + (r - k + m) % m;
  }
  if (p > q) {
    int t = p;
    p = q;
    q = t;
  }
}

template <bool SMEM>
__global__ void __launch_bounds__(JAC_THREADS) jacobi_kernel(int n, double *__restrict__ Ag, double *__restrict__ wg,
                                                             double *__restrict__ Vg, double *__restrict__ work,
                                                             int max_sweeps, double tol, int *__restrict__ status) {
  extern __shared__ double sm[];
  const int b = blockIdx.x;
  const size_t n2 = (size_t)n * n;
  double *Ain = Ag + n2 * b;
  double *A, *V;
  if (SMEM) {
    A = sm;
    V = sm + n2;
  } else {
    A = work + 2 * n2 * b;
    V = A + n2;
  }
  __shared__ double cs[2 * 512];  // (c, s) per pair of a round, n <= 1024
  __shared__ double red[JAC_THREADS / 32];
  __shared__ int done;
  const int tid = threadIdx.x;
  for (size_t idx = tid; idx < n2; idx += blockDim.x) {
    A[idx] = Ain[idx];
    V[idx] = (idx % (n + 1) == 0) ? 1.0 : 0.0;
  }
  __syncthreads();
  // ||A||_F for the stopping rule
  double fro = 0.0;
  for (size_t idx = tid; idx < n2; idx += blockDim.x) fro += A[idx] * A[idx];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) fro += __shfl_xor_sync(0xffffffffu, fro, o);
  if ((tid & 31) == 0) red[tid >> 5] = fro;
  __syncthreads();
  if (tid == 0) {
    double t = 0;
    for (int w = 0; w < JAC_THREADS / 32; ++w) t += red[w];
    red[0] = t;
    done = 0;
  }
  __syncthreads();
  const double stop2 = tol * tol * red[0];
  __syncthreads();
  const int np = n + (n & 1), half = np / 2;
  int sweep = 0;
  for (; sweep < max_sweeps; ++sweep) {
    // off-diagonal norm
    double off = 0.0;
    for (size_t idx = tid; idx < n2; idx += blockDim.x) {
      const int i = (int)(idx % n), j = (int)(idx / n);
      if (i != j) off += A[idx] * A[idx];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) off += __shfl_xor_sync(0xffffffffu, off, o);
    __syncthreads();
    if ((tid & 31) == 0) red[tid >> 5] = off;
    __syncthreads();
    if (tid == 0) {
      double t = 0;
      for (int w = 0; w < JAC_THREADS / 32; ++w) t += red[w];
      done = (t <= stop2);
    }
    __syncthreads();
    if (done) break;
    for (int r = 0; r < np - 1; ++r) {
      // 1) rotation angles
      for (int k = tid; k < half; k += blockDim.x) {
        int p, q;
        rr_pair(np, r, k, p, q);
        double c = 1.0, s = 0.0;
        if (q < n) {
          const double apq = A[p + (size_t)n * q];
          if (apq != 0.0) {
            const double app = A[p + (size_t)n * p], aqq = A[q + (size_t)n * q];
            const double theta = (aqq - app) / (2.0 * apq);
            const double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
            c = rsqrt(t * t + 1.0);
            s = t * c;
          }
        }
        cs[2 * k] = c;
        cs[2 * k + 1] = s;
      }
      __syncthreads();
      // 2) rows p, q of A:  A <- J^T A
      for (int idx = tid; idx < half * n; idx += blockDim.x) {
        const int k = idx / n, j = idx % n;
        int p, q;
        rr_pair(np, r, k, p, q);
        if (q >= n) continue;
        const double c = cs[2 * k], s = cs[2 * k + 1];
        if (s == 0.0) continue;
        const double ap = A[p + (size_t)n * j], aq = A[q + (size_t)n * j];
        A[p + (size_t)n * j] = c * ap - s * aq;
        A[q + (size_t)n * j] = s * ap + c * aq;
      }
      __syncthreads();
      // 3) columns p, q of A and V:  A <- A J, V <- V J
      for (int idx = tid; idx < half * n; idx += blockDim.x) {
        const int k = idx / n, i = idx % n;
        int p, q;
        rr_pair(np, r, k, p, q);
        if (q >= n) continue;
        const double c = cs[2 * k], s = cs[2 * k + 1];
        if (s == 0.0) continue;
        double *ap = A + (size_t)n * p, *aq = A + (size_t)n * q;
        const double x = ap[i], y = aq[i];
        ap[i] = c * x - s * y;
        aq[i] = s * x + c * y;
        double *vp = V + (size_t)n * p, *vq = V + (size_t)n * q;
        const double vx = vp[i], vy = vq[i];
        vp[i] = c * vx - s * vy;
        vq[i] = s * vx + c * vy;
      }
      __syncthreads();
    }
  }
  if (tid == 0 && sweep >= max_sweeps) atomicExch(status, 1);
  // sort ascending: rank of each eigenvalue, ties broken by index
  for (int i = tid; i < n; i += blockDim.x) {
    const double wi = A[i + (size_t)n * i];
    int rank = 0;
    for (int j = 0; j < n; ++j) {
      const double wj = A[j + (size_t)n * j];
      rank += (wj < wi) || (wj == wi && j < i);
    }
    wg[(size_t)n * b + rank] = wi;
    // eigenvector i -> column rank, sign fixed so the largest component is positive
    double big = 0.0;
    for (int k = 0; k < n; ++k)
      if (fabs(V[k + (size_t)n * i]) > fabs(big)) big = V[k + (size_t)n * i];
    const double sg = big < 0 ? -1.0 : 1.0;
    for (int k = 0; k < n; ++k) Vg[n2 * b + k + (size_t)n * rank] = sg * V[k + (size_t)n * i];
  }
}

int syev_batched_device(mq_ctx *c, int n, int batch, double *d_A, double *d_w, double *d_V) {
  if (n <= 0 || batch <= 0) return set_err(c, MQ_EINVAL, "syev: bad size");
  if (n > 1024) return set_err(c, MQ_EINVAL, "syev: n > 1024");
  const size_t n2 = (size_t)n * n;
  const size_t smem = 2 * n2 * sizeof(double);
  int *status = (int *)buf(c, "jacobi_work", 64 + (smem > 200 * 1024 ? 2 * n2 * sizeof(double) * batch : 0));
  if (!status) return MQ_ENOMEM;
  MQ_CUDA(c, cudaMemsetAsync(status, 0, sizeof(int), c->stream));
  const int max_sweeps = 60;
  const double tol = 1e-15;
  if (smem <= 200 * 1024) {
    MQ_CUDA(c, cudaFuncSetAttribute(jacobi_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    jacobi_kernel<true><<<batch, JAC_THREADS, smem, c->stream>>>(n, d_A, d_w, d_V, nullptr, max_sweeps, tol, status);
  } else {
    double *work = (double *)((char *)status + 64);
    jacobi_kernel<false><<<batch, JAC_THREADS, 0, c->stream>>>(n, d_A, d_w, d_V, work, max_sweeps, tol, status);
  }
  c->stats.launches += 1;
  MQ_CUDA(c, cudaGetLastError());
  int h = 0;
  MQ_CUDA(c, cudaMemcpyAsync(&h, status, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  MQ_CUDA(c, cudaStreamSynchronize(c->stream));
  if (h) return set_err(c, MQ_ENOCONV, "Jacobi eigensolver did not converge");
  return MQ_OK;
}

static cublasHandle_t handle(mq_ctx *c) {
  if (!c->cublas) {
    cublasHandle_t h;
    if (cublasCreate(&h) != CUBLAS_STATUS_SUCCESS) return nullptr;
    c->cublas = h;
  }
  cublasHandle_t h = (cublasHandle_t)c->cublas;
  cublasSetStream(h, c->stream);
  return h;
}

void cublas_destroy(void *h) { cublasDestroy((cublasHandle_t)h); }

static cublasOperation_t op(char t) { return (t == 'T' || t == 't') ? CUBLAS_OP_T : CUBLAS_OP_N; }

int gemm(mq_ctx *c, char ta, char tb, int m, int n, int k, double alpha, const double *A, int lda, const double *B,
         int ldb, double beta, double *C, int ldc) {
  cublasHandle_t h = handle(c);
  if (!h) return set_err(c, MQ_ECUDA, "cublasCreate failed");
  if (cublasDgemm(h, op(ta), op(tb), m, n, k, &alpha, A, lda, B, ldb, &beta, C, ldc) != CUBLAS_STATUS_SUCCESS)
    return set_err(c, MQ_ECUDA, "cublasDgemm failed");
  c->stats.launches += 1;
  return MQ_OK;
}

int gemm_strided_batched(mq_ctx *c, char ta, char tb, int m, int n, int k, double alpha, const double *A, int lda,
                         long long sA, const double *B, int ldb, long long sB, double beta, double *C, int ldc,
                         long long sC, int batch) {
  cublasHandle_t h = handle(c);
  if (!h) return set_err(c, MQ_ECUDA, "cublasCreate failed");
  if (cublasDgemmStridedBatched(h, op(ta), op(tb), m, n, k, &alpha, A, lda, sA, B, ldb, sB, &beta, C, ldc, sC,
                                batch) != CUBLAS_STATUS_SUCCESS)
    return set_err(c, MQ_ECUDA, "cublasDgemmStridedBatched failed");
  c->stats.launches += 1;
  return MQ_OK;
}

// D = factor * C(:, 0:nocc-1) C(:, 0:nocc-1)^T, the sums of dens.f90:115-124
int density_device(mq_ctx *c, int n, int nocc, const double *d_C, double factor, double *d_D) {
  if (nocc <= 0) {
    MQ_CUDA(c, cudaMemsetAsync(d_D, 0, sizeof(double) * n * n, c->stream));
    return MQ_OK;
  }
  return gemm(c, 'N', 'T', n, n, nocc, factor, d_C, n, d_C, n, 0.0, d_D, n);
}

}  // namespace mq
