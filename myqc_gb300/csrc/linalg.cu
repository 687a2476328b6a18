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

#include <string>

#include "internal.h"
#include "gridsync.cuh"
#include "jacobi.cuh"

namespace mq {

constexpr int JAC_THREADS = 512;

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
  __shared__ int flag;
  for (size_t idx = threadIdx.x; idx < n2; idx += blockDim.x) A[idx] = Ain[idx];
  __syncthreads();
  const bool ok = jacobi_block(n, A, V, cs, red, &flag, max_sweeps, tol);
  if (threadIdx.x == 0 && !ok) atomicExch(status, 1);
  jacobi_sorted_out(n, A, V, wg + (size_t)n * b, Vg + n2 * b);
}

// ---------------------------------------------------------------------------
// Multi-CTA Jacobi for one large matrix (n > JAC_SMEM_MAX).  Each round of the
// tournament applies A <- J^T A J as independent 2x2 block transforms
// A[P,Q] <- J_P^T A[P,Q] J_Q over index pairs P >= Q (the mirror block is the
// transpose), and V <- V J row by row; no element is touched by two threads,
// so a round needs a single grid barrier.  Every CTA recomputes the round's
// rotation angles from the diagonal it reads after the barrier.  The barrier
// (gridsync.cuh) raises an error flag on time-out and every CTA leaves.
// Launched cooperatively so that all CTAs are resident.
constexpr int JG_THREADS = 256;
__global__ void __launch_bounds__(JG_THREADS) jacobi_grid_kernel(int n, double *__restrict__ A,
                                                                  double *__restrict__ V, double *__restrict__ w,
                                                                  double *__restrict__ Vout, double *part,
                                                                  GridSync gs, int max_sweeps, double tol,
                                                                  int *__restrict__ info) {
  __shared__ double cs[2 * 512];
  __shared__ double red[JG_THREADS / 32];
  const int np = n + (n & 1), half = np / 2;
  const unsigned nb = gridDim.x;
  const int tid = threadIdx.x;
  const long long gtid = (long long)blockIdx.x * blockDim.x + tid, gstride = (long long)nb * blockDim.x;
  const size_t N = n;
  // ||A||_F^2
  auto reduce_store = [&](double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((tid & 31) == 0) red[tid >> 5] = v;
    __syncthreads();
    if (tid == 0) {
      double t = 0;
      for (int k = 0; k < JG_THREADS / 32; ++k) t += red[k];
      part[blockIdx.x] = t;
    }
  };
  auto reduce_all = [&]() {
    double t = 0;
    for (unsigned k = 0; k < nb; ++k) t += ((volatile double *)part)[k];
    return t;
  };
  {
    double f = 0;
    for (long long i = gtid; i < (long long)N * N; i += gstride) f += A[i] * A[i];
    reduce_store(f);
  }
  if (!grid_barrier(gs, nb)) return;
  const double stop2 = tol * tol * reduce_all();
  const double skip = sqrt(stop2) / n;
  if (!grid_barrier(gs, nb)) return;
  int sweep = 0;
  for (; sweep < max_sweeps; ++sweep) {
    double off = 0;
    for (long long i = gtid; i < (long long)N * N; i += gstride) {
      const int r = (int)(i % n), col = (int)(i / n);
      if (r != col) off += A[i] * A[i];
    }
    reduce_store(off);
    if (!grid_barrier(gs, nb)) return;
    const bool done = reduce_all() <= stop2;
    if (!grid_barrier(gs, nb)) return;  // everyone has read part[] before it is rewritten
    if (done) break;
    for (int r = 0; r < np - 1; ++r) {
      int active = 0;
      for (int k = tid; k < half; k += blockDim.x) {
        int p, q;
        rr_pair(np, r, k, p, q);
        double c = 1.0, s = 0.0;
        if (q < n) {
          const double apq = A[p + N * q];
          const double app = A[p + N * p], aqq = A[q + N * q];
          // negligible rotations are skipped: below 2^-60 of the diagonal, or
          // below skip = tol ||A||_F / n (all such pairs together stay under
          // the stopping threshold)
          if (fabs(apq) > fmax(0x1p-60 * (fabs(app) + fabs(aqq)), skip)) {
            const double theta = (aqq - app) / (2.0 * apq);
            const double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
            c = rsqrt(t * t + 1.0);
            s = t * c;
            active = 1;
          }
        }
        cs[2 * k] = c;
        cs[2 * k + 1] = s;
      }
      // every CTA reads the same A, so all skip a round without rotations
      // together, barrier included
      if (!__syncthreads_or(active)) continue;
      // blocks (P, Q) with P >= Q, and V rows
      const long long nblk = (long long)half * (half + 1) / 2;
      for (long long idx = gtid; idx < nblk + (long long)N * half; idx += gstride) {
        if (idx < nblk) {
          int P = (int)((sqrt(8.0 * (double)idx + 1.0) - 1.0) * 0.5);
          while ((long long)P * (P + 1) / 2 > idx) --P;
          while ((long long)(P + 1) * (P + 2) / 2 <= idx) ++P;
          const int Q = (int)(idx - (long long)P * (P + 1) / 2);
          int p, q, u, v;
          rr_pair(np, r, P, p, q);
          rr_pair(np, r, Q, u, v);
          const double cP = cs[2 * P], sP = cs[2 * P + 1], cQ = cs[2 * Q], sQ = cs[2 * Q + 1];
          const bool qv = q < n, vv = v < n;
          if (P == Q) {
            if (!qv) continue;
            const double app = A[p + N * p], aqq = A[q + N * q], apq = A[p + N * q];
            // diagonalised 2x2 block
            A[p + N * p] = cP * cP * app - 2 * cP * sP * apq + sP * sP * aqq;
            A[q + N * q] = sP * sP * app + 2 * cP * sP * apq + cP * cP * aqq;
            A[p + N * q] = 0.0;
            A[q + N * p] = 0.0;
            continue;
          }
          // rows {p,q} x cols {u,v}
          const double a_pu = A[p + N * u], a_qu = qv ? A[q + N * u] : 0.0;
          const double a_pv = vv ? A[p + N * v] : 0.0, a_qv = (qv && vv) ? A[q + N * v] : 0.0;
          // J_P^T (rows)
          const double b_pu = cP * a_pu - sP * a_qu, b_qu = sP * a_pu + cP * a_qu;
          const double b_pv = cP * a_pv - sP * a_qv, b_qv = sP * a_pv + cP * a_qv;
          // J_Q (columns)
          const double n_pu = cQ * b_pu - sQ * b_pv, n_pv = sQ * b_pu + cQ * b_pv;
          const double n_qu = cQ * b_qu - sQ * b_qv, n_qv = sQ * b_qu + cQ * b_qv;
          A[p + N * u] = n_pu;
          A[u + N * p] = n_pu;
          if (qv) {
            A[q + N * u] = n_qu;
            A[u + N * q] = n_qu;
          }
          if (vv) {
            A[p + N * v] = n_pv;
            A[v + N * p] = n_pv;
          }
          if (qv && vv) {
            A[q + N * v] = n_qv;
            A[v + N * q] = n_qv;
          }
        } else {
          const long long t = idx - nblk;
          const int i = (int)(t % n), K = (int)(t / n);
          int p, q;
          rr_pair(np, r, K, p, q);
          if (q >= n) continue;
          const double c = cs[2 * K], s = cs[2 * K + 1];
          const double x = V[i + N * p], y = V[i + N * q];
          V[i + N * p] = c * x - s * y;
          V[i + N * q] = s * x + c * y;
        }
      }
      if (!grid_barrier(gs, nb)) return;
    }
  }
  if (sweep >= max_sweeps && blockIdx.x == 0 && tid == 0) atomicExch(gs.err, 1);
  if (blockIdx.x == 0 && tid == 0) info[0] = sweep;
  // sorted output: each global thread ranks one eigenvalue
  for (long long i = gtid; i < n; i += gstride) {
    const double wi = A[i + N * i];
    int rank = 0;
    for (int j = 0; j < n; ++j) {
      const double wj = A[j + N * j];
      rank += (wj < wi) || (wj == wi && j < i);
    }
    w[rank] = wi;
    double big = 0.0;
    for (int k = 0; k < n; ++k)
      if (fabs(V[k + N * i]) > fabs(big)) big = V[k + N * i];
    const double sg = big < 0 ? -1.0 : 1.0;
    for (int k = 0; k < n; ++k) Vout[k + N * rank] = sg * V[k + N * i];
  }
}

__global__ void set_identity_kernel(double *V, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) V[i + (size_t)n * i] = 1.0;
}

// One large matrix: A (n x n, device, overwritten), optional start vectors V0
// (A must then already be V0^T A V0), eigenvalues w, eigenvectors Vout.
int syev_large_device(mq_ctx *c, int n, double *d_A, const double *d_V0, double *d_w, double *d_V, bool async) {
  const size_t n2 = (size_t)n * n;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
  int per_sm = 0;
  MQ_CUDA(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, jacobi_grid_kernel, JG_THREADS, 0));
  const int half = (n + 1) / 2;
  int nblocks = std::min(sms * std::max(per_sm, 1), std::max(1, (half * (half + 1) / 2 + JG_THREADS - 1) / JG_THREADS));
  nblocks = std::max(1, std::min(nblocks, sms));
  char *ws = (char *)buf(c, "jacobi_grid", 256 + sizeof(double) * (n2 + nblocks));
  if (!ws) return MQ_ENOMEM;
  GridSync gs{(unsigned *)ws, (unsigned *)(ws + 64), (int *)(ws + 128)};
  double *V = (double *)(ws + 256), *part = V + n2;
  MQ_CUDA(c, cudaMemsetAsync(ws, 0, 256, c->stream));
  if (d_V0) {
    MQ_CUDA(c, cudaMemcpyAsync(V, d_V0, n2 * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
  } else {
    MQ_CUDA(c, cudaMemsetAsync(V, 0, n2 * sizeof(double), c->stream));
    set_identity_kernel<<<(n + 255) / 256, 256, 0, c->stream>>>(V, n);
  }
  int max_sweeps = 40;
  double tol = 1e-14;  // ||offdiag||_F / ||A||_F at stop; eigenvalue error ~ tol^2 ||A|| / gap
  int *info = (int *)(ws + 192);
  void *args[] = {&n, &d_A, &V, &d_w, &d_V, &part, &gs, &max_sweeps, &tol, &info};
  // every CTA of a grid-barrier kernel must be resident at once: nothing of
  // the side stream (the transform's XX slicing) runs beside it
  if (c->stream != c->side) MQ_TRY(join_side(c));
  MQ_CUDA(c, cudaLaunchCooperativeKernel((void *)jacobi_grid_kernel, dim3(nblocks), dim3(JG_THREADS), args, 0,
                                         c->stream));
  c->stats.launches += 2;
  if (async) return MQ_OK;
  return syev_large_status(c);
}

int syev_large_status(mq_ctx *c) {
  auto it = c->bufs.find("jacobi_grid");
  if (it == c->bufs.end() || !it->second.ptr) return MQ_OK;  // no grid solve ran
  const char *ws = (const char *)it->second.ptr;
  int h[4] = {0, 0, 0, 0}, sw = 0;
  MQ_CUDA(c, cudaMemcpyAsync(h, ws + 128, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  MQ_CUDA(c, cudaMemcpyAsync(&sw, ws + 192, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  MQ_CUDA(c, cudaStreamSynchronize(c->stream));
  c->stats.eig_jacobi_sweeps = sw;
  if (h[0] == 2)
    return set_err(c, MQ_ETIMEOUT, "Jacobi grid barrier timed out (" + std::to_string(h[1]) + " arrivals counted, CTA " +
                                       std::to_string(h[2]) + ", barrier " + std::to_string(h[3]) + ", sweeps " +
                                       std::to_string(sw) + ")");
  if (h[0] == 1) return set_err(c, MQ_ENOCONV, "Jacobi eigensolver did not converge");
  return MQ_OK;
}

int syev_batched_device(mq_ctx *c, int n, int batch, double *d_A, double *d_w, double *d_V) {
  if (n <= 0 || batch <= 0) return set_err(c, MQ_EINVAL, "syev: bad size");
  if (n > 1024) return set_err(c, MQ_EINVAL, "syev: n > 1024");
  const size_t n2 = (size_t)n * n;
  if (n > JAC_SMEM_MAX) {
    for (int b = 0; b < batch; ++b) MQ_TRY(syev_large_cold(c, n, d_A + n2 * b, d_w + (size_t)n * b, d_V + n2 * b));
    return MQ_OK;
  }
  const size_t smem = 2 * n2 * sizeof(double);
  int *status = (int *)buf(c, "jacobi_work", 64 + (smem > 200 * 1024 ? 2 * n2 * sizeof(double) * batch : 0));
  if (!status) return MQ_ENOMEM;
  MQ_CUDA(c, cudaMemsetAsync(status, 0, sizeof(int), c->stream));
  const int max_sweeps = 60;
  const double tol = 1e-14;  // ||offdiag||_F / ||A||_F at stop; eigenvalue error ~ tol^2 ||A|| / gap
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

int gemm(mq_ctx *c, char ta, char tb, int m, int n, int k, double alpha, const double *A, int lda, const double *B,
         int ldb, double beta, double *C, int ldc) {
  return dgemm_batched(c, ta, tb, m, n, k, alpha, A, lda, 0, B, ldb, 0, beta, C, ldc, 0, 1);
}

// lower triangle of C = alpha A A^T + beta C (n x n, A n x k); the product
// forms the whole of C (the upper triangle gets the same values)
int syrk_lower(mq_ctx *c, int n, int k, double alpha, const double *A, int lda, double beta, double *C, int ldc) {
  return dgemm_batched(c, 'N', 'T', n, n, k, alpha, A, lda, 0, A, lda, 0, beta, C, ldc, 0, 1);
}

int gemm_strided_batched(mq_ctx *c, char ta, char tb, int m, int n, int k, double alpha, const double *A, int lda,
                         long long sA, const double *B, int ldb, long long sB, double beta, double *C, int ldc,
                         long long sC, int batch) {
  return dgemm_batched(c, ta, tb, m, n, k, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, batch);
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
