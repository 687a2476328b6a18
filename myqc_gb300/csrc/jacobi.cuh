// jacobi.cuh -- one-CTA cyclic Jacobi eigensolver for a symmetric matrix, as
// device routines shared by the batched eigensolver kernel (linalg.cu) and the
// per-molecule SCF kernels of the batch engine (batch.cu).
//
// Each sweep runs the n'-1 rounds of a round-robin tournament (n' = n rounded
// up to even); a round rotates n'/2 disjoint index pairs at once: rotation
// angles, then rows, then columns of A and V, with a block barrier between
// phases.  Converges when the off-diagonal Frobenius norm falls below
// tol * ||A||_F.  Replaces the eigen step of DSYEV/DSYGV (src/scf/scf.f90:692,
// 478, 848).
#pragma once

namespace mq {

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

// Sum over the block of one value per thread (red: blockDim.x/32 doubles).
__device__ __forceinline__ double jac_block_sum(double v, double *red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
  return t;
}

// Diagonalise A in place (n x n, column-major, shared or global memory of this
// CTA), V <- the rotations (starts as the identity).  cs: n' doubles (a cosine
// and a sine per pair of a round, n' = n rounded up to even), red:
// blockDim.x/32 doubles, flag: a shared int (unused, kept for callers).
// Returns false when max_sweeps did not reach the tolerance.
static __device__ bool jacobi_block(int n, double *A, double *V, double *cs, double *red, int *flag, int max_sweeps,
                             double tol) {
  const int tid = threadIdx.x;
  const size_t n2 = (size_t)n * n;
  for (size_t idx = tid; idx < n2; idx += blockDim.x) V[idx] = (idx % (n + 1) == 0) ? 1.0 : 0.0;
  double fro = 0.0;
  for (size_t idx = tid; idx < n2; idx += blockDim.x) fro += A[idx] * A[idx];
  const double stop2 = tol * tol * jac_block_sum(fro, red);
  const int np = n + (n & 1), half = np / 2;
  for (int sweep = 0; sweep < max_sweeps; ++sweep) {
    double off = 0.0;
    for (size_t idx = tid; idx < n2; idx += blockDim.x) {
      const int i = (int)(idx % n), j = (int)(idx / n);
      if (i != j) off += A[idx] * A[idx];
    }
    off = jac_block_sum(off, red);
    if (off <= stop2) return true;
    for (int r = 0; r < np - 1; ++r) {
      // 1) rotation angles
      for (int k = tid; k < half; k += blockDim.x) {
        int p, q;
        rr_pair(np, r, k, p, q);
        double c = 1.0, s = 0.0;
        if (q < n) {
          const double apq = A[p + (size_t)n * q];
          const double app = A[p + (size_t)n * p], aqq = A[q + (size_t)n * q];
          if (fabs(apq) > 0x1p-60 * (fabs(app) + fabs(aqq))) {  // negligible rotations are skipped
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
  (void)flag;
  return false;
}

// Rank of eigenvalue i among the diagonal of A (ascending, ties by index).
__device__ __forceinline__ int jacobi_rank(int n, const double *A, int i) {
  const double wi = A[i + (size_t)n * i];
  int rank = 0;
  for (int j = 0; j < n; ++j) {
    const double wj = A[j + (size_t)n * j];
    rank += (wj < wi) || (wj == wi && j < i);
  }
  return rank;
}

// Eigenvalues ascending into w, eigenvectors into the matching columns of Vout,
// each with its largest component positive.
static __device__ void jacobi_sorted_out(int n, const double *A, const double *V, double *w, double *Vout) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const int rank = jacobi_rank(n, A, i);
    w[rank] = A[i + (size_t)n * i];
    double big = 0.0;
    for (int k = 0; k < n; ++k)
      if (fabs(V[k + (size_t)n * i]) > fabs(big)) big = V[k + (size_t)n * i];
    const double sg = big < 0 ? -1.0 : 1.0;
    for (int k = 0; k < n; ++k) Vout[k + (size_t)n * rank] = sg * V[k + (size_t)n * i];
  }
}

}  // namespace mq
