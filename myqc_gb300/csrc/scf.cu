// scf.cu -- RHF/UHF SCF on the device.
//
// Restates the scf executable's loop (src/scf/scf.f90: RHF :61-216,
// UHF :221-404, initRHF/initUHF :410-622, RHFiter :720-904, UHFiter
// :909-1117, checkConv :1157-1267) with the dens and RHFI2G/UHFI2G child
// processes folded in.  Iteration k takes the input density D_k (from the
// orbitals of iteration k-1; D_0 from the core-Hamiltonian guess), forms
// G[D_k], F = H + G and E_k = 1/2 sum D_k (F + H) + E_nuc, solves F C = S C e,
// builds D_{k+1}, and for k > 0 stops when max|D_{k+1} - D_k| < threshold --
// the reference's rule; the reported energy is E_k, as scf.f90:900 prints it.
// Optional DIIS (a method addition with the same fixed point) extrapolates F
// from the last m Fock matrices with commutator errors F D S - S D F.
//
// The generalized problem is solved as C = X C' with X = S^-1/2 and
// X^T F X C' = C' e (Jacobi), which gives the C^T S C = 1 normalisation and
// ascending eigenvalues that DSYGV(1,'V','L') returns.  With opts->purify the
// iterations build D_{k+1} from the spectral projector of X^T F X by
// trace-correcting purification instead (purify.cu), and the eigensolver runs
// once, on the last iteration's F, for the orbitals and eigenvalues.
#include <cmath>
#include <vector>

#include "internal.h"

namespace mq {

static inline bool cuda_ok(cudaError_t e) { return e == cudaSuccess; }

__global__ void sub_kernel(const double *a, const double *b, double *c, size_t n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) c[i] = a[i] - b[i];
}

__global__ void add_kernel(const double *a, const double *b, double *c, size_t n) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) c[i] = a[i] + b[i];
}

// Reductions over n^2 elements in two launches: RED_BLOCKS CTAs write
// partial sums, one CTA adds them in CTA order (deterministic).  A single CTA
// would run the FP64 arithmetic of the whole matrix on one SM.
constexpr int RED_BLOCKS = 64, RED_THREADS = 256;

__device__ __forceinline__ double red_sum(double v, double *sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sh[w];
  return t;
}
__device__ __forceinline__ double red_max(double v, double *sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t = fmax(t, sh[w]);
  return t;
}

// part[b] = partial of sum D (F + H)
__global__ void __launch_bounds__(RED_THREADS) energy_part_kernel(const double *__restrict__ D,
                                                                  const double *__restrict__ F,
                                                                  const double *__restrict__ H, size_t n2,
                                                                  double *__restrict__ part) {
  __shared__ double sh[RED_THREADS / 32];
  double e = 0.0;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += (size_t)gridDim.x * blockDim.x)
    e += D[i] * (F[i] + H[i]);
  e = red_sum(e, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = e;
}
// out[2 slot] = 1/2 sum of the partials
__global__ void energy_final_kernel(const double *__restrict__ part, int nb, double *__restrict__ out, int slot) {
  if (threadIdx.x != 0) return;
  double e = 0.0;
  for (int b = 0; b < nb; ++b) e += part[b];
  out[2 * slot] = 0.5 * e;
}

// part[2b], part[2b+1] = partial max |Dn - Do| and sum (Dn - Do)^2
__global__ void __launch_bounds__(RED_THREADS) diff_part_kernel(const double *__restrict__ Dn,
                                                                const double *__restrict__ Do, size_t n2,
                                                                double *__restrict__ part) {
  __shared__ double sh[RED_THREADS / 32];
  double m = 0.0, s2 = 0.0;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += (size_t)gridDim.x * blockDim.x) {
    const double d = Dn[i] - Do[i];
    m = fmax(m, fabs(d));
    s2 += d * d;
  }
  m = red_max(m, sh);
  s2 = red_sum(s2, sh);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = m;
    part[2 * blockIdx.x + 1] = s2;
  }
}
// out[0] = max |Dn - Do|, out[1] = RMS over all spin blocks
__global__ void diff_final_kernel(const double *__restrict__ part, int nb, size_t n2, double *__restrict__ out) {
  if (threadIdx.x != 0) return;
  double m = 0.0, s2 = 0.0;
  for (int b = 0; b < nb; ++b) {
    m = fmax(m, part[2 * b]);
    s2 += part[2 * b + 1];
  }
  out[0] = m;
  out[1] = sqrt(s2 / (double)n2);
}

// X = U diag(s^-1/2) U^T: scale columns of U into W = U diag(s^-1/2)
__global__ void scale_cols_kernel(const double *U, const double *s, double *W, int n, double power) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (size_t)n * n) return;
  const int col = (int)(i / n);
  W[i] = U[i] * pow(s[col], power);
}

// e = A - A^T  (commutator F D S - S D F for symmetric F, D, S)
__global__ void antisym_kernel(const double *A, double *E, int n) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (size_t)n * n) return;
  const int r = (int)(i % n), c = (int)(i / n);
  E[i] = A[i] - A[c + (size_t)n * r];
}

// part[16 b + j] = partial of <E_row, E_j> for j < m (m <= 16)
__global__ void __launch_bounds__(RED_THREADS) dots_part_kernel(const double *__restrict__ E, size_t n2, int row,
                                                                int m, size_t stride, double *__restrict__ part) {
  __shared__ double sh[RED_THREADS / 32];
  double s[16];
#pragma unroll
  for (int j = 0; j < 16; ++j) s[j] = 0.0;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += (size_t)gridDim.x * blockDim.x) {
    const double er = E[stride * row + i];
#pragma unroll
    for (int j = 0; j < 16; ++j)
      if (j < m) s[j] += er * E[stride * j + i];
  }
#pragma unroll
  for (int j = 0; j < 16; ++j) {
    if (j >= m) break;
    const double t = red_sum(s[j], sh);
    if (threadIdx.x == 0) part[16 * blockIdx.x + j] = t;
  }
}
// B[j] = sum over CTAs of the partials, j < m
__global__ void dots_final_kernel(const double *__restrict__ part, int nb, int m, double *__restrict__ B) {
  const int j = threadIdx.x;
  if (j >= m) return;
  double t = 0.0;
  for (int b = 0; b < nb; ++b) t += part[16 * b + j];
  B[j] = t;
}

__global__ void lincomb_kernel(const double *F, size_t stride, const double *coef, int m, double *out, size_t n2) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n2) return;
  double s = 0.0;
  for (int k = 0; k < m; ++k) s += coef[k] * F[stride * k + i];
  out[i] = s;
}

// solve the DIIS system [B -1; -1 0][c; l] = [0; -1] (m <= 16) by Gaussian elimination
static bool diis_solve(const std::vector<double> &B, int m, std::vector<double> &cvec) {
  const int N = m + 1;
  std::vector<double> A((size_t)N * N, 0.0), b(N, 0.0);
  double scale = 0;
  for (int i = 0; i < m; ++i) scale = std::max(scale, std::fabs(B[(size_t)i * m + i]));
  if (scale <= 0) return false;
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < m; ++j) A[(size_t)i * N + j] = B[(size_t)i * m + j] / scale;
  for (int i = 0; i < m; ++i) A[(size_t)i * N + m] = A[(size_t)m * N + i] = -1.0;
  b[m] = -1.0;
  for (int k = 0; k < N; ++k) {
    int piv = k;
    for (int i = k + 1; i < N; ++i)
      if (std::fabs(A[(size_t)i * N + k]) > std::fabs(A[(size_t)piv * N + k])) piv = i;
    if (std::fabs(A[(size_t)piv * N + k]) < 1e-300) return false;
    if (piv != k) {
      for (int j = 0; j < N; ++j) std::swap(A[(size_t)k * N + j], A[(size_t)piv * N + j]);
      std::swap(b[k], b[piv]);
    }
    for (int i = k + 1; i < N; ++i) {
      const double f = A[(size_t)i * N + k] / A[(size_t)k * N + k];
      for (int j = k; j < N; ++j) A[(size_t)i * N + j] -= f * A[(size_t)k * N + j];
      b[i] -= f * b[k];
    }
  }
  std::vector<double> x(N);
  for (int i = N - 1; i >= 0; --i) {
    double s = b[i];
    for (int j = i + 1; j < N; ++j) s -= A[(size_t)i * N + j] * x[j];
    x[i] = s / A[(size_t)i * N + i];
  }
  cvec.assign(x.begin(), x.begin() + m);
  return true;
}

static double nuclear_repulsion(const mq_ctx *c) {
  // getEnr, src/scf/scf.f90:1122-1152
  double E = 0.0;
  for (int a = 0; a < c->nnuc; ++a)
    for (int b = 0; b < a; ++b) {
      double r2 = 0;
      for (int k = 0; k < 3; ++k) {
        const double d = c->xyz[3 * a + k] - c->xyz[3 * b + k];
        r2 += d * d;
      }
      E += c->Z[a] * c->Z[b] / std::sqrt(r2);
    }
  return E;
}

static unsigned blocks(size_t n, int tb = 256) { return (unsigned)((n + tb - 1) / tb); }

int scf_device(mq_ctx *c, const double *S, const double *H, const mq_scf_opts *o, double *C, double *eps, double *D,
               double *energy, int *iters, double *history) {
  const int n = c->nao;
  const size_t n2 = (size_t)n * n;
  const bool uhf = o->uhf != 0;
  const int ns = uhf ? 2 : 1;
  const int max_iter = o->max_iter > 0 ? o->max_iter : (uhf ? 300 : 500);
  const double thr = o->conv > 0 ? o->conv : 1e-7;
  const int ndiis = std::min(o->diis, 16);
  const int nocc[2] = {uhf ? o->nalpha : (o->nalpha + o->nbeta) / 2, o->nbeta};
  const double occf = uhf ? 1.0 : 2.0;
  if (!uhf && o->nalpha != o->nbeta) return set_err(c, MQ_EINVAL, "RHF needs nalpha == nbeta");
  if (nocc[0] > n || nocc[1] > n || nocc[0] < 0 || nocc[1] < 0) return set_err(c, MQ_EINVAL, "bad occupation");
  if (c->nparts > 1)
    return set_err(c, MQ_EINVAL, "a molecule split over processes iterates on the host (one all-reduce of G per "
                                 "iteration); mq_scf needs mq_set_partition(ctx, 0, 1)");
  if (!o->direct && !c->xx_valid && !c->qs.valid)
    return set_err(c, MQ_ESTATE, "no stored integrals for a conventional SCF");

  // device workspace
  const size_t nmat = 8 + 8 * ns + (size_t)2 * ndiis * ns;
  double *w = (double *)buf(c, "scf_work", sizeof(double) * (n2 * nmat + 256 + n * ns + 16 * RED_BLOCKS));
  if (!w) return MQ_ENOMEM;
  double *dS = w, *dH = dS + n2, *dX = dH + n2, *dT1 = dX + n2, *dT2 = dT1 + n2, *dT3 = dT2 + n2;
  double *dU = dT3 + n2, *dW = dU + n2;
  double *dD = dW + n2;            // ns input densities
  double *dDn = dD + n2 * ns;      // ns new densities
  double *dG = dDn + n2 * ns;      // ns
  double *dF = dG + n2 * ns;       // ns
  double *dC = dF + n2 * ns;       // ns
  double *dFp = dC + n2 * ns;      // ns (orthogonal-basis Fock / eigvec scratch)
  double *dFh = dFp + n2 * ns;     // DIIS Fock history ns * ndiis
  double *dEh = dFh + n2 * ns * ndiis;  // DIIS error history
  double *dGp = dEh + n2 * ns * ndiis;  // ns: G of the previous build (incremental builds)
  double *dDp = dGp + n2 * ns;          // ns: the density it was built from
  double *dScal = dDp + n2 * ns;        // 256 scalars
  double *dEps = dScal + 256;           // n * ns
  double *dRed = dEps + n * ns;         // reduction partials, 16 per CTA
  // X = S^-1/2: Newton-Schulz (GEMMs only) with purification, else (and as its
  // fallback) the eigendecomposition S = U s U^T.  Newton-Schulz needs S alone:
  // it runs on the aux stream, so that it does not wait for work queued on
  // the main stream before this call (an integral pass), and the main stream
  // waits for it before any use of S, X or its scratch.
  bool have_x = false;
  if (o->purify) {
    MQ_TRY(ensure_aux(c));
    cudaStream_t main = c->stream;
    c->stream = c->aux;
    int ns_steps = 0;
    int rc = cuda_ok(cudaMemcpyAsync(dS, S, n2 * sizeof(double), cudaMemcpyHostToDevice, c->stream))
                 ? inv_sqrt_ns(c, n, dS, dX, dT1, dScal + 128, &ns_steps)  // scratch dT1..dW (5 n^2)
                 : set_err(c, MQ_ECUDA, "S upload");
    const bool rec = cudaEventRecord(c->ev_early, c->stream) == cudaSuccess;
    c->stream = main;
    if (rec) MQ_CUDA(c, cudaStreamWaitEvent(c->stream, c->ev_early, 0));
    else MQ_CUDA(c, cudaStreamSynchronize(c->aux));
    if (rc != MQ_OK && rc != MQ_ENOCONV) return rc;
    have_x = rc == MQ_OK;
  } else {
    MQ_CUDA(c, cudaMemcpyAsync(dS, S, n2 * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  }
  MQ_CUDA(c, cudaMemcpyAsync(dH, H, n2 * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  if (!have_x) {
    MQ_CUDA(c, cudaMemcpyAsync(dT1, dS, n2 * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    MQ_TRY(syev_batched_device(c, n, 1, dT1, dEps, dU));
    std::vector<double> sev(n);
    MQ_CUDA(c, cudaMemcpyAsync(sev.data(), dEps, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    MQ_CUDA(c, cudaStreamSynchronize(c->stream));
    if (sev[0] <= 0.0) return set_err(c, MQ_EINVAL, "overlap matrix is not positive definite");
    scale_cols_kernel<<<blocks(n2), 256, 0, c->stream>>>(dU, dEps, dW, n, -0.5);
    MQ_TRY(gemm(c, 'N', 'T', n, n, n, 1.0, dW, n, dU, n, 0.0, dX, n));
  }

  // solve F C = S C e for ns Fock matrices in dF -> dC, dEps.  Eigenvectors
  // (orthogonal basis) go to dU (and dW, which follows it, for beta).  Large
  // orders start the Jacobi sweeps from the previous iteration's vectors:
  // A0 = U^T F' U is nearly diagonal once the SCF settles, so few sweeps remain.
  bool have_prev = false;
  bool refine_prev = false;  // dU holds vectors of an earlier SCF iteration's Fock matrix (the early eigensolve)
  auto diagonalize = [&](const double *Fm) -> int {
    for (int s = 0; s < ns; ++s) {
      MQ_TRY(gemm(c, 'T', 'N', n, n, n, 1.0, dX, n, Fm + n2 * s, n, 0.0, dT1, n));
      MQ_TRY(gemm(c, 'N', 'N', n, n, n, 1.0, dT1, n, dX, n, 0.0, dFp + n2 * s, n));
    }
    if (n <= JAC_SMEM_MAX) {
      MQ_TRY(syev_batched_device(c, n, ns, dFp, dEps, dU));
    } else {
      for (int s = 0; s < ns; ++s) {
        double *A = dFp + n2 * s, *U = dU + n2 * s;
        if (refine_prev) {  // start vectors of an earlier Fock matrix: refine, then the Jacobi cleanup
          MQ_TRY(syev_large_warm(c, n, A, dEps + (size_t)n * s, U));
          continue;
        }
        if (have_prev) {
          MQ_TRY(gemm(c, 'T', 'N', n, n, n, 1.0, U, n, A, n, 0.0, dT1, n));
          MQ_TRY(gemm(c, 'N', 'N', n, n, n, 1.0, dT1, n, U, n, 0.0, A, n));
        }
        if (have_prev)
          MQ_TRY(syev_large_device(c, n, A, U, dEps + (size_t)n * s, U));
        else
          MQ_TRY(syev_large_cold(c, n, A, dEps + (size_t)n * s, U));
      }
      have_prev = true;
      refine_prev = false;
    }
    return MQ_OK;
  };
  auto orbitals_to_density = [&](double *Dout) -> int {
    for (int s = 0; s < ns; ++s) {
      MQ_TRY(gemm(c, 'N', 'N', n, n, n, 1.0, dX, n, dU + n2 * s, n, 0.0, dC + n2 * s, n));
      MQ_TRY(density_device(c, n, nocc[s], dC + n2 * s, occf, Dout + n2 * s));
    }
    return MQ_OK;
  };
  // new densities from the Fock matrices Fm: the eigensolver, or purification
  // of F' = X F X into the projector P and D = occf X P X.  Purification that
  // stalls (degenerate frontier levels) falls back to the eigensolver, cold
  // started: the warm-start vectors in dU/dW are overwritten by its scratch.
  const bool purify = o->purify != 0;
  // Early eigensolve (purification, RHF, JAC_SMEM_MAX < n): once the density
  // changes by less than EARLY_EIG_RMS, the cold eigensolve of that
  // iteration's Fock matrix is queued on the aux stream and overlaps the
  // remaining iterations; the final eigensolve then starts from its vectors
  // (a few FP64 Jacobi sweeps) instead of cold.  Its own buffers: the Fock
  // copy, X^T F X, the vectors, the eigenvalues, a GEMM temporary.
  constexpr double EARLY_EIG_RMS = 1e-5;
  bool early = false;  // queued, not yet joined
  double *dFe = nullptr, *dAe = nullptr, *dUe = nullptr, *dTe = nullptr, *dEe = nullptr;
  bool early_vectors = false;  // the early solve queued start vectors into dUe
  auto join_early = [&](bool use) -> int {  // the main stream after the early solve; its vectors into dU when use
    if (!early) return MQ_OK;
    early = false;
    MQ_CUDA(c, cudaStreamWaitEvent(c->stream, c->ev_early, 0));
    if (!use || !early_vectors) return MQ_OK;
    MQ_CUDA(c, cudaMemcpyAsync(dU, dUe, n2 * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    have_prev = true;
    refine_prev = true;
    c->stats.eig_early = 1;
    return MQ_OK;
  };
  auto launch_early = [&](const double *Fm) -> int {
    double *e = (double *)buf(c, "scf_early", sizeof(double) * (4 * n2 + n));
    if (!e) return MQ_ENOMEM;
    dFe = e;
    dAe = e + n2;
    dUe = e + 2 * n2;
    dTe = e + 3 * n2;
    dEe = e + 4 * n2;
    MQ_TRY(ensure_aux(c));
    MQ_CUDA(c, cudaMemcpyAsync(dFe, Fm, n2 * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    MQ_CUDA(c, cudaEventRecord(c->ev_early, c->stream));
    MQ_CUDA(c, cudaStreamWaitEvent(c->aux, c->ev_early, 0));
    cudaStream_t main = c->stream;
    c->stream = c->aux;
    int rc = gemm(c, 'T', 'N', n, n, n, 1.0, dX, n, dFe, n, 0.0, dTe, n);
    if (rc == MQ_OK) rc = gemm(c, 'N', 'N', n, n, n, 1.0, dTe, n, dX, n, 0.0, dAe, n);
    // start vectors only: the grid-barrier FP64 Jacobi of the final solve
    // runs on the main stream after the iterations, never beside another
    // cooperatively launched kernel (the purification)
    bool started = false;
    if (rc == MQ_OK) {
      rc = syev_large_start(c, n, dAe, dUe);
      started = rc == MQ_OK;
      if (rc == MQ_EINVAL) rc = MQ_OK;  // an order without the cluster solver: no warm start
    }
    // the event marks the end of whatever was queued on the aux stream
    const cudaError_t ev = cudaEventRecord(c->ev_early, c->aux);
    if (rc == MQ_OK && ev != cudaSuccess) rc = cuda_check(c, ev, "cudaEventRecord (early eigensolve)");
    c->stream = main;
    MQ_TRY(rc);
    early = true;
    early_vectors = started;
    return MQ_OK;
  };
  auto density_step = [&](const double *Fm, double *Dout) -> int {
    if (purify) {
      bool ok = true;
      for (int s = 0; s < ns && ok; ++s) {
        MQ_TRY(gemm(c, 'T', 'N', n, n, n, 1.0, dX, n, Fm + n2 * s, n, 0.0, dT1, n));
        MQ_TRY(gemm(c, 'N', 'N', n, n, n, 1.0, dT1, n, dX, n, 0.0, dFp + n2 * s, n));
        int steps = 0;
        const int rc = purify_projector(c, n, nocc[s], dFp + n2 * s, dT3, dT2, dW, dScal + 128, &steps);
        c->stats.purify_steps += steps;
        if (rc == MQ_ENOCONV) {
          ok = false;
          break;
        }
        MQ_TRY(rc);
        MQ_TRY(gemm(c, 'N', 'N', n, n, n, 1.0, dX, n, dT3, n, 0.0, dT1, n));
        MQ_TRY(gemm(c, 'N', 'N', n, n, n, occf, dT1, n, dX, n, 0.0, Dout + n2 * s, n));
      }
      if (ok) return MQ_OK;
      MQ_TRY(join_early(false));  // the eigensolver's buffers are the early solve's too
      have_prev = false;
    }
    MQ_TRY(diagonalize(Fm));
    c->stats.diag_calls += 1;
    return orbitals_to_density(Dout);
  };

  // initial density
  c->stats.diag_calls = 0;
  c->stats.purify_steps = 0;
  c->stats.purify_persistent = c->stats.purify_stepwise = 0;
  if (o->guess == 2 && o->D_in) {
    MQ_CUDA(c, cudaMemcpyAsync(dD, o->D_in, n2 * ns * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  } else if (purify && !(o->guess == 1 && o->C_in)) {  // core Hamiltonian, purified
    for (int s = 0; s < ns; ++s)
      MQ_CUDA(c, cudaMemcpyAsync(dF + n2 * s, dH, n2 * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    MQ_TRY(density_step(dF, dD));
  } else {
    if (o->guess == 1 && o->C_in) {
      MQ_CUDA(c, cudaMemcpyAsync(dC, o->C_in, n2 * ns * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    } else {  // core Hamiltonian (initRHF / initUHF): same orbitals for both spins
      for (int s = 0; s < ns; ++s)
        MQ_CUDA(c, cudaMemcpyAsync(dF + n2 * s, dH, n2 * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
      MQ_TRY(diagonalize(dF));
      for (int s = 0; s < ns; ++s)
        MQ_TRY(gemm(c, 'N', 'N', n, n, n, 1.0, dX, n, dU + n2 * s, n, 0.0, dC + n2 * s, n));
    }
    for (int s = 0; s < ns; ++s) MQ_TRY(density_device(c, n, nocc[s], dC + n2 * s, occf, dD + n2 * s));
  }

  const double enuc = nuclear_repulsion(c);
  StageTimer t_fock, t_diag, t_all, t_full;  // t_full: the full builds of a screened-increment SCF
  c->t_fock_kernel.collect();
  c->t_fock_kernel.total = 0;
  c->stats.fock_kernel_launches = 0;
  t_all.start(c->stream);
  std::vector<double> Bm((size_t)ndiis * ndiis * 4, 0.0);
  int nh = 0, head = 0;
  double E = 0.0;
  bool conv = false;
  int it = 0;
  std::vector<double> hist;
  const double *lastF = nullptr;
  // incremental builds: once the density moves by less than fock_inc_tau
  // (max |D_k - D_{k-1}|), G_k = G_{k-1} + G[D_k - D_{k-1}] with the increment
  // digested in FP32; its error scales with the increment, so the converged
  // energy stays within ~1e-9 Eh of the full builds'
  const bool inc = !o->direct && c->fock_inc_tau > 0.0;
  // screened FP64 increments from the quartet store (RHF): after the first
  // build, G_k = G_{k-1} + G[D_k - D_{k-1}] over the shell quartets with
  // Q_P Q_Q max|D_k - D_{k-1}| >= fock_inc_screen -- the Schwarz screen's
  // criterion applied to the density change, in FP64 throughout
  const bool inc_store = !o->direct && !uhf && c->qs.valid && !c->fock_df32 && c->fock_inc_screen > 0.0;
  double *dInc = nullptr;
  if (inc_store) {
    dInc = (double *)buf(c, "scf_dinc", sizeof(double) * n2);
    if (!dInc) return MQ_ENOMEM;
  }
  c->stats.fock_screened_builds = 0;
  c->stats.fock_full_builds = 0;
  bool have_prev_g = false;
  double last_maxdiff = INFINITY, prev_rms = INFINITY;
  bool early_done = false;
  c->stats.fock_inc_builds = 0;
  c->stats.eig_early = 0;
  // the transform's first operand depends on the integrals alone: slice it on
  // the side stream from here on, memory-bound work beside the FP64-bound
  // iterations (purification steps launch singly while it runs)
  if (purify && c->ao2mo_prefetch && !o->direct && c->qs.valid && !c->xx_sliced) MQ_TRY(ao2mo_preslice_xx(c));
  for (; it < max_iter && !conv; ++it) {
    // G[D_k]
    t_fock.start(c->stream);
    if (o->direct && !uhf && !c->fock_df32) {  // RHF: integral blocks recomputed into the store, digested from it
      c->t_fock_kernel.start(c->stream);
      MQ_TRY(fock_direct_store_rhf(c, dD, dG));
      c->t_fock_kernel.stop(c->stream);
      c->stats.fock_kernel_launches += 1;
    } else if (o->direct) {
      double *J = dT1, *Ka = dT2, *Kb = uhf ? dT3 : nullptr;
      MQ_TRY(fock_direct_device(c, dD, uhf ? dD + n2 : nullptr, J, Ka, Kb));
      MQ_TRY(direct_combine(c, J, Ka, Kb, dG, uhf ? dG + n2 : nullptr));
    } else if (inc_store && have_prev_g) {
      c->t_fock_kernel.collect();
      c->t_fock_kernel.start(c->stream);
      sub_kernel<<<blocks(n2), 256, 0, c->stream>>>(dD, dDp, dInc, n2);
      const double kscreen = last_maxdiff > 0.0 ? c->fock_inc_screen / last_maxdiff : INFINITY;
      MQ_TRY(qstore_fock_rhf(c, dInc, dG, dGp, kscreen));
      c->t_fock_kernel.stop(c->stream);
      c->stats.fock_kernel_launches += 1;
      c->stats.fock_screened_builds += 1;
      c->stats.launches += 1;
    } else if (inc && have_prev_g && last_maxdiff < c->fock_inc_tau) {
      MQ_TRY(fock_stored_increment(c, dD, uhf ? dD + n2 : nullptr, dDp, uhf ? dDp + n2 : nullptr, dGp,
                                   uhf ? dGp + n2 : nullptr, dG, uhf ? dG + n2 : nullptr));
      c->stats.fock_inc_builds += 1;
    } else {
      t_full.start(c->stream);
      MQ_TRY(fock_stored_device(c, dD, uhf ? dD + n2 : nullptr, dG, uhf ? dG + n2 : nullptr));
      t_full.stop(c->stream);
      c->stats.fock_full_builds += 1;
    }
    if (inc || inc_store) {
      MQ_CUDA(c, cudaMemcpyAsync(dGp, dG, n2 * ns * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
      MQ_CUDA(c, cudaMemcpyAsync(dDp, dD, n2 * ns * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
      have_prev_g = true;
    }
    t_fock.stop(c->stream);
    for (int s = 0; s < ns; ++s) add_kernel<<<blocks(n2), 256, 0, c->stream>>>(dH, dG + n2 * s, dF + n2 * s, n2);
    for (int s = 0; s < ns; ++s) {
      energy_part_kernel<<<RED_BLOCKS, RED_THREADS, 0, c->stream>>>(dD + n2 * s, dF + n2 * s, dH, n2, dRed);
      energy_final_kernel<<<1, 32, 0, c->stream>>>(dRed, RED_BLOCKS, dScal, s);
    }
    const double *Fdiag = dF;
    if (ndiis > 0) {
      // commutator errors e_s = F D S - S D F, stored with F in ring slot `head`
      for (int s = 0; s < ns; ++s) {
        double *Fs = dFh + n2 * ((size_t)ns * head + s), *Es = dEh + n2 * ((size_t)ns * head + s);
        MQ_CUDA(c, cudaMemcpyAsync(Fs, dF + n2 * s, n2 * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
        MQ_TRY(gemm(c, 'N', 'N', n, n, n, 1.0, dF + n2 * s, n, dD + n2 * s, n, 0.0, dT1, n));
        MQ_TRY(gemm(c, 'N', 'N', n, n, n, 1.0, dT1, n, dS, n, 0.0, dT2, n));
        antisym_kernel<<<blocks(n2), 256, 0, c->stream>>>(dT2, Es, n);
      }
      nh = std::min(nh + 1, ndiis);
      // new row of B: sum over spins of <e_head, e_j>
      for (int j = 0; j < ndiis; ++j) Bm[(size_t)head * ndiis + j] = Bm[(size_t)j * ndiis + head] = 0.0;
      std::vector<double> row(ndiis, 0.0);
      for (int s = 0; s < ns; ++s) {
        dots_part_kernel<<<RED_BLOCKS, RED_THREADS, 0, c->stream>>>(dEh + n2 * s, n2, head, nh, n2 * ns, dRed);
        dots_final_kernel<<<1, 32, 0, c->stream>>>(dRed, RED_BLOCKS, nh, dScal + 16 + 16 * s);
      }
      std::vector<double> hrow(32);
      MQ_CUDA(c, cudaMemcpyAsync(hrow.data(), dScal + 16, 32 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
      MQ_CUDA(c, cudaStreamSynchronize(c->stream));
      for (int j = 0; j < nh; ++j) {
        double v = hrow[j] + (uhf ? hrow[16 + j] : 0.0);
        Bm[(size_t)head * ndiis + j] = Bm[(size_t)j * ndiis + head] = v;
      }
      if (nh >= 2) {
        std::vector<double> Bs((size_t)nh * nh), cv;
        for (int i = 0; i < nh; ++i)
          for (int j = 0; j < nh; ++j) Bs[(size_t)i * nh + j] = Bm[(size_t)i * ndiis + j];
        if (diis_solve(Bs, nh, cv)) {
          MQ_CUDA(c, cudaMemcpyAsync(dScal + 64, cv.data(), nh * sizeof(double), cudaMemcpyHostToDevice, c->stream));
          // extrapolated Fock matrices into dG (free once F = H + G is formed)
          for (int s = 0; s < ns; ++s)
            lincomb_kernel<<<blocks(n2), 256, 0, c->stream>>>(dFh + n2 * s, n2 * ns, dScal + 64, nh, dG + n2 * s,
                                                              n2);
          Fdiag = dG;
        }
      }
      head = (head + 1) % ndiis;
    }
    if (purify && !uhf && !early_done && n > JAC_SMEM_MAX && prev_rms < EARLY_EIG_RMS) {
      MQ_TRY(launch_early(Fdiag));
      early_done = true;
    }
    t_diag.start(c->stream);
    MQ_TRY(density_step(Fdiag, dDn));
    t_diag.stop(c->stream);
    lastF = Fdiag;
    diff_part_kernel<<<RED_BLOCKS, RED_THREADS, 0, c->stream>>>(dDn, dD, n2 * ns, dRed);
    diff_final_kernel<<<1, 32, 0, c->stream>>>(dRed, RED_BLOCKS, n2 * ns, dScal + 8);
    c->stats.launches += 2 + 2 * ns;
    double hs[10];
    MQ_CUDA(c, cudaMemcpyAsync(hs, dScal, 10 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    MQ_CUDA(c, cudaStreamSynchronize(c->stream));
    t_fock.collect();
    t_full.collect();
    t_diag.collect();
    c->t_fock_kernel.collect();
    E = hs[0] + (uhf ? hs[2] : 0.0) + enuc;
    const double diff = o->conv_rms ? hs[9] : hs[8];
    last_maxdiff = hs[8];  // max |D_{k+1} - D_k|: the next build's increment
    prev_rms = hs[9];
    hist.push_back(E);
    hist.push_back(it > 0 ? diff : NAN);
    if (it > 0) conv = diff < thr;
    if (!conv) {
      // D_{k+1} becomes the next input density
      MQ_CUDA(c, cudaMemcpyAsync(dD, dDn, n2 * ns * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    }
  }
  // outputs: orbitals and eigenvalues of the last diagonalisation, D_k of the last iteration
  c->stats.ms_eig_final = 0;
  if (purify && lastF) {  // one eigensolve of the last iteration's Fock matrices for C and eps
    // the transform's XX slices need no orbitals: form them beside the eigensolve
    if (c->ao2mo_prefetch && !o->direct && !c->xx_sliced) MQ_TRY(ao2mo_preslice_xx(c));
    StageTimer t_eig;
    t_eig.start(c->stream);
    have_prev = false;
    MQ_TRY(join_early(true));  // warm start from the early eigensolve when there was one
    MQ_TRY(diagonalize(lastF));
    c->stats.diag_calls += 1;
    for (int s = 0; s < ns; ++s)
      MQ_TRY(gemm(c, 'N', 'N', n, n, n, 1.0, dX, n, dU + n2 * s, n, 0.0, dC + n2 * s, n));
    t_eig.stop(c->stream);
    t_eig.collect_sync();
    c->stats.ms_eig_final = t_eig.total;
  }
  MQ_TRY(join_early(false));  // (an SCF that ended without a final eigensolve)
  MQ_CUDA(c, cudaMemcpyAsync(C, dC, n2 * ns * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  MQ_CUDA(c, cudaMemcpyAsync(eps, dEps, (size_t)n * ns * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  if (D) MQ_CUDA(c, cudaMemcpyAsync(D, dD, n2 * ns * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  t_all.stop(c->stream);
  MQ_CUDA(c, cudaStreamSynchronize(c->stream));
  t_all.collect();
  c->stats.ms_scf = t_all.total;
  c->stats.ms_fock = t_fock.total;
  c->stats.ms_fock_full = t_full.total;
  c->stats.ms_fock_kernel = c->t_fock_kernel.total;
  c->stats.ms_diag = t_diag.total;
  c->stats.fock_calls = it;
  c->stats.scf_iters = it;
  *energy = E;
  *iters = it;
  if (history)
    for (size_t k = 0; k < hist.size(); ++k) history[k] = hist[k];
  return conv ? MQ_OK : set_err(c, MQ_ENOCONV, "SCF did not converge");
}

}  // namespace mq
