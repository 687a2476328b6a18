// eigen.cu -- cold eigendecomposition of one symmetric matrix of moderate
// order (JAC_SMEM_MAX < n <= CJ_MAX), the eigen step of DSYEV/DSYGV
// (src/scf/scf.f90:692, 478, 848) when no start vectors are known.
//
// FP64 arithmetic runs at a small fraction of the FP32 rate on this GPU, and a
// grid-wide Jacobi pays a software grid barrier per round, so the solve is
// split in three:
//  1. a cyclic Jacobi in FP32 on one thread-block cluster (16 CTAs, else 8):
//     CTA c keeps columns j = c, c + C, .. of A and V in shared memory; a round
//     reads every pair's angle inputs and each own column's partner column (A
//     and V) from the owners' shared memory (DSMEM), one cluster barrier, then
//     every CTA rewrites its own columns (rows and columns of the round's 2x2
//     blocks), a second cluster barrier.  Converges to the FP32 floor.
//  2. refinement in FP64 with GEMMs only: X is made orthonormal by Bjorck
//     steps X <- X (3 I - X^T X) / 2 (each squares the orthogonality error),
//     then twice: B = X^T A X, a first-order rotation of every well-separated
//     pair, E_ij = b_ij / (b_jj - b_ii) where |b_ij| <= 1e-3 |b_jj - b_ii|
//     (E is antisymmetric; the remaining near-degenerate pairs are left
//     alone), X <- X (I + E), and two Bjorck steps.  Each correction squares
//     the error of the separated pairs.
//  3. the FP64 grid Jacobi (linalg.cu) on X^T A X from X: only pairs left
//     coupled by step 2 (near-degenerate eigenvalues) are above its skip
//     threshold, and rounds without a rotation cost no barrier.
#include <cooperative_groups.h>

#include <cstring>

#include "internal.h"
#include "jacobi.cuh"

namespace cg = cooperative_groups;

namespace mq {

constexpr int CJ_THREADS = 512;
constexpr int CJ_MAX = 512;

// partner of index j in round r of the circle-method tournament of rr_pair
// (np players, m = np - 1 rounds; player 0 fixed)
__device__ __forceinline__ int cj_partner(int j, int r, int m) {
  // j in [0, m], r in [0, m): every residue below is one conditional step away
  if (j == 0) return 1 + r;
  if (j - 1 == r) return 0;
  int x = 2 * r - j + 1;  // in (-m, 2m)
  if (x < 0) x += m;
  if (x >= m) x -= m;
  return 1 + x;
}
// pair k of round r as rr_pair gives it, without integer division
__device__ __forceinline__ void cj_pair(int np, int r, int k, int &p, int &q) {
  const int m = np - 1;
  if (k == 0) {
    p = 0;
    q = 1 + r;
    return;
  }
  int a = r + k, b = r - k;
  if (a >= m) a -= m;
  if (b < 0) b += m;
  p = 1 + a;
  q = 1 + b;
  if (p > q) {
    const int t = p;
    p = q;
    q = t;
  }
}

// rotation halves with a fixed rounding sequence: c x - s y and s x + c y
__device__ __forceinline__ float rlo(float c, float s, float x, float y) { return __fmaf_rn(c, x, -__fmul_rn(s, y)); }
__device__ __forceinline__ float rhi(float c, float s, float x, float y) { return __fmaf_rn(s, x, __fmul_rn(c, y)); }

constexpr int CJ_TX = 128;  // threads along a pair / row index; CJ_THREADS / CJ_TX along own columns

template <int LC>  // cluster of C = 2^LC CTAs
__global__ void __launch_bounds__(CJ_THREADS, 1)
    jacobi_cluster_f32_kernel(int n, const double *__restrict__ Ain, double *__restrict__ Vout, int max_sweeps,
                              float tol, int *__restrict__ info) {
  constexpr int C = 1 << LC;
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (int)cl.block_rank();
  const int tid = threadIdx.x, nt = blockDim.x;
  const int tx = tid % CJ_TX, ty = tid / CJ_TX, ny = nt / CJ_TX;
  const int np = n + (n & 1), m = np - 1, half = np / 2;
  const int T = (n - rank + C - 1) / C;  // own columns j = rank + C t, t < T
  const int Tmax = (n + C - 1) / C;
  const int ld = (n + 3) & ~3, L4 = ld / 4;
  const size_t blk = (size_t)Tmax * ld;
  // A and V double-buffered by round parity: a round reads the current
  // buffers (its own and, over DSMEM, its peers') and writes its own columns
  // into the other pair, so one cluster barrier per round orders everything
  extern __shared__ float4 sm4[];
  float *Ab0 = reinterpret_cast<float *>(sm4);
  float *Ab1 = Ab0 + blk, *Vb0 = Ab1 + blk, *Vb1 = Vb0 + blk;
  float *BA = Vb1 + blk, *BV = BA + blk;  // partner columns of A and V in this round
  float *ang = BV + blk;                  // (c, s, t) of each pair, at 3 * (its smaller index)
  float *part = ang + 3 * np;             // [2][C] cluster partial sums
  int *pt = reinterpret_cast<int *>(part + 2 * C);  // partner of each own column in this round
  int *pu = pt + Tmax, *pv = pu + half;            // the round's pairs u < v
  __shared__ float red[CJ_THREADS / 32];

  for (size_t idx = tid; idx < blk; idx += nt) {
    const int t = (int)(idx / ld), i = (int)(idx % ld), j = rank + C * t;
    float a = 0.f, v = 0.f;
    if (t < T && i < n) {
      a = (float)(0.5 * (Ain[i + (size_t)n * j] + Ain[j + (size_t)n * i]));
      v = (i == j) ? 1.f : 0.f;
    }
    Ab0[idx] = a;
    Vb0[idx] = v;
    Ab1[idx] = 0.f;
    Vb1[idx] = 0.f;
    BA[idx] = 0.f;
    BV[idx] = 0.f;
  }
  cl.sync();  // every CTA of the cluster has started before any DSMEM access
  // cluster-wide sum: every CTA adds the same C partials in the same order
  auto cluster_sum = [&](float v, int slot) -> float {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((tid & 31) == 0) red[tid >> 5] = v;
    __syncthreads();
    if (tid < C) {
      float tot = 0.f;
      for (int w = 0; w < nt / 32; ++w) tot += red[w];
      cl.map_shared_rank(part, tid)[slot * C + rank] = tot;
    }
    cl.sync();
    float s = 0.f;
    for (int q = 0; q < C; ++q) s += part[slot * C + q];
    return s;
  };
  float fro = 0.f;
  for (int t = ty; t < T; t += ny)
    for (int i = tx; i < n; i += CJ_TX) fro += Ab0[t * ld + i] * Ab0[t * ld + i];
  fro = cluster_sum(fro, 0);
  const float stop2 = tol * tol * fro;
  float off_prev = INFINITY, off = INFINITY;
  int it = 0, sweep = 0;  // it: rounds done; the current A, V are buffer it & 1
  for (; sweep < max_sweeps; ++sweep) {
    const float *Acur = (it & 1) ? Ab1 : Ab0;
    off = 0.f;
    for (int t = ty; t < T; t += ny)
      for (int i = tx; i < n; i += CJ_TX)
        if (i != rank + C * t) off += Acur[t * ld + i] * Acur[t * ld + i];
    off = cluster_sum(off, 1);
    if (off <= stop2) break;
    if (off < 1e-8f * fro && off > 0.25f * off_prev) break;  // stalled at the FP32 floor
    off_prev = off;
    for (int r = 0; r < m; ++r, ++it) {
      float *A = (it & 1) ? Ab1 : Ab0, *V = (it & 1) ? Vb1 : Vb0;
      float *An = (it & 1) ? Ab0 : Ab1, *Vn = (it & 1) ? Vb0 : Vb1;
      // phase 1: the round's pairs and angles, this CTA's partner columns
      for (int k = tid; k < half; k += nt) {
        int p, q;
        cj_pair(np, r, k, p, q);
        pu[k] = p;
        pv[k] = q;
        float c = 1.f, s = 0.f, t = 0.f;
        if (q < n) {
          const float *Aq = cl.map_shared_rank(A, q & (C - 1)) + (size_t)(q >> LC) * ld;
          const float *Ap = cl.map_shared_rank(A, p & (C - 1)) + (size_t)(p >> LC) * ld;
          const float apq = Aq[p], aqq = Aq[q], app = Ap[p];
          if (fabsf(apq) > 0x1p-26f * (fabsf(app) + fabsf(aqq)) && apq != 0.f) {
            const float theta = (aqq - app) / (2.f * apq);
            t = (theta >= 0.f ? 1.f : -1.f) / (fabsf(theta) + sqrtf(theta * theta + 1.f));
            c = rsqrtf(t * t + 1.f);
            s = t * c;
          }
        }
        ang[3 * p] = c;
        ang[3 * p + 1] = s;
        ang[3 * p + 2] = t;
      }
      for (int t = tid; t < T; t += nt) pt[t] = cj_partner(rank + C * t, r, m);
      __syncthreads();
      // partner columns: warp w copies column t = w, w + 16, ..; lane e its float4s
      for (int t = tid >> 5; t < T; t += nt >> 5) {
        const int pj = pt[t];
        if (pj >= n) continue;
        const size_t off_src = (size_t)(pj >> LC) * ld;
        const float4 *sa = reinterpret_cast<const float4 *>(cl.map_shared_rank(A, pj & (C - 1)) + off_src);
        const float4 *sv = reinterpret_cast<const float4 *>(cl.map_shared_rank(V, pj & (C - 1)) + off_src);
        float4 *da = reinterpret_cast<float4 *>(BA + (size_t)t * ld), *dv = reinterpret_cast<float4 *>(BV + (size_t)t * ld);
        for (int e = tid & 31; e < L4; e += 32) {
          da[e] = sa[e];
          dv[e] = sv[e];
        }
      }
      __syncthreads();
      // phase 2: every element of the own columns of A and V, new values into
      // the other buffers.  Item (t, k): rows u < v of pair k, column j of pair
      // (pm, max).  The rotation of the pair with the smaller index is applied
      // first, the same order the owner of the mirror element uses, so A stays
      // exactly symmetric.
      for (int t = ty; t < T; t += ny) {
        const int j = rank + C * t, pj = pt[t];
        const bool ok = pj < n, jp = j < pj;
        const int pm = jp ? j : pj;
        const float cP = ang[3 * pm], sP = ang[3 * pm + 1], tP = ang[3 * pm + 2];
        const float *own = A + (size_t)t * ld, *oth = BA + (size_t)t * ld;
        float *dst = An + (size_t)t * ld;
        for (int k = tx; k < half; k += CJ_TX) {
          const int u = pu[k], v = pv[k];
          const bool vv = v < n;
          if (u == pm) {  // the 2x2 diagonal block of this column's own pair
            if (!ok || sP == 0.f) {
              dst[u] = own[u];
              if (vv) dst[v] = own[v];
            } else {
              dst[j] = jp ? own[j] - tP * oth[j] : own[j] + tP * own[pj];  // a_pp - t a_pq, a_qq + t a_pq
              dst[pj] = 0.f;
            }
            continue;
          }
          const float cQ = ang[3 * u], sQ = ang[3 * u + 1];
          const float xu = own[u], xv = vv ? own[v] : 0.f;
          const float yu = ok ? oth[u] : 0.f, yv = (ok && vv) ? oth[v] : 0.f;
          const float a_up = jp ? xu : yu, a_uq = jp ? yu : xu;
          const float a_vp = jp ? xv : yv, a_vq = jp ? yv : xv;
          float nu, nv;
          if (pm < u) {
            const float cu = jp ? rlo(cP, sP, a_up, a_uq) : rhi(cP, sP, a_up, a_uq);
            const float cv = jp ? rlo(cP, sP, a_vp, a_vq) : rhi(cP, sP, a_vp, a_vq);
            nu = rlo(cQ, sQ, cu, cv);
            nv = rhi(cQ, sQ, cu, cv);
          } else {
            const float qpu = rlo(cQ, sQ, a_up, a_vp), qpv = rhi(cQ, sQ, a_up, a_vp);
            const float qqu = rlo(cQ, sQ, a_uq, a_vq), qqv = rhi(cQ, sQ, a_uq, a_vq);
            nu = jp ? rlo(cP, sP, qpu, qqu) : rhi(cP, sP, qpu, qqu);
            nv = jp ? rlo(cP, sP, qpv, qqv) : rhi(cP, sP, qpv, qqv);
          }
          dst[u] = nu;
          if (vv) dst[v] = nv;
        }
        // V <- V J
        const float *vs = V + (size_t)t * ld, *vo = BV + (size_t)t * ld;
        float *vd = Vn + (size_t)t * ld;
        const bool rot = ok && sP != 0.f;
        for (int i = tx; i < n; i += CJ_TX)
          vd[i] = !rot ? vs[i] : (jp ? rlo(cP, sP, vs[i], vo[i]) : rhi(cP, sP, vo[i], vs[i]));
      }
      cl.sync();
    }
  }
  const float *Vf = (it & 1) ? Vb1 : Vb0;
  for (int t = ty; t < T; t += ny)
    for (int i = tx; i < n; i += CJ_TX) Vout[i + (size_t)n * (rank + C * t)] = (double)Vf[(size_t)t * ld + i];
  if (rank == 0 && tid == 0) {
    info[0] = sweep;
    info[1] = __float_as_int(sqrtf(off / fro));
  }
}

// FP32 start vectors into V (n x n, double); MQ_EINVAL when no cluster shape fits
static int jacobi_cluster_f32(mq_ctx *c, int n, const double *A, double *V, int *info) {
  const int max_sweeps = 30;
  const float tol = 2e-6f;
  for (int C : {16, 8}) {
    const int Tmax = (n + C - 1) / C, ld = (n + 3) & ~3, np = n + (n & 1);
    const size_t smem = (size_t)(6 * Tmax * ld + 3 * np + 2 * C + Tmax + np) * sizeof(float) + 16;
    if (smem > 200 * 1024) continue;
    const void *kern = C == 16 ? (const void *)jacobi_cluster_f32_kernel<4> : (const void *)jacobi_cluster_f32_kernel<3>;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
      cudaGetLastError();
      continue;
    }
    if (C > 8 && cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
      cudaGetLastError();
      continue;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(C);
    cfg.blockDim = dim3(CJ_THREADS);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = c->stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = C;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int ncl = 0;
    if (cudaOccupancyMaxActiveClusters(&ncl, kern, &cfg) != cudaSuccess || ncl < 1) {
      cudaGetLastError();
      continue;
    }
    if (C == 16)
      MQ_CUDA(c, cudaLaunchKernelEx(&cfg, jacobi_cluster_f32_kernel<4>, n, A, V, max_sweeps, tol, info));
    else
      MQ_CUDA(c, cudaLaunchKernelEx(&cfg, jacobi_cluster_f32_kernel<3>, n, A, V, max_sweeps, tol, info));
    c->stats.launches += 1;
    c->stats.eig_cluster = C;
    return MQ_OK;
  }
  return MQ_EINVAL;
}

// ---- refinement kernels
constexpr int RF_THREADS = 256;

// E = first-order rotation generators of the well-separated pairs of B
__global__ void __launch_bounds__(RF_THREADS) first_order_kernel(int n, const double *__restrict__ B,
                                                                double *__restrict__ E) {
  const size_t N = n, n2 = N * N;
  for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n2; idx += (size_t)gridDim.x * blockDim.x) {
    const size_t i = idx % N, j = idx / N;
    double e = 0.0;
    if (i != j) {
      const double b = 0.5 * (B[idx] + B[j + N * i]), d = B[j + N * j] - B[i + N * i];
      if (fabs(b) <= 1e-3 * fabs(d)) e = b / d;
    }
    E[idx] = e;
  }
}

// Steps 2 and 3 from start vectors d_V that nearly diagonalise d_A (the FP32
// cluster solve's, or a previous solve's): orthonormalise, two first-order
// corrections, FP64 Jacobi cleanup.  d_A keeps the matrix until the last step.
static int refine_from(mq_ctx *c, int n, double *d_A, double *d_w, double *d_V, bool async, StageTimer *t2,
                       StageTimer *t3, bool jacobi = true) {
  const size_t n2 = (size_t)n * n;
  double *ws = (double *)buf(c, "eig_refine", 3 * n2 * sizeof(double) + 64);
  if (!ws) return MQ_ENOMEM;
  double *G = ws, *T = ws + n2, *E = ws + 2 * n2;
  if (t2) t2->start(c->stream);
  double *X = d_V;
  auto bjorck = [&]() -> int {  // X <- X (3 I - X^T X) / 2
    MQ_TRY(gemm(c, 'T', 'N', n, n, n, 1.0, X, n, X, n, 0.0, G, n));
    MQ_CUDA(c, cudaMemcpyAsync(T, X, n2 * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    return gemm(c, 'N', 'N', n, n, n, -0.5, T, n, G, n, 1.5, X, n);
  };
  auto xtax = [&](double *B) -> int {  // B = X^T A X
    MQ_TRY(gemm(c, 'N', 'N', n, n, n, 1.0, d_A, n, X, n, 0.0, T, n));
    return gemm(c, 'T', 'N', n, n, n, 1.0, X, n, T, n, 0.0, B, n);
  };
  MQ_TRY(bjorck());
  MQ_TRY(bjorck());
  const unsigned grid = (unsigned)std::min<size_t>((n2 + RF_THREADS - 1) / RF_THREADS, 1024);
  for (int it = 0; it < 2; ++it) {
    MQ_TRY(xtax(G));
    first_order_kernel<<<grid, RF_THREADS, 0, c->stream>>>(n, G, E);
    c->stats.launches += 1;
    MQ_CUDA(c, cudaMemcpyAsync(T, X, n2 * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    MQ_TRY(gemm(c, 'N', 'N', n, n, n, 1.0, T, n, E, n, 1.0, X, n));
    MQ_TRY(bjorck());
    MQ_TRY(bjorck());
  }
  if (!jacobi) {  // start vectors only: A is left as it was
    MQ_CUDA(c, cudaGetLastError());
    if (t2) t2->stop(c->stream);
    return MQ_OK;
  }
  // B = X^T A X replaces A; the FP64 Jacobi rotates from X
  MQ_TRY(gemm(c, 'N', 'N', n, n, n, 1.0, d_A, n, X, n, 0.0, T, n));
  MQ_TRY(gemm(c, 'T', 'N', n, n, n, 1.0, X, n, T, n, 0.0, d_A, n));
  MQ_CUDA(c, cudaGetLastError());
  if (t2) t2->stop(c->stream);
  if (t3) t3->start(c->stream);
  MQ_TRY(syev_large_device(c, n, d_A, d_V, d_w, d_V, async));
  if (t3) t3->stop(c->stream);
  return MQ_OK;
}

int syev_large_warm(mq_ctx *c, int n, double *d_A, double *d_w, double *d_V) {
  if (n > CJ_MAX || n <= JAC_SMEM_MAX) {  // the grid Jacobi from the start vectors: A <- V^T A V first
    double *T = (double *)buf(c, "eig_warm", (size_t)n * n * sizeof(double));
    if (!T) return MQ_ENOMEM;
    MQ_TRY(gemm(c, 'T', 'N', n, n, n, 1.0, d_V, n, d_A, n, 0.0, T, n));
    MQ_TRY(gemm(c, 'N', 'N', n, n, n, 1.0, T, n, d_V, n, 0.0, d_A, n));
    return syev_large_device(c, n, d_A, d_V, d_w, d_V);
  }
  return refine_from(c, n, d_A, d_w, d_V, false, nullptr, nullptr);
}

int syev_large_start(mq_ctx *c, int n, const double *d_A, double *d_V) {
  if (n > CJ_MAX || n <= JAC_SMEM_MAX) return set_err(c, MQ_EINVAL, "start vectors: order outside the cluster range");
  const size_t n2 = (size_t)n * n;
  double *ws = (double *)buf(c, "eig_refine", 3 * n2 * sizeof(double) + 64);
  if (!ws) return MQ_ENOMEM;
  MQ_TRY(jacobi_cluster_f32(c, n, d_A, d_V, (int *)(ws + 3 * n2)));
  return refine_from(c, n, const_cast<double *>(d_A), nullptr, d_V, true, nullptr, nullptr, false);
}

int syev_large_cold(mq_ctx *c, int n, double *d_A, double *d_w, double *d_V, bool async) {
  if (n > CJ_MAX || n <= JAC_SMEM_MAX) return syev_large_device(c, n, d_A, nullptr, d_w, d_V, async);
  const size_t n2 = (size_t)n * n;
  double *ws = (double *)buf(c, "eig_refine", 3 * n2 * sizeof(double) + 64);
  if (!ws) return MQ_ENOMEM;
  int *info = (int *)(ws + 3 * n2);
  StageTimer t1, t2, t3;  // not used by an async solve (they would need a synchronisation)
  if (!async) t1.start(c->stream);
  if (jacobi_cluster_f32(c, n, d_A, d_V, info) != MQ_OK)
    return syev_large_device(c, n, d_A, nullptr, d_w, d_V, async);
  MQ_CUDA(c, cudaGetLastError());
  if (async) return refine_from(c, n, d_A, d_w, d_V, true, nullptr, nullptr);
  t1.stop(c->stream);
  MQ_TRY(refine_from(c, n, d_A, d_w, d_V, false, &t2, &t3));
  int h[2] = {0, 0};
  MQ_CUDA(c, cudaMemcpyAsync(h, info, 2 * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  MQ_CUDA(c, cudaStreamSynchronize(c->stream));
  t1.collect();
  t2.collect();
  t3.collect();
  c->stats.eig_f32_sweeps = h[0];
  float r;
  memcpy(&r, &h[1], sizeof(float));
  c->stats.eig_f32_off = r;
  c->stats.ms_eig_f32 = t1.total;
  c->stats.ms_eig_refine = t2.total;
  c->stats.ms_eig_jacobi = t3.total;
  return MQ_OK;
}

}  // namespace mq
