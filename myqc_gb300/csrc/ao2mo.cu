// ao2mo.cu -- (ia|jb) four-index transform and MP2 pair sums.
//
// (ia|jb) = sum_{uvld} C_ui C_va C_lj C_db (uv|ld), the quantity the reference
// builds with four naive quarter transforms (src/ao2mo/ao2mo.f90:1306-1439,
// called in the order i, a, j, b at :506-562).  Here the virtual index b goes
// first (nv < no makes the dominant n^4 step cheaper), as four GEMMs over the
// device-resident XX:
//   Y1[uvl,b] = XX[uvl,d] Cb[d,b]                 (n^3 x n) (n x nv2)
//   Y2[uv,j,b] = Y1[uv,l,b] Cj[l,j]  per b         (n^2 x n) (n x no2)
//   Y3[u,a,jb] = Y2[u,v,jb] Ca[v,a]  per jb        (n x n)   (n x nv1)
//   Om[i,ajb] = Ci[u,i]^T Y3[u,ajb]                (no1 x n) (n x nv1 no2 nv2)
// Om(i,a,j,b) has i fastest, the layout of the reference's Om array
// (ao2mo.f90:566-582 writes Om(i,:,j,:) records from it).
//
// MP2 (src/mp2/mp2.f90:79-232): E(AB) = sum_{ijab} (ia|jb)^2 / D and
// E(AA) = sum_{i<j,a<b} [(ia|jb) - (ib|ja)]^2 / D, D = e_i + e_j - e_a - e_b,
// reduced in a fixed order (per-block partials, then one block).
#include "df32.cuh"
#include "internal.h"

namespace mq {

int ao2mo_device(mq_ctx *c, const double *Ci, int no1, const double *Ca, int nv1, const double *Cj, int no2,
                 const double *Cb, int nv2, int precision, double *d_out) {
  const long long n = c->nao;
  if (no1 == 0 || nv1 == 0 || no2 == 0 || nv2 == 0) return MQ_OK;  // empty block (e.g. no beta electrons)
  const int planes = precision == MQ_PREC_SPLIT_BF16X3 ? 3 : 2;
  // the FP64 transform reads the n^4 array (filled from the quartet store if
  // that is what mq_eri_store kept); the split one slices from either
  if (precision == MQ_PREC_FP64) MQ_TRY(ensure_xx_full(c));
  else if (!c->xx_valid && !c->qs.valid) return set_err(c, MQ_ESTATE, "no integrals on the device");
  if (precision == MQ_PREC_FP64) MQ_TRY(join_side(c));
  if (precision != MQ_PREC_FP64)
    return ao2mo_split_device(c, Ci, no1, Ca, nv1, Cj, no2, Cb, nv2, d_out, planes);
  const size_t y1 = (size_t)(n * n * n) * nv2, y2 = (size_t)(n * n) * no2 * nv2, y3 = (size_t)n * nv1 * no2 * nv2;
  double *Y1 = (double *)buf(c, "ao2mo_y1", sizeof(double) * std::max(y1, y3));
  double *Y2 = (double *)buf(c, "ao2mo_y2", sizeof(double) * y2);
  if (!Y1 || !Y2) return MQ_ENOMEM;
  double *Y3 = Y1;  // Y1 is dead once Y2 exists
  MQ_TRY(gemm(c, 'N', 'N', (int)(n * n * n), nv2, (int)n, 1.0, c->d_XX, (int)(n * n * n), Cb, (int)n, 0.0, Y1,
              (int)(n * n * n)));
  MQ_TRY(gemm_strided_batched(c, 'N', 'N', (int)(n * n), no2, (int)n, 1.0, Y1, (int)(n * n), n * n * n, Cj, (int)n,
                              0, 0.0, Y2, (int)(n * n), n * n * no2, nv2));
  MQ_TRY(gemm_strided_batched(c, 'N', 'N', (int)n, nv1, (int)n, 1.0, Y2, (int)n, n * n, Ca, (int)n, 0, 0.0, Y3,
                              (int)n, n * nv1, no2 * nv2));
  MQ_TRY(gemm(c, 'T', 'N', no1, nv1 * no2 * nv2, (int)n, 1.0, Ci, (int)n, Y3, (int)n, 0.0, d_out, no1));
  return MQ_OK;
}

// one thread per (i, a, j); loops over b.  part[2*block] = sum_os, [2*block+1] = sum_ss
__global__ void mp2_partial_kernel(const double *__restrict__ Om, int no1, int nv1, int no2, int nv2,
                                   const double *__restrict__ eo1, const double *__restrict__ ev1,
                                   const double *__restrict__ eo2, const double *__restrict__ ev2, int same_spin,
                                   double *__restrict__ part) {
  __shared__ double s_os[256], s_ss[256];
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long tot = (long long)no1 * nv1 * no2;
  double os = 0.0, ss = 0.0;
  if (idx < tot) {
    const int i = (int)(idx % no1);
    const int a = (int)((idx / no1) % nv1);
    const int j = (int)(idx / ((long long)no1 * nv1));
    const size_t sb = (size_t)no1 * nv1 * no2;  // stride of b
    const double eija = eo1[i] + eo2[j] - ev1[a];
    for (int b = 0; b < nv2; ++b) {
      const double x = Om[idx + sb * b];
      const double inv = 1.0 / (eija - ev2[b]);
      os += x * x * inv;
      if (same_spin && i < j && a < b) {
        const double y = x - Om[i + (size_t)no1 * (b + (size_t)nv1 * j) + sb * a];
        ss += y * y * inv;
      }
    }
  }
  s_os[threadIdx.x] = os;
  s_ss[threadIdx.x] = ss;
  __syncthreads();
  for (int k = blockDim.x / 2; k > 0; k >>= 1) {
    if (threadIdx.x < k) {
      s_os[threadIdx.x] += s_os[threadIdx.x + k];
      s_ss[threadIdx.x] += s_ss[threadIdx.x + k];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = s_os[0];
    part[2 * blockIdx.x + 1] = s_ss[0];
  }
}

// The same pair sums over (ia|jb) from the split-precision transform, whose
// values carry ~2^-24 relative error already: arithmetic on the FP32 pipes
// (GB300's FP64 rate would make the FP64 divide the bottleneck).  Each
// integral is split into float hi + lo (integer operations), squares are
// hi^2 + 2 hi lo, the same-spin difference is (hi - hi') + (lo - lo'), the
// denominators and reciprocals are FP32 (round to nearest: the per-term errors
// are unbiased), the sum over b is FP32 and everything after it FP64.
__global__ void mp2_partial_f32_kernel(const double *__restrict__ Om, int no1, int nv1, int no2, int nv2,
                                       const double *__restrict__ eo1, const double *__restrict__ ev1,
                                       const double *__restrict__ eo2, const double *__restrict__ ev2, int same_spin,
                                       double *__restrict__ part) {
  __shared__ double s_os[256], s_ss[256];
  extern __shared__ float evf[];  // ev2 as floats
  for (int b = threadIdx.x; b < nv2; b += blockDim.x) evf[b] = (float)ev2[b];
  __syncthreads();
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long tot = (long long)no1 * nv1 * no2;
  double os = 0.0, ss = 0.0;
  if (idx < tot) {
    const int i = (int)(idx % no1);
    const int a = (int)((idx / no1) % nv1);
    const int j = (int)(idx / ((long long)no1 * nv1));
    const size_t sb = (size_t)no1 * nv1 * no2;
    const float eija = (float)(eo1[i] + eo2[j] - ev1[a]);
    const bool ssp = same_spin && i < j;
    float fo = 0.f, fs = 0.f;
    // b in runs of MP2_RUN: the run's integrals (and their exchange partners)
    // are loaded before any is used, so a thread has up to 2 MP2_RUN loads in
    // flight; the sums still take b in ascending order
    constexpr int MP2_RUN = 8;
    const double *xpb = Om + i + (size_t)no1 * nv1 * j + sb * a;  // (ib|ja) at xpb[no1 b]
    for (int b0 = 0; b0 < nv2; b0 += MP2_RUN) {
      double xv[MP2_RUN], xpv[MP2_RUN];
#pragma unroll
      for (int u = 0; u < MP2_RUN; ++u) {
        const int b = b0 + u;
        xv[u] = b < nv2 ? __ldcs(Om + idx + sb * b) : 0.0;
        xpv[u] = (b < nv2 && ssp && a < b) ? xpb[(size_t)no1 * b] : 0.0;
      }
#pragma unroll
      for (int u = 0; u < MP2_RUN; ++u) {
        const int b = b0 + u;
        if (b >= nv2) break;
        const float2 x = split_f64(xv[u]);
        const float inv = __frcp_rn(eija - evf[b]);
        fo = fmaf(fmaf(2.f * x.x, x.y, x.x * x.x), inv, fo);
        if (ssp && a < b) {
          const float2 xp = split_f64(xpv[u]);
          const float yh = x.x - xp.x, yl = x.y - xp.y;
          fs = fmaf(fmaf(2.f * yh, yl, yh * yh), inv, fs);
        }
      }
    }
    os = fo;
    ss = fs;
  }
  s_os[threadIdx.x] = os;
  s_ss[threadIdx.x] = ss;
  __syncthreads();
  for (int k = blockDim.x / 2; k > 0; k >>= 1) {
    if (threadIdx.x < k) {
      s_os[threadIdx.x] += s_os[threadIdx.x + k];
      s_ss[threadIdx.x] += s_ss[threadIdx.x + k];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = s_os[0];
    part[2 * blockIdx.x + 1] = s_ss[0];
  }
}

__global__ void mp2_final_kernel(const double *part, int nblk, double *out) {
  __shared__ double s_os[1024], s_ss[1024];
  double os = 0.0, ss = 0.0;
  for (int k = threadIdx.x; k < nblk; k += blockDim.x) {
    os += part[2 * k];
    ss += part[2 * k + 1];
  }
  s_os[threadIdx.x] = os;
  s_ss[threadIdx.x] = ss;
  __syncthreads();
  for (int k = blockDim.x / 2; k > 0; k >>= 1) {
    if (threadIdx.x < k) {
      s_os[threadIdx.x] += s_os[threadIdx.x + k];
      s_ss[threadIdx.x] += s_ss[threadIdx.x + k];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = s_os[0];
    out[1] = s_ss[0];
  }
}

// sums[0] = opposite-spin type sum (all ijab), sums[1] = same-spin antisymmetrised sum
int mp2_pair_sums(mq_ctx *c, const double *d_Om, int no1, int nv1, int no2, int nv2, const double *d_e1,
                  const double *d_e2, int same_spin, double *sums) {
  const long long tot = (long long)no1 * nv1 * no2;
  const int tb = 256;
  const int nblk = (int)((tot + tb - 1) / tb);
  double *part = (double *)buf(c, "mp2_partials", sizeof(double) * (2 * (size_t)nblk + 2));
  if (!part) return MQ_ENOMEM;
  const bool f32 = d_Om == c->d_iajb && c->iajb_precision != MQ_PREC_FP64;  // split-precision (ia|jb)
  cudaEvent_t e0, e1;  // the pair-sum kernels alone (stat "mp2")
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, c->stream);
  if (nblk > 0 && f32)
    mp2_partial_f32_kernel<<<nblk, tb, sizeof(float) * nv2, c->stream>>>(
        d_Om, no1, nv1, no2, nv2, d_e1, d_e1 + no1, d_e2, d_e2 + no2, same_spin, part);
  else if (nblk > 0)
    mp2_partial_kernel<<<nblk, tb, 0, c->stream>>>(d_Om, no1, nv1, no2, nv2, d_e1, d_e1 + no1, d_e2, d_e2 + no2,
                                                   same_spin, part);
  mp2_final_kernel<<<1, 1024, 0, c->stream>>>(part, nblk, part + 2 * (size_t)nblk);
  cudaEventRecord(e1, c->stream);
  c->stats.launches += 2;
  const cudaError_t le = cudaGetLastError();
  const cudaError_t ce = cudaMemcpyAsync(sums, part + 2 * (size_t)nblk, 2 * sizeof(double), cudaMemcpyDeviceToHost,
                                         c->stream);
  const cudaError_t se = cudaStreamSynchronize(c->stream);
  float ms = 0.f;
  if (se == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  MQ_CUDA(c, le);
  MQ_CUDA(c, ce);
  MQ_CUDA(c, se);
  c->stats.ms_mp2 = ms;
  return MQ_OK;
}

int mp2_rhf_device(mq_ctx *c, const double *d_iajb, const double *d_eig, int nocc, int nvir, double *e_out) {
  double s[2];
  MQ_TRY(mp2_pair_sums(c, d_iajb, nocc, nvir, nocc, nvir, d_eig, d_eig, 1, s));
  e_out[0] = s[1];
  e_out[1] = s[0];
  e_out[2] = 2.0 * s[1] + s[0];
  return MQ_OK;
}

}  // namespace mq
