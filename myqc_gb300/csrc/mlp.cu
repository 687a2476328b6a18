// mlp.cu -- the learned density guess's network: a 3-layer MLP
// (nin -> W -> W -> nout, SiLU) with BF16 weights and activations, FP32
// accumulation, trained with Adam.  No reference counterpart (the reference
// starts every SCF from the core Hamiltonian, src/scf/scf.f90:410-512).
//
// Every matrix product is one tensor-core kernel, D[b][m][n] = sum_k
// A[b][m][k] B[b|0][n][k] (A, B K-major BF16, TMA 128-byte-swizzled tiles,
// tcgen05.mma M = 128, N = the whole output width <= 256, FP32 accumulator in
// TMEM), with the layer's pointwise work fused into the epilogue:
//   forward      z = acc + bias, y = SiLU(z)      (z kept in FP32, y in BF16)
//   output       out = acc + bias                  (FP32)
//   backward dX  dz = acc * SiLU'(z_prev)         (BF16)
//   weight grad  acc -> FP32 partial per K-chunk  (split-K over the samples)
// Weight gradients multiply transposed activations and output gradients
// (dW = dZ^T X), with the sample dimension as K cut into chunks, one batch
// entry per chunk; a small kernel sums the chunks.  Bias gradients, the loss
// and its gradient, transposes and the Adam update are elementwise kernels.
// The FP32 master weights stay on the device; Adam writes them and the BF16
// copies W (forward, [n][k]) and W^T (backward, [k][n]).
#include <algorithm>
#include <cmath>
#include <vector>

#include "internal.h"
#include "tc.cuh"

namespace mq {

enum { EPI_BIAS_ACT = 0, EPI_BIAS = 1, EPI_DACT = 2, EPI_F32 = 3 };

struct MlpGemm {
  int M, N, K, batch, ntile, tmem_cols, b_batched;
  const float *bias;       // [N]
  const float *zin;        // EPI_DACT: z of this layer's input, [M][ldz]
  float *zout;             // EPI_BIAS_ACT: z, [M][ldz]
  float *out32;            // EPI_BIAS / EPI_F32: [batch][M][ldo]
  bf16 *out16;             // EPI_BIAS_ACT: y / EPI_DACT: dz, [M][ldo]
  int ldo, ldz;
  long long s_b;           // EPI_F32: batch stride of out32
  int *err;
};

struct MlpMaps {
  CUtensorMap a, b;
};

__device__ __forceinline__ float sigm(float z) { return 1.0f / (1.0f + expf(-z)); }

template <int EPI, int STAGES>
__global__ void __launch_bounds__(GEMM_THREADS, 1) mlp_gemm_kernel(const __grid_constant__ MlpMaps maps, MlpGemm g) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  const int ntile = g.ntile;
  const uint32_t a_bytes = UM * UK * 2, b_bytes = (uint32_t)ntile * UK * 2;
  const uint32_t stage_bytes = a_bytes + b_bytes;
  uint64_t *full = (uint64_t *)(smem + STAGES * stage_bytes);
  uint64_t *empty = full + STAGES;
  uint64_t *acc_full = empty + STAGES;
  uint64_t *acc_empty = acc_full + 1;
  uint64_t *drain = acc_empty + 1;
  uint32_t *tmem_slot = (uint32_t *)(drain + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int mtiles = (g.M + UM - 1) / UM;
  const long long ntiles = (long long)mtiles * g.batch;
  const int kchunks = (g.K + UK - 1) / UK;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(full + s, 1);
      mbar_init(empty + s, 1);
    }
    mbar_init(acc_full, 1);
    mbar_init(acc_empty, 4);
    mbar_init(drain, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    __syncwarp();
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(tmem_slot)),
                 "r"(g.tmem_cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *(volatile uint32_t *)tmem_slot;

  if (warp == 0) {
    if (lane == 0) {  // TMA producer
      int s = 0;
      uint32_t ph = 1;
      unsigned armed = 0, armed_par = 0;
      for (long long t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int mt = (int)(t % mtiles), bt = (int)(t / mtiles);
        for (int kc = 0; kc < kchunks; ++kc) {
          if (!mbar_wait(empty + s, ph, g.err)) goto prod_exit;
          uint8_t *st = smem + s * stage_bytes;
          mbar_expect_tx(full + s, stage_bytes);
          tma_load_3d(st, &maps.a, full + s, kc * UK, mt * UM, bt);
          tma_load_3d(st + a_bytes, &maps.b, full + s, kc * UK, 0, g.b_batched ? bt : 0);
          armed |= 1u << s;
          armed_par = (armed_par & ~(1u << s)) | ((ph ^ 1u) << s);
          if (++s == STAGES) {
            s = 0;
            ph ^= 1;
          }
        }
      }
    prod_exit:
      for (int k = 0; k < STAGES; ++k)
        if (armed & (1u << k)) mbar_drain(full + k, (armed_par >> k) & 1u);
    }
  } else if (warp == 1) {
    if (lane == 0) {  // MMA issuer: D F32, A/B BF16 K-major, N >> 3 at bit 17, M >> 4 at bit 24
      const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(ntile >> 3) << 17) |
                             ((uint32_t)(UM >> 4) << 24);
      int s = 0;
      uint32_t ph = 0, acc_ph = 1;
      bool ok = true;
      for (long long t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
        if (!mbar_wait(acc_empty, acc_ph, g.err)) break;
        acc_ph ^= 1;
        tc_fence_after();
        for (int kc = 0; kc < kchunks; ++kc) {
          if (!mbar_wait(full + s, ph, g.err)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t base = su32(smem + s * stage_bytes);
#pragma unroll
          for (int kk = 0; kk < UK / 16; ++kk) {
            const uint32_t off = kk * 32;
            umma(tmem, sdesc(base + off), sdesc(base + a_bytes + off), idesc, (kc == 0 && kk == 0) ? 0u : 1u);
          }
          umma_commit(empty + s);
          if (++s == STAGES) {
            s = 0;
            ph ^= 1;
          }
        }
        if (ok) umma_commit(acc_full);
      }
      umma_commit(drain);
      mbar_drain(drain, 0);
    }
  } else {  // epilogue: warps 2..5 own TMEM lane quadrants 2, 3, 0, 1
    const int q = warp & 3;
    const int row = q * 32 + lane;
    uint32_t acc_ph = 0;
    for (long long t = blockIdx.x; t < ntiles; t += gridDim.x) {
      const int mt = (int)(t % mtiles), bt = (int)(t / mtiles);
      int ok = 0;
      if (lane == 0) ok = mbar_wait(acc_full, acc_ph, g.err);
      ok = __shfl_sync(0xffffffffu, ok, 0);
      if (!ok) break;
      acc_ph ^= 1;
      tc_fence_after();
      const long long m = (long long)mt * UM + row;
      const bool live = m < g.M;
      for (int c0 = 0; c0 < ntile; c0 += 16) {
        float v[16];
        tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)c0, v);
        if (!live) continue;
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          const int n = c0 + i;
          if (n >= g.N) break;
          if (EPI == EPI_BIAS_ACT) {
            const float z = v[i] + g.bias[n];
            g.zout[m * g.ldz + n] = z;
            g.out16[m * g.ldo + n] = __float2bfloat16_rn(z * sigm(z));
          } else if (EPI == EPI_BIAS) {
            g.out32[m * g.ldo + n] = v[i] + g.bias[n];
          } else if (EPI == EPI_DACT) {
            const float z = g.zin[m * g.ldz + n], sg = sigm(z);
            g.out16[m * g.ldo + n] = __float2bfloat16_rn(v[i] * sg * (1.0f + z * (1.0f - sg)));
          } else {
            g.out32[(long long)bt * g.s_b + m * g.ldo + n] = v[i];
          }
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(acc_empty);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    __syncwarp();
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(g.tmem_cols) : "memory");
  }
}

// ---------------------------------------------------------------- pointwise
// src (rows x cols, leading dimension lds) -> dst in chunk-major transposed
// layout: sample s, column c at (s / kc) * cols * kc + c * kc + s % kc, so that
// each chunk of kc samples is a contiguous cols x kc K-major operand
__global__ void transpose_chunked_kernel(const bf16 *__restrict__ src, int rows, int cols, int lds, int kc,
                                         bf16 *__restrict__ dst) {
  __shared__ bf16 tile[32][33];
  const int r0 = blockIdx.y * 32, c0 = blockIdx.x * 32;
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    const int r = r0 + i, c = c0 + threadIdx.x;
    tile[i][threadIdx.x] = (r < rows && c < cols) ? src[(size_t)r * lds + c] : __float2bfloat16_rn(0.f);
  }
  __syncthreads();
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    const int c = c0 + i, r = r0 + threadIdx.x;
    if (c < cols && r < rows) dst[(size_t)(r / kc) * cols * kc + (size_t)c * kc + r % kc] = tile[threadIdx.x][i];
  }
}

// FP32 rows -> BF16 rows of width ldd (zero padded)
__global__ void to_bf16_kernel(const float *__restrict__ src, long long rows, int cols, int lds,
                               bf16 *__restrict__ dst, int ldd) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= rows * ldd) return;
  const long long r = i / ldd;
  const int c = (int)(i % ldd);
  dst[i] = __float2bfloat16_rn(c < cols ? src[r * lds + c] : 0.f);
}

// rows of src picked by idx -> dst (dataset minibatch gather)
__global__ void gather_rows_kernel(const bf16 *__restrict__ src, const float *__restrict__ t,
                                   const float *__restrict__ w, const int *__restrict__ idx, int rows, int ld_in,
                                   int nout, bf16 *__restrict__ xb, float *__restrict__ tb, float *__restrict__ wb) {
  const int r = blockIdx.x;
  if (r >= rows) return;
  const long long s = idx[r];
  for (int c = threadIdx.x; c < ld_in; c += blockDim.x) xb[(size_t)r * ld_in + c] = src[s * ld_in + c];
  for (int c = threadIdx.x; c < nout; c += blockDim.x) {
    tb[(size_t)r * nout + c] = t[s * nout + c];
    wb[(size_t)r * nout + c] = w[s * nout + c];
  }
}

// weighted squared error: loss partials per block; dy = 2 w (y - t) / wsum as
// BF16 rows of width ldd (zero padded)
__global__ void loss_kernel(const float *__restrict__ y, const float *__restrict__ t, const float *__restrict__ w,
                            int rows, int nout, float inv_wsum, bf16 *__restrict__ dy, int ldd,
                            double *__restrict__ partial) {
  __shared__ double red[32];
  double acc = 0.0;
  const long long total = (long long)rows * ldd;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
    const long long r = i / ldd;
    const int c = (int)(i % ldd);
    float g = 0.f;
    if (c < nout) {
      const long long j = r * nout + c;
      const float d = y[j] - t[j];
      acc += (double)w[j] * d * d;
      g = 2.f * w[j] * d * inv_wsum;
    }
    dy[i] = __float2bfloat16_rn(g);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += red[k];
    partial[blockIdx.x] = s;
  }
}

// column sums of a BF16 [rows][ld] matrix (bias gradient), one block per column
__global__ void colsum_kernel(const bf16 *__restrict__ a, int rows, int ld, float *__restrict__ out) {
  __shared__ float red[32];
  const int c = blockIdx.x;
  float s = 0.f;
  for (int r = threadIdx.x; r < rows; r += blockDim.x) s += __bfloat162float(a[(size_t)r * ld + c]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.f;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += red[k];
    out[c] = t;
  }
}

// out[i] = sum_b part[b][i] (fixed order)
__global__ void chunk_sum_kernel(const float *__restrict__ part, int nchunk, long long stride, long long n,
                                 float *__restrict__ out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float s = 0.f;
  for (int b = 0; b < nchunk; ++b) s += part[b * stride + i];
  out[i] = s;
}

// Adam on one layer: W (nout x nin, FP32 master), b; writes BF16 W [nout][ldw]
// and W^T [nin][ldt] (zero padding beyond the real sizes is left as set up)
__global__ void adam_kernel(float *__restrict__ W, float *__restrict__ mW, float *__restrict__ vW,
                            const float *__restrict__ gW, int nout, int nin, float *__restrict__ b,
                            float *__restrict__ mb, float *__restrict__ vb, const float *__restrict__ gb, float lr,
                            float b1, float b2, float eps, float c1, float c2, bf16 *__restrict__ Wb, int ldw,
                            bf16 *__restrict__ Wt, int ldt) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long nw = (long long)nout * nin;
  if (i < nw) {
    const float g = gW[i];
    const float m = b1 * mW[i] + (1.f - b1) * g, v = b2 * vW[i] + (1.f - b2) * g * g;
    mW[i] = m;
    vW[i] = v;
    const float w = W[i] - lr * (m * c1) / (sqrtf(v * c2) + eps);
    W[i] = w;
    const int o = (int)(i / nin), k = (int)(i % nin);
    Wb[(size_t)o * ldw + k] = __float2bfloat16_rn(w);
    Wt[(size_t)k * ldt + o] = __float2bfloat16_rn(w);
  } else if (i < nw + nout) {
    const int o = (int)(i - nw);
    const float g = gb[o];
    const float m = b1 * mb[o] + (1.f - b1) * g, v = b2 * vb[o] + (1.f - b2) * g * g;
    mb[o] = m;
    vb[o] = v;
    b[o] -= lr * (m * c1) / (sqrtf(v * c2) + eps);
  }
}

// BF16 copies of a layer's FP32 weights (after parameters are set)
__global__ void weights_bf16_kernel(const float *__restrict__ W, int nout, int nin, bf16 *__restrict__ Wb, int ldw,
                                    bf16 *__restrict__ Wt, int ldt) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)nout * nin) return;
  const int o = (int)(i / nin), k = (int)(i % nin);
  Wb[(size_t)o * ldw + k] = __float2bfloat16_rn(W[i]);
  Wt[(size_t)k * ldt + o] = __float2bfloat16_rn(W[i]);
}

// ---------------------------------------------------------------- host side
static int pad64(int x) { return (x + 63) / 64 * 64; }

// tensor map of a BF16 operand: `kdim` elements along K (contiguous), `rows`
// rows `row_stride` elements apart, `batch` entries `batch_stride` apart
static int map_general(mq_ctx *c, CUtensorMap *m, const bf16 *ptr, long long kdim, long long rows,
                       long long row_stride, long long batch, long long batch_stride, int box_rows) {
  auto fn = encode_fn();
  if (!fn) return set_err(c, MQ_ECUDA, "cuTensorMapEncodeTiled unavailable");
  if (batch == 1) batch_stride = rows * row_stride;
  if ((row_stride * 2) % 16 || (batch_stride * 2) % 16 || ((uintptr_t)ptr & 15))
    return set_err(c, MQ_EINVAL, "MLP operand not 16-byte aligned");
  cuuint64_t dims[3] = {(cuuint64_t)kdim, (cuuint64_t)rows, (cuuint64_t)batch};
  cuuint64_t strides[2] = {(cuuint64_t)row_stride * 2, (cuuint64_t)batch_stride * 2};
  cuuint32_t box[3] = {(cuuint32_t)UK, (cuuint32_t)box_rows, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, (void *)ptr, dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return set_err(c, MQ_ECUDA, "cuTensorMapEncodeTiled failed");
  return MQ_OK;
}

struct GemmOperand {
  const bf16 *ptr;
  long long kdim, rows, row_stride, batch, batch_stride;
};

template <int EPI>
static int mlp_gemm(mq_ctx *c, const GemmOperand &A, const GemmOperand &B, MlpGemm g) {
  if (g.N <= 0 || g.M <= 0) return MQ_OK;
  if (g.N > 256) return set_err(c, MQ_EINVAL, "MLP GEMM: N > 256");
  g.ntile = (g.N + 15) / 16 * 16;
  MlpMaps maps;
  MQ_TRY(map_general(c, &maps.a, A.ptr, A.kdim, A.rows, A.row_stride, A.batch, A.batch_stride, UM));
  MQ_TRY(map_general(c, &maps.b, B.ptr, B.kdim, B.rows, B.row_stride, B.batch, B.batch_stride, g.ntile));
  g.K = (int)A.kdim;
  g.batch = (int)A.batch;
  g.b_batched = B.batch > 1;
  int cols = 32;
  while (cols < g.ntile) cols <<= 1;
  g.tmem_cols = cols;
  const size_t stage = (size_t)UM * UK * 2 + (size_t)g.ntile * UK * 2;
  const size_t limit = 227 * 1024 - 1024 - 256;
  const int stages = limit >= 4 * stage ? 4 : (limit >= 3 * stage ? 3 : 2);
  const size_t smem = stages * stage + 1024 + 256;
  int sms = 148;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
  const long long tiles = (long long)(g.M + UM - 1) / UM * g.batch;
  const int grid = (int)std::min<long long>(tiles, sms);
  auto kern = stages == 4 ? mlp_gemm_kernel<EPI, 4> : (stages == 3 ? mlp_gemm_kernel<EPI, 3> : mlp_gemm_kernel<EPI, 2>);
  MQ_CUDA(c, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  kern<<<grid, GEMM_THREADS, smem, c->stream>>>(maps, g);
  c->stats.launches += 1;
  MQ_CUDA(c, cudaGetLastError());
  return MQ_OK;
}

// The network's device state.  Layer l maps d[l] -> d[l+1]; K widths padded
// to multiples of 64 (kp), output widths of hidden layers are the next kp.
struct Mlp {
  int d[4] = {0, 0, 0, 0}, kp[4] = {0, 0, 0, 0};
  int step = 0;
  float *W[3], *b[3], *mW[3], *vW[3], *mb[3], *vb[3], *gW[3], *gb[3];
  bf16 *Wb[3], *Wt[3];
  // dataset (training)
  long long nsamp = 0;
  bf16 *X = nullptr;
  float *T = nullptr, *Wt8 = nullptr;
  double wsum = 0.0;
};

static Mlp *mlp_of(mq_ctx *c) { return (Mlp *)c->mlp; }

static int mark_params(mq_ctx *c);

int mlp_init(mq_ctx *c, int nin, int width, int nout) {
  if (nin <= 0 || width <= 0 || nout <= 0 || width > 256 || nout > 256 || nin % 8)
    return set_err(c, MQ_EINVAL, "MLP sizes: width and nout <= 256, nin a multiple of 8");
  delete mlp_of(c);
  Mlp *m = new Mlp();
  c->mlp = m;
  m->d[0] = nin;
  m->d[1] = m->d[2] = width;
  m->d[3] = nout;
  for (int l = 0; l < 4; ++l) m->kp[l] = pad64(m->d[l]);
  size_t tot = 0;
  for (int l = 0; l < 3; ++l) tot += (size_t)m->d[l + 1] * m->d[l] + m->d[l + 1];
  float *p = (float *)buf(c, "mlp_params", tot * 5 * sizeof(float));  // W b | m | v | grads | spare
  if (!p) return MQ_ENOMEM;
  MQ_CUDA(c, cudaMemsetAsync(p, 0, tot * 5 * sizeof(float), c->stream));
  size_t bf = 0;
  for (int l = 0; l < 3; ++l) bf += (size_t)m->d[l + 1] * m->kp[l] + (size_t)m->d[l] * m->kp[l + 1];
  bf16 *q = (bf16 *)buf(c, "mlp_bf16", bf * sizeof(bf16) + 64);
  int *err = (int *)buf(c, "mlp_err", 64);
  if (!q || !err) return MQ_ENOMEM;
  MQ_CUDA(c, cudaMemsetAsync(err, 0, 64, c->stream));  // the GEMMs' time-out flag
  MQ_CUDA(c, cudaMemsetAsync(q, 0, bf * sizeof(bf16) + 64, c->stream));
  for (int l = 0; l < 3; ++l) {
    const size_t nw = (size_t)m->d[l + 1] * m->d[l], nb = m->d[l + 1];
    m->W[l] = p;
    m->b[l] = p + nw;
    m->mW[l] = p + tot;
    m->mb[l] = p + tot + nw;
    m->vW[l] = p + 2 * tot;
    m->vb[l] = p + 2 * tot + nw;
    m->gW[l] = p + 3 * tot;
    m->gb[l] = p + 3 * tot + nw;
    p += nw + nb;
    m->Wb[l] = q;
    q += (size_t)m->d[l + 1] * m->kp[l];
    m->Wt[l] = q;
    q += (size_t)m->d[l] * m->kp[l + 1];
  }
  return mark_params(c);  // the zeroed parameters
}

int mlp_dims(mq_ctx *c, int dims[4]) {
  Mlp *m = mlp_of(c);
  if (!m) return set_err(c, MQ_ESTATE, "no MLP (mq_mlp_init)");
  for (int k = 0; k < 4; ++k) dims[k] = m->d[k];
  return MQ_OK;
}

int mlp_param_count(mq_ctx *c) {
  Mlp *m = mlp_of(c);
  if (!m) return 0;
  int n = 0;
  for (int l = 0; l < 3; ++l) n += m->d[l + 1] * m->d[l] + m->d[l + 1];
  return n;
}

int mlp_set_params(mq_ctx *c, const float *h) {
  Mlp *m = mlp_of(c);
  if (!m) return set_err(c, MQ_ESTATE, "no MLP (mq_mlp_init)");
  const int n = mlp_param_count(c);
  MQ_CUDA(c, cudaMemcpyAsync(m->W[0], h, n * sizeof(float), cudaMemcpyHostToDevice, c->stream));
  MQ_CUDA(c, cudaMemsetAsync(m->mW[0], 0, 2 * (size_t)n * sizeof(float), c->stream));
  m->step = 0;
  for (int l = 0; l < 3; ++l) {
    const long long nw = (long long)m->d[l + 1] * m->d[l];
    weights_bf16_kernel<<<(unsigned)((nw + 255) / 256), 256, 0, c->stream>>>(m->W[l], m->d[l + 1], m->d[l], m->Wb[l],
                                                                             m->kp[l], m->Wt[l], m->kp[l + 1]);
  }
  c->stats.launches += 3;
  MQ_CUDA(c, cudaGetLastError());
  return mark_params(c);
}

int mlp_get_params(mq_ctx *c, float *h) {
  Mlp *m = mlp_of(c);
  if (!m) return set_err(c, MQ_ESTATE, "no MLP (mq_mlp_init)");
  MQ_CUDA(c, cudaMemcpyAsync(h, m->W[0], mlp_param_count(c) * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
  MQ_CUDA(c, cudaStreamSynchronize(c->stream));
  return MQ_OK;
}

// Activations of a batch of `rows` samples: row-major BF16 operands (rows
// rounded up to 128), their chunk-major transposes for the weight gradients
// (rows rounded up to the split-K chunk, zero beyond `rows`), FP32 z and
// outputs, and scratch for split-K and loss partials.
constexpr int KCHUNK = 2048;
struct Acts {
  bf16 *x, *y1, *y2, *dy3, *dz2, *dz1, *t_x, *t_y1, *t_y2, *t_dy3, *t_dz2, *t_dz1;
  float *z1, *z2, *out, *part32;
  double *loss_part;
  int rows, rp;  // rp: rows rounded up to KCHUNK
  size_t t_elems;
};

static int acts_alloc(mq_ctx *c, Mlp *m, int rows, Acts &a) {
  const size_t R = ((size_t)rows + 127) / 128 * 128;
  const size_t Rp = ((size_t)rows + KCHUNK - 1) / KCHUNK * KCHUNK;
  a.rows = rows;
  a.rp = (int)Rp;
  const int k0 = m->kp[0], k1 = m->kp[1], k2 = m->kp[2], k3 = m->kp[3];
  const size_t rowmajor = R * (size_t)(k0 + k1 + k2 + k3 + k2 + k1);
  const int d0 = m->d[0], d1 = m->d[1], d2 = m->d[2], d3 = m->d[3];
  a.t_elems = Rp * (size_t)(d0 + d1 + d2 + d3 + d2 + d1);
  bf16 *b = (bf16 *)buf(c, "mlp_acts16", (rowmajor + a.t_elems) * sizeof(bf16) + 256);
  const size_t nchunk = Rp / KCHUNK;
  size_t maxw = 0;
  for (int l = 0; l < 3; ++l) maxw = std::max(maxw, (size_t)m->d[l + 1] * m->d[l]);
  float *f = (float *)buf(c, "mlp_acts32", (R * (size_t)(d1 + d2 + d3) + nchunk * maxw) * sizeof(float) +
                                               512 * sizeof(double) + 256);
  if (!b || !f) return MQ_ENOMEM;
  MQ_CUDA(c, cudaMemsetAsync(b, 0, rowmajor * sizeof(bf16), c->stream));  // K padding columns stay zero
  a.x = b;
  a.y1 = a.x + R * k0;
  a.y2 = a.y1 + R * k1;
  a.dy3 = a.y2 + R * k2;
  a.dz2 = a.dy3 + R * k3;
  a.dz1 = a.dz2 + R * k2;
  bf16 *t = a.dz1 + R * k1;
  a.t_x = t;
  a.t_y1 = a.t_x + Rp * d0;
  a.t_y2 = a.t_y1 + Rp * d1;
  a.t_dy3 = a.t_y2 + Rp * d2;
  a.t_dz2 = a.t_dy3 + Rp * d3;
  a.t_dz1 = a.t_dz2 + Rp * d2;
  a.z1 = f;
  a.z2 = a.z1 + R * d1;
  a.out = a.z2 + R * d2;
  a.loss_part = (double *)(a.out + R * d3 + (R * d3) % 2);
  a.part32 = (float *)(a.loss_part + 512);
  return MQ_OK;
}

static int forward(mq_ctx *c, Mlp *m, Acts &a) {
  const int R = a.rows;
  MlpGemm g{};
  g.err = (int *)buf(c, "mlp_err", 64);
  if (!g.err) return MQ_ENOMEM;
  // layer 1: z1 = x W1^T + b1, y1 = SiLU(z1)
  g.M = R;
  g.N = m->d[1];
  g.bias = m->b[0];
  g.zout = a.z1;
  g.ldz = m->d[1];
  g.out16 = a.y1;
  g.ldo = m->kp[1];
  MQ_TRY(mlp_gemm<EPI_BIAS_ACT>(c, {a.x, m->kp[0], R, m->kp[0], 1, 0}, {m->Wb[0], m->kp[0], m->d[1], m->kp[0], 1, 0}, g));
  // layer 2
  g.N = m->d[2];
  g.bias = m->b[1];
  g.zout = a.z2;
  g.ldz = m->d[2];
  g.out16 = a.y2;
  g.ldo = m->kp[2];
  MQ_TRY(mlp_gemm<EPI_BIAS_ACT>(c, {a.y1, m->kp[1], R, m->kp[1], 1, 0}, {m->Wb[1], m->kp[1], m->d[2], m->kp[1], 1, 0}, g));
  // layer 3: out = y2 W3^T + b3
  g.N = m->d[3];
  g.bias = m->b[2];
  g.out32 = a.out;
  g.ldo = m->d[3];
  MQ_TRY(mlp_gemm<EPI_BIAS>(c, {a.y2, m->kp[2], R, m->kp[2], 1, 0}, {m->Wb[2], m->kp[2], m->d[3], m->kp[2], 1, 0}, g));
  return MQ_OK;
}

static int transpose(mq_ctx *c, const bf16 *src, int rows, int cols, int lds, bf16 *dst) {
  dim3 grid((cols + 31) / 32, (rows + 31) / 32), block(32, 8);
  transpose_chunked_kernel<<<grid, block, 0, c->stream>>>(src, rows, cols, lds, KCHUNK, dst);
  c->stats.launches += 1;
  MQ_CUDA(c, cudaGetLastError());
  return MQ_OK;
}

// dW[l] = dZ^T Y (split-K over chunks of KCHUNK samples, one batch entry per
// chunk of the chunk-major transposes), db[l] = column sums of dZ
static int weight_grad(mq_ctx *c, Mlp *m, int l, const bf16 *t_dz, const bf16 *t_y, const bf16 *dz, int ld_dz, int R,
                       int Rp, float *part) {
  const int nout = m->d[l + 1], nin = m->d[l];
  const int nchunk = Rp / KCHUNK;
  MlpGemm g{};
  g.err = (int *)buf(c, "mlp_err", 64);
  g.M = nout;
  g.N = nin;
  g.out32 = part;
  g.ldo = nin;
  g.s_b = (long long)nout * nin;
  MQ_TRY(mlp_gemm<EPI_F32>(c, {t_dz, KCHUNK, nout, KCHUNK, nchunk, (long long)nout * KCHUNK},
                           {t_y, KCHUNK, nin, KCHUNK, nchunk, (long long)nin * KCHUNK}, g));
  const long long n = (long long)nout * nin;
  chunk_sum_kernel<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(part, nchunk, n, n, m->gW[l]);
  colsum_kernel<<<nout, 256, 0, c->stream>>>(dz, R, ld_dz, m->gb[l]);
  c->stats.launches += 2;
  MQ_CUDA(c, cudaGetLastError());
  return MQ_OK;
}

// forward + loss + backward on the batch in a (x filled); tb, wb: targets and
// loss weights [R][nout]; gradients into m->gW/gb; loss partials summed on the host
static int backward(mq_ctx *c, Mlp *m, Acts &a, const float *tb, const float *wb, double wsum, double *loss) {
  const int R = a.rows;
  MQ_TRY(forward(c, m, a));
  const int nb = 256;
  loss_kernel<<<nb, 256, 0, c->stream>>>(a.out, tb, wb, R, m->d[3], (float)(1.0 / wsum), a.dy3, m->kp[3], a.loss_part);
  c->stats.launches += 1;
  std::vector<double> part(nb);
  MQ_CUDA(c, cudaMemcpyAsync(part.data(), a.loss_part, nb * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  MlpGemm g{};
  g.err = (int *)buf(c, "mlp_err", 64);
  // dz2 = (dy3 W3) * SiLU'(z2)
  g.M = R;
  g.N = m->d[2];
  g.zin = a.z2;
  g.ldz = m->d[2];
  g.out16 = a.dz2;
  g.ldo = m->kp[2];
  MQ_TRY(mlp_gemm<EPI_DACT>(c, {a.dy3, m->kp[3], R, m->kp[3], 1, 0}, {m->Wt[2], m->kp[3], m->d[2], m->kp[3], 1, 0}, g));
  // dz1 = (dz2 W2) * SiLU'(z1)
  g.N = m->d[1];
  g.zin = a.z1;
  g.ldz = m->d[1];
  g.out16 = a.dz1;
  g.ldo = m->kp[1];
  MQ_TRY(mlp_gemm<EPI_DACT>(c, {a.dz2, m->kp[2], R, m->kp[2], 1, 0}, {m->Wt[1], m->kp[2], m->d[1], m->kp[2], 1, 0}, g));
  // chunk-major transposes (zero beyond the batch's rows) and the weight gradients
  MQ_CUDA(c, cudaMemsetAsync(a.t_x, 0, a.t_elems * sizeof(bf16), c->stream));
  MQ_TRY(transpose(c, a.x, R, m->d[0], m->kp[0], a.t_x));
  MQ_TRY(transpose(c, a.y1, R, m->d[1], m->kp[1], a.t_y1));
  MQ_TRY(transpose(c, a.y2, R, m->d[2], m->kp[2], a.t_y2));
  MQ_TRY(transpose(c, a.dy3, R, m->d[3], m->kp[3], a.t_dy3));
  MQ_TRY(transpose(c, a.dz2, R, m->d[2], m->kp[2], a.t_dz2));
  MQ_TRY(transpose(c, a.dz1, R, m->d[1], m->kp[1], a.t_dz1));
  MQ_TRY(weight_grad(c, m, 2, a.t_dy3, a.t_y2, a.dy3, m->kp[3], R, a.rp, a.part32));
  MQ_TRY(weight_grad(c, m, 1, a.t_dz2, a.t_y1, a.dz2, m->kp[2], R, a.rp, a.part32));
  MQ_TRY(weight_grad(c, m, 0, a.t_dz1, a.t_x, a.dz1, m->kp[1], R, a.rp, a.part32));
  MQ_CUDA(c, cudaStreamSynchronize(c->stream));
  int herr = 0;
  MQ_CUDA(c, cudaMemcpy(&herr, g.err, sizeof(int), cudaMemcpyDeviceToHost));
  if (herr) return set_err(c, MQ_ETIMEOUT, "MLP GEMM wait timed out");
  double s = 0.0;
  for (double v : part) s += v;
  *loss = s / wsum;
  return MQ_OK;
}

static int adam(mq_ctx *c, Mlp *m, float lr) {
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  m->step += 1;
  const float c1 = 1.0f / (1.0f - powf(b1, (float)m->step)), c2 = 1.0f / (1.0f - powf(b2, (float)m->step));
  for (int l = 0; l < 3; ++l) {
    const long long n = (long long)m->d[l + 1] * m->d[l] + m->d[l + 1];
    adam_kernel<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(
        m->W[l], m->mW[l], m->vW[l], m->gW[l], m->d[l + 1], m->d[l], m->b[l], m->mb[l], m->vb[l], m->gb[l], lr, b1, b2,
        eps, c1, c2, m->Wb[l], m->kp[l], m->Wt[l], m->kp[l + 1]);
  }
  c->stats.launches += 3;
  MQ_CUDA(c, cudaGetLastError());
  return MQ_OK;
}

static int upload_x(mq_ctx *c, Mlp *m, const float *X, int rows, Acts &a) {
  float *tmp = (float *)buf(c, "mlp_xin", (size_t)rows * m->d[0] * sizeof(float) + 16);
  if (!tmp) return MQ_ENOMEM;
  MQ_CUDA(c, cudaMemcpyAsync(tmp, X, (size_t)rows * m->d[0] * sizeof(float), cudaMemcpyHostToDevice, c->stream));
  const long long n = (long long)rows * m->kp[0];
  to_bf16_kernel<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(tmp, rows, m->d[0], m->d[0], a.x, m->kp[0]);
  c->stats.launches += 1;
  MQ_CUDA(c, cudaGetLastError());
  return MQ_OK;
}

// Parameters written on the main stream: later forward passes on the aux
// stream start after this point, not after the main stream's later work.
static int mark_params(mq_ctx *c) {
  if (!c->ev_params) MQ_CUDA(c, cudaEventCreateWithFlags(&c->ev_params, cudaEventDisableTiming));
  MQ_CUDA(c, cudaEventRecord(c->ev_params, c->stream));
  return MQ_OK;
}

static int forward_on_stream(mq_ctx *c, Mlp *m, int rows, const float *X, float *Y) {
  Acts a;
  MQ_TRY(acts_alloc(c, m, rows, a));
  MQ_TRY(upload_x(c, m, X, rows, a));
  MQ_TRY(forward(c, m, a));
  MQ_CUDA(c, cudaMemcpyAsync(Y, a.out, (size_t)rows * m->d[3] * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
  MQ_CUDA(c, cudaStreamSynchronize(c->stream));
  return MQ_OK;
}

// The forward pass of rows feature vectors already on the device (FP32, rows x
// nin), on the context's stream; *dY points at the rows x nout outputs (FP32,
// valid until the next network call).
int mlp_forward_device(mq_ctx *c, int rows, const float *dX, float **dY) {
  Mlp *m = mlp_of(c);
  if (!m) return set_err(c, MQ_ESTATE, "no MLP (mq_mlp_init)");
  if (rows <= 0) return set_err(c, MQ_EINVAL, "network forward: no rows");
  if (!c->ev_params) MQ_TRY(mark_params(c));
  MQ_CUDA(c, cudaStreamWaitEvent(c->stream, c->ev_params, 0));
  Acts a;
  MQ_TRY(acts_alloc(c, m, rows, a));
  const long long n = (long long)rows * m->kp[0];
  to_bf16_kernel<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(dX, rows, m->d[0], m->d[0], a.x, m->kp[0]);
  c->stats.launches += 1;
  MQ_CUDA(c, cudaGetLastError());
  MQ_TRY(forward(c, m, a));
  *dY = a.out;
  return MQ_OK;
}

// The forward pass runs on the aux stream (highest priority), ordered after
// the last parameter write only: a guess evaluated while the integral pass is
// queued on the main stream returns without waiting for it.  The network's
// activation buffers are used by this call alone, which returns synchronised.
int mlp_forward(mq_ctx *c, int rows, const float *X, float *Y) {
  Mlp *m = mlp_of(c);
  if (!m) return set_err(c, MQ_ESTATE, "no MLP (mq_mlp_init)");
  if (rows <= 0) return MQ_OK;
  MQ_TRY(ensure_aux(c));
  if (!c->ev_params) MQ_TRY(mark_params(c));
  MQ_CUDA(c, cudaStreamWaitEvent(c->aux, c->ev_params, 0));
  cudaStream_t main = c->stream;
  c->stream = c->aux;
  const int rc = forward_on_stream(c, m, rows, X, Y);
  c->stream = main;
  return rc;
}

int mlp_grad(mq_ctx *c, int rows, const float *X, const float *T, const float *Wl, float *grads, double *loss) {
  Mlp *m = mlp_of(c);
  if (!m) return set_err(c, MQ_ESTATE, "no MLP (mq_mlp_init)");
  Acts a;
  MQ_TRY(acts_alloc(c, m, rows, a));
  MQ_TRY(upload_x(c, m, X, rows, a));
  const size_t nt = (size_t)rows * m->d[3];
  float *tw = (float *)buf(c, "mlp_tw", 2 * nt * sizeof(float) + 16);
  if (!tw) return MQ_ENOMEM;
  MQ_CUDA(c, cudaMemcpyAsync(tw, T, nt * sizeof(float), cudaMemcpyHostToDevice, c->stream));
  MQ_CUDA(c, cudaMemcpyAsync(tw + nt, Wl, nt * sizeof(float), cudaMemcpyHostToDevice, c->stream));
  double wsum = 0.0;
  for (size_t i = 0; i < nt; ++i) wsum += Wl[i];
  MQ_TRY(backward(c, m, a, tw, tw + nt, wsum > 0 ? wsum : 1.0, loss));
  // packed like the parameters: gW then gb per layer
  float *dst = grads;
  for (int l = 0; l < 3; ++l) {
    const size_t nw = (size_t)m->d[l + 1] * m->d[l];
    MQ_CUDA(c, cudaMemcpy(dst, m->gW[l], nw * sizeof(float), cudaMemcpyDeviceToHost));
    MQ_CUDA(c, cudaMemcpy(dst + nw, m->gb[l], m->d[l + 1] * sizeof(float), cudaMemcpyDeviceToHost));
    dst += nw + m->d[l + 1];
  }
  return MQ_OK;
}

int mlp_set_data(mq_ctx *c, long long n, const float *X, const float *T, const float *Wl) {
  Mlp *m = mlp_of(c);
  if (!m) return set_err(c, MQ_ESTATE, "no MLP (mq_mlp_init)");
  m->nsamp = n;
  m->X = (bf16 *)buf(c, "mlp_data_x", (size_t)n * m->kp[0] * sizeof(bf16) + 16);
  m->T = (float *)buf(c, "mlp_data_t", (size_t)n * m->d[3] * sizeof(float) + 16);
  m->Wt8 = (float *)buf(c, "mlp_data_w", (size_t)n * m->d[3] * sizeof(float) + 16);
  if (!m->X || !m->T || !m->Wt8) return MQ_ENOMEM;
  // features in slices through a staging buffer
  const long long step = 1 << 20;
  float *tmp = (float *)buf(c, "mlp_xin", (size_t)step * m->d[0] * sizeof(float) + 16);
  if (!tmp) return MQ_ENOMEM;
  for (long long r0 = 0; r0 < n; r0 += step) {
    const long long r = std::min(step, n - r0);
    MQ_CUDA(c, cudaMemcpyAsync(tmp, X + r0 * m->d[0], (size_t)r * m->d[0] * sizeof(float), cudaMemcpyHostToDevice,
                               c->stream));
    const long long e = r * m->kp[0];
    to_bf16_kernel<<<(unsigned)((e + 255) / 256), 256, 0, c->stream>>>(tmp, r, m->d[0], m->d[0],
                                                                       m->X + r0 * m->kp[0], m->kp[0]);
    MQ_CUDA(c, cudaStreamSynchronize(c->stream));
  }
  MQ_CUDA(c, cudaMemcpyAsync(m->T, T, (size_t)n * m->d[3] * sizeof(float), cudaMemcpyHostToDevice, c->stream));
  MQ_CUDA(c, cudaMemcpyAsync(m->Wt8, Wl, (size_t)n * m->d[3] * sizeof(float), cudaMemcpyHostToDevice, c->stream));
  MQ_CUDA(c, cudaStreamSynchronize(c->stream));
  return MQ_OK;
}

// One epoch of minibatch Adam over the uploaded data in the order `perm`
// (a permutation of the samples); mean minibatch loss to *loss.
int mlp_train_epoch(mq_ctx *c, const int *perm, int batch, float lr, double *loss) {
  Mlp *m = mlp_of(c);
  if (!m || !m->X) return set_err(c, MQ_ESTATE, "no MLP training data (mq_mlp_set_data)");
  if (batch <= 0 || batch % 128) return set_err(c, MQ_EINVAL, "batch must be a positive multiple of 128");
  const long long n = m->nsamp;
  int *d_perm = (int *)buf(c, "mlp_perm", (size_t)n * sizeof(int) + 16);
  if (!d_perm) return MQ_ENOMEM;
  MQ_CUDA(c, cudaMemcpyAsync(d_perm, perm, (size_t)n * sizeof(int), cudaMemcpyHostToDevice, c->stream));
  Acts a;
  MQ_TRY(acts_alloc(c, m, batch, a));
  float *tb = (float *)buf(c, "mlp_tw", 2 * (size_t)batch * m->d[3] * sizeof(float) + 16);
  if (!tb) return MQ_ENOMEM;
  float *wb = tb + (size_t)batch * m->d[3];
  double total = 0.0;
  int nb = 0;
  for (long long r0 = 0; r0 + batch <= n; r0 += batch) {
    gather_rows_kernel<<<batch, 128, 0, c->stream>>>(m->X, m->T, m->Wt8, d_perm + r0, batch, m->kp[0], m->d[3], a.x,
                                                     tb, wb);
    c->stats.launches += 1;
    // the loss is normalised by the minibatch's weight sum (host side, from a device sum)
    std::vector<float> hw((size_t)batch * m->d[3]);
    MQ_CUDA(c, cudaMemcpyAsync(hw.data(), wb, hw.size() * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
    MQ_CUDA(c, cudaStreamSynchronize(c->stream));
    double wsum = 0.0;
    for (float v : hw) wsum += v;
    double l = 0.0;
    MQ_TRY(backward(c, m, a, tb, wb, wsum > 0 ? wsum : 1.0, &l));
    MQ_TRY(adam(c, m, lr));
    total += l;
    ++nb;
  }
  MQ_CUDA(c, cudaStreamSynchronize(c->stream));
  *loss = nb ? total / nb : 0.0;
  return mark_params(c);
}

void mlp_free(mq_ctx *c) {
  delete mlp_of(c);
  c->mlp = nullptr;
}

}  // namespace mq
