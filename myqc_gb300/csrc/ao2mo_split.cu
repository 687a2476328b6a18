// ao2mo_split.cu -- (ia|jb) on the 5th-generation tensor cores with split
// hi+lo BF16 operands and FP32 accumulation (the precision option of the
// four-index transform that src/ao2mo/ao2mo.f90:1306-1439 does in FP64).
//
// Each FP64/FP32 operand x is stored as two BF16 numbers, hi = bf16(x) and
// lo = bf16(x - hi), and a product is accumulated as hi*hi + hi*lo + lo*hi
// (lo*lo is below the FP32 accumulator's resolution).
//
// One GEMM kernel serves all four quarter transforms:
//     D[m][n] = sum_k A[m][k] * B[n][k]      (A, B K-major BF16 hi/lo)
// TMA (cp.async.bulk.tensor, 128-byte swizzle) stages 128 x 64 A tiles and
// N x 64 B tiles through a ring of shared-memory stages; one thread issues
// tcgen05.mma (M = 128, K = 16, N = the whole output width) into a TMEM
// accumulator; four epilogue warps read it back with tcgen05.ld and write
// either the next step's split operand or the FP64 result.  Warp roles:
//   warp 0: TMA producer, warp 1: TMEM owner + MMA issuer, warps 2-5: epilogue.
// Every mbarrier wait is bounded; on time-out the kernel raises an error flag,
// drains its own copies and MMAs (bounded), frees TMEM and returns.
//
// The four steps use the integral symmetry (uv|ld) = (dl|uv) = (vu|ld) so that
// XX itself is the first step's K-major A and each epilogue writes the next
// step's A with coalesced stores:
//   1  Y1[b][(l,u,v)]   = sum_d XX(d,l,u,v) Cb(d,b)       A1 rows (l,u,v), K = d
//   2  Y2[j,b][(u,v)]   = sum_l Y1[b][(l,u,v)] Cj(l,j)     A2 rows (u,v),   K = l
//   3  Y3[a,j,b][v]     = sum_u Y2[j,b][(u,v)] Ca(u,a)     A3 rows v,       K = u
//   4  Om(i,a,j,b)      = sum_v Y3[a,j,b][v] Ci(v,i)       A4 rows (a,j,b), K = v
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "internal.h"

namespace mq {

typedef __nv_bfloat16 bf16;
typedef unsigned short h16;  // storage of one 16-bit operand (BF16 or FP16 bits)

constexpr int UM = 128;         // MMA M (rows per tile)
constexpr int UK = 64;          // K elements per stage (one 128-byte swizzle row)
constexpr int GEMM_THREADS = 192;
constexpr long long WAIT_LIMIT = 1ll << 26;

// ------------------------------------------------------------------ PTX helpers
__device__ __forceinline__ uint32_t su32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *b, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(su32(b)) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint64_t *b, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(su32(b)), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait that ignores the error flag (drains on the way out)
__device__ __forceinline__ bool mbar_drain(uint64_t *b, uint32_t parity) {
  for (long long i = 0; i < WAIT_LIMIT; ++i)
    if (mbar_try(b, parity)) return true;
  return false;
}
// bounded wait; false once the kernel's error flag is up
__device__ __forceinline__ bool mbar_wait(uint64_t *b, uint32_t parity, int *err) {
  for (long long i = 0;; ++i) {
    if (mbar_try(b, parity)) return true;
    if ((i & 255) == 255) {
      if (*(volatile int *)err) return false;
      if (i > WAIT_LIMIT) {
        atomicExch(err, 3);
        return false;
      }
    }
  }
}

__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, uint64_t *bar, int c0, int c1, int c2) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5}], [%2];" ::
          "r"(su32(dst)),
      "l"((uint64_t)map), "r"(su32(bar)), "r"(c0), "r"(c1), "r"(c2)
      : "memory");
}
__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, uint64_t *bar, int c0, int c1) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(
          su32(dst)),
      "l"((uint64_t)map), "r"(su32(bar)), "r"(c0), "r"(c1)
      : "memory");
}

// shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups 1024 B apart
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
  d |= (uint64_t)1 << 16;           // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;  // stride byte offset
  d |= (uint64_t)1 << 46;           // descriptor version
  d |= (uint64_t)2 << 61;           // SWIZZLE_128B
  return d;
}

__device__ __forceinline__ void umma(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\ttcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(
          tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void umma_commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(bar))
               : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// warp-collective (.sync.aligned): every lane of the warp must arrive converged
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  __syncwarp();
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// ------------------------------------------------------------------ kernels
struct GemmArgs {
  int M, N, K, batch;       // logical sizes (K is the padded K)
  int ntile;                // N rounded up to a multiple of 16
  int tmem_cols;            // power of two >= ntile
  int fp16;                 // operand format: 1 FP16, 0 BF16
  int out_f64;              // 1: FP64 output; 0: split 16-bit output
  float out_scale;          // exact power of two applied to the accumulator
  long long mdiv, s_m0, s_m1, s_n, s_b;  // out index = (m%mdiv)*s_m0 + (m/mdiv)*s_m1 + n*s_n + batch*s_b
  double *out;
  h16 *out_hi, *out_lo;
  int *err;
};

// split one FP32 value into two 16-bit numbers (hi + lo ~ x)
__device__ __forceinline__ void split2(float x, int fp16, h16 &h, h16 &l) {
  if (fp16) {
    const __half a = __float2half_rn(x);
    const __half b = __float2half_rn(x - __half2float(a));
    h = __half_as_ushort(a);
    l = __half_as_ushort(b);
  } else {
    const bf16 a = __float2bfloat16_rn(x);
    const bf16 b = __float2bfloat16_rn(x - __bfloat162float(a));
    h = __bfloat16_as_ushort(a);
    l = __bfloat16_as_ushort(b);
  }
}

template <int STAGES>
__global__ void __launch_bounds__(GEMM_THREADS, 1) split_gemm_kernel(const __grid_constant__ CUtensorMap mAh,
                                                                    const __grid_constant__ CUtensorMap mAl,
                                                                    const __grid_constant__ CUtensorMap mBh,
                                                                    const __grid_constant__ CUtensorMap mBl,
                                                                    GemmArgs g) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  // 1024-byte aligned base for the swizzled tiles
  uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  const int ntile = g.ntile;
  const uint32_t a_bytes = UM * UK * 2, b_bytes = (uint32_t)ntile * UK * 2;
  const uint32_t stage_bytes = 2 * a_bytes + 2 * b_bytes;
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
    // ---------------- TMA producer
    if (lane == 0) {
      int s = 0;
      uint32_t ph = 1;
      unsigned armed = 0, armed_par = 0;  // stages whose copies were issued, and the full-barrier parity
      for (long long t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int mt = (int)(t % mtiles), bt = (int)(t / mtiles);
        for (int kc = 0; kc < kchunks; ++kc) {
          if (!mbar_wait(empty + s, ph, g.err)) goto prod_exit;
          uint8_t *st = smem + s * stage_bytes;
          mbar_expect_tx(full + s, stage_bytes);
          tma_load_3d(st, &mAh, full + s, kc * UK, mt * UM, bt);
          tma_load_3d(st + a_bytes, &mAl, full + s, kc * UK, mt * UM, bt);
          tma_load_2d(st + 2 * a_bytes, &mBh, full + s, kc * UK, 0);
          tma_load_2d(st + 2 * a_bytes + b_bytes, &mBl, full + s, kc * UK, 0);
          armed |= 1u << s;
          armed_par = (armed_par & ~(1u << s)) | ((ph ^ 1u) << s);  // the consumer waits on parity ph^1
          if (++s == STAGES) {
            s = 0;
            ph ^= 1;
          }
        }
      }
    prod_exit:
      // every issued copy lands before the CTA may exit: wait (bounded) on the
      // full barrier phase of each stage's last issued copy
      for (int k = 0; k < STAGES; ++k)
        if (armed & (1u << k)) mbar_drain(full + k, (armed_par >> k) & 1u);
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer
    if (lane == 0) {
      // D = F32; A, B = BF16 (format 1) or F16 (format 0); both K-major
      const uint32_t fmt = g.fp16 ? 0u : 1u;
      const uint32_t idesc = (1u << 4) | (fmt << 7) | (fmt << 10) | ((uint32_t)(ntile >> 3) << 17) |
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
            const uint32_t off = kk * 32;  // 16 BF16 = 32 bytes along the swizzled row
            const uint64_t ah = sdesc(base + off), al = sdesc(base + a_bytes + off);
            const uint64_t bh = sdesc(base + 2 * a_bytes + off), bl = sdesc(base + 2 * a_bytes + b_bytes + off);
            umma(tmem, ah, bh, idesc, (kc | kk) != 0);
            umma(tmem, ah, bl, idesc, 1);
            umma(tmem, al, bh, idesc, 1);
          }
          umma_commit(empty + s);  // stage free once these MMAs have read it
          if (++s == STAGES) {
            s = 0;
            ph ^= 1;
          }
        }
        if (ok) umma_commit(acc_full);
      }
      // all MMAs issued by this thread complete before TMEM is released
      umma_commit(drain);
      mbar_drain(drain, 0);
    }
  } else {
    // ---------------- epilogue: warps 2..5 cover TMEM lane quadrants 2,3,0,1
    const int q = warp & 3;
    const int row = q * 32 + lane;
    uint32_t acc_ph = 0;
    for (long long t = blockIdx.x; t < ntiles; t += gridDim.x) {
      const int mt = (int)(t % mtiles), bt = (int)(t / mtiles);
      // one lane polls, the warp reconverges before the aligned TMEM loads
      int ok = 0;
      if (lane == 0) ok = mbar_wait(acc_full, acc_ph, g.err);
      ok = __shfl_sync(0xffffffffu, ok, 0);
      if (!ok) break;
      acc_ph ^= 1;
      tc_fence_after();
      const long long m = (long long)mt * UM + row;
      const bool live = m < g.M;
      const long long base = live ? (m % g.mdiv) * g.s_m0 + (m / g.mdiv) * g.s_m1 + (long long)bt * g.s_b : 0;
      for (int c0 = 0; c0 < ntile; c0 += 16) {
        float v[16];
        tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)c0, v);
        if (!live) continue;
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          const int n = c0 + i;
          if (n >= g.N) break;
          const long long o = base + (long long)n * g.s_n;
          if (g.out_f64) {
            g.out[o] = (double)(v[i] * g.out_scale);
          } else {
            h16 h, l;
            split2(v[i] * g.out_scale, g.fp16, h, l);
            g.out_hi[o] = h;
            g.out_lo[o] = l;
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

// FP64 -> (hi, lo) BF16 without FP64 arithmetic: the double is truncated to
// FP32 with integer operations (exponent rebias, top 23 mantissa bits; values
// below the FP32 normal range become 0), then split in FP32.
__device__ __forceinline__ float f64_to_f32_bits(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
  const int e = (int)((hi >> 20) & 0x7ff) - 1023 + 127;
  if (e <= 0) return 0.0f;
  if (e >= 255) return __uint_as_float((hi & 0x80000000u) | 0x7f800000u);
  const unsigned m = ((hi & 0xfffffu) << 3) | (lo >> 29);
  return __uint_as_float((hi & 0x80000000u) | ((unsigned)e << 23) | m);
}

// out[r*Kp + k] = split(scale * in[k + ld*r]) for k < kvalid, 0 for kvalid <= k < Kp
__global__ void split_rows_kernel(const double *__restrict__ in, long long rows, int kvalid, long long ld, int Kp,
                                  float scale, int fp16, h16 *__restrict__ hi, h16 *__restrict__ lo) {
  const long long tot = rows * Kp;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < tot; i += (long long)gridDim.x * blockDim.x) {
    const long long r = i / Kp;
    const int k = (int)(i - r * Kp);
    h16 h = 0, l = 0;  // +0 in both formats
    if (k < kvalid) split2(f64_to_f32_bits(__ldcs(in + k + ld * r)) * scale, fp16, h, l);
    hi[i] = h;
    lo[i] = l;
  }
}

// per column of an n x cols block: max |c| and the 1-norm; out[2] = {max|c|, max_col ||c||_1}
__global__ void col_norms_kernel(const double *__restrict__ C, int n, int cols, double *__restrict__ out) {
  __shared__ double smax[256], snorm[256];
  double mx = 0.0, nm = 0.0;
  for (int col = threadIdx.x; col < cols; col += blockDim.x) {
    double s = 0.0;
    for (int r = 0; r < n; ++r) {
      const double v = fabs(C[r + (size_t)n * col]);
      s += v;
      mx = fmax(mx, v);
    }
    nm = fmax(nm, s);
  }
  smax[threadIdx.x] = mx;
  snorm[threadIdx.x] = nm;
  __syncthreads();
  for (int k = blockDim.x / 2; k > 0; k >>= 1) {
    if (threadIdx.x < k) {
      smax[threadIdx.x] = fmax(smax[threadIdx.x], smax[threadIdx.x + k]);
      snorm[threadIdx.x] = fmax(snorm[threadIdx.x], snorm[threadIdx.x + k]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = smax[0];
    out[1] = snorm[0];
  }
}

__global__ void max_kernel(const double *__restrict__ x, int n, double *__restrict__ out) {
  __shared__ double s[256];
  double m = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) m = fmax(m, fabs(x[i]));
  s[threadIdx.x] = m;
  __syncthreads();
  for (int k = blockDim.x / 2; k > 0; k >>= 1) {
    if (threadIdx.x < k) s[threadIdx.x] = fmax(s[threadIdx.x], s[threadIdx.x + k]);
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = s[0];
}

// ------------------------------------------------------------------ host side
static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    cudaDriverEntryPointQueryResult q;
    void *p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
  }
  return fn;
}

// rank-3 map of a K-major 16-bit operand [batch][rows][Kp] (Kp % 8 == 0), box (64, box_rows, 1)
static int make_map(mq_ctx *c, CUtensorMap *m, const h16 *ptr, int fp16, int Kp, long long rows, long long batch,
                    long long batch_stride_elems, int box_rows) {
  auto fn = encode_fn();
  if (!fn) return set_err(c, MQ_ECUDA, "cuTensorMapEncodeTiled unavailable");
  if (batch == 1) batch_stride_elems = rows * Kp;  // unused, but must be a valid stride
  if (Kp % 8 || ((uintptr_t)ptr & 15) || (batch_stride_elems * 2) % 16)
    return set_err(c, MQ_EINVAL, "TMA operand not 16-byte aligned");
  cuuint64_t dims[3] = {(cuuint64_t)Kp, (cuuint64_t)rows, (cuuint64_t)batch};
  cuuint64_t strides[2] = {(cuuint64_t)Kp * 2, (cuuint64_t)batch_stride_elems * 2};
  cuuint32_t box[3] = {(cuuint32_t)UK, (cuuint32_t)box_rows, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = fn(m, fp16 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, (void *)ptr, dims,
                  strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return set_err(c, MQ_ECUDA, "cuTensorMapEncodeTiled failed");
  return MQ_OK;
}

struct SplitOperand {
  h16 *hi, *lo;
};

// D = A B^T over split operands; A: [batch][M][Kp], B: [N][Kp] (shared by all batches)
static int split_gemm(mq_ctx *c, SplitOperand A, long long M, int batch, long long a_batch_stride, SplitOperand B,
                      int N, int Kp, GemmArgs g) {
  if (N <= 0 || M <= 0 || batch <= 0) return MQ_OK;
  if (N > 256) return set_err(c, MQ_EINVAL, "split GEMM: N > 256");
  if (M > 2147483647LL) return set_err(c, MQ_EINVAL, "split GEMM: M too large");
  CUtensorMap mAh, mAl, mBh, mBl;
  const int ntile = (N + 15) / 16 * 16;
  MQ_TRY(make_map(c, &mAh, A.hi, g.fp16, Kp, M, batch, a_batch_stride, UM));
  MQ_TRY(make_map(c, &mAl, A.lo, g.fp16, Kp, M, batch, a_batch_stride, UM));
  MQ_TRY(make_map(c, &mBh, B.hi, g.fp16, Kp, N, 1, 0, ntile));
  MQ_TRY(make_map(c, &mBl, B.lo, g.fp16, Kp, N, 1, 0, ntile));
  g.M = (int)M;
  g.N = N;
  g.K = Kp;
  g.batch = batch;
  g.ntile = ntile;
  int cols = 32;
  while (cols < ntile) cols <<= 1;
  g.tmem_cols = cols;
  const size_t stage = 2 * (size_t)UM * UK * 2 + 2 * (size_t)ntile * UK * 2;
  const size_t limit = 227 * 1024 - 1024 - 256;
  const int stages = limit >= 4 * stage ? 4 : (limit >= 3 * stage ? 3 : 2);
  const size_t smem = stages * stage + 1024 + 256;
  int sms = 148;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
  const long long tiles = (M + UM - 1) / UM * batch;
  const int grid = (int)std::min<long long>(tiles, sms);
  auto kern = stages == 4 ? split_gemm_kernel<4> : (stages == 3 ? split_gemm_kernel<3> : split_gemm_kernel<2>);
  MQ_CUDA(c, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  kern<<<grid, GEMM_THREADS, smem, c->stream>>>(mAh, mAl, mBh, mBl, g);
  c->stats.launches += 1;
  MQ_CUDA(c, cudaGetLastError());
  return sync_check(c, "split_gemm");
}

static int split_rows(mq_ctx *c, const double *in, long long rows, int kvalid, long long ld, int Kp, float scale,
                      int fp16, SplitOperand o) {
  const long long tot = rows * Kp;
  const int tb = 256;
  const long long blocks = std::max<long long>(1, std::min<long long>((tot + tb - 1) / tb, 1 << 20));
  split_rows_kernel<<<(unsigned)blocks, tb, 0, c->stream>>>(in, rows, kvalid, ld, Kp, scale, fp16, o.hi, o.lo);
  c->stats.launches += 1;
  MQ_CUDA(c, cudaGetLastError());
  return sync_check(c, "split_rows");
}

// power of two s with bound * s <= 2^14 (FP16 operands keep their hi and lo
// parts inside the normal range with room for the FP32 sums)
static double pow2_scale(double bound) {
  if (!(bound > 0)) return 1.0;
  return std::ldexp(1.0, 14 - (int)std::ceil(std::log2(bound)));
}

int ao2mo_split_device(mq_ctx *c, const double *Ci, int no1, const double *Ca, int nv1, const double *Cj, int no2,
                       const double *Cb, int nv2, double *d_out, int fp16) {
  const long long n = c->nao;
  const int Kp = (int)((n + 7) / 8 * 8);
  if (no1 > 256 || nv1 > 256 || no2 > 256 || nv2 > 256)
    return set_err(c, MQ_EINVAL, "split transform: orbital blocks above 256 are not supported");
  const long long n2 = n * n, n3 = n2 * n;
  // buffers (16-bit elements)
  const size_t eX = (size_t)n3 * Kp, e1 = (size_t)nv2 * n2 * Kp, e2 = (size_t)no2 * nv2 * n * Kp,
               e3 = (size_t)nv1 * no2 * nv2 * Kp, eC = (size_t)(no1 + nv1 + no2 + nv2) * Kp;
  h16 *bx = (h16 *)buf(c, "split_xx", 2 * eX * sizeof(h16));
  h16 *b1 = (h16 *)buf(c, "split_y1", 2 * std::max(e1, e3) * sizeof(h16));
  h16 *b2 = (h16 *)buf(c, "split_y2", 2 * e2 * sizeof(h16));
  h16 *bc = (h16 *)buf(c, "split_c", 2 * eC * sizeof(h16));
  int *err = (int *)buf(c, "split_err", 64);
  double *nrm = (double *)buf(c, "split_norms", 16 * sizeof(double));
  if (!bx || !b1 || !b2 || !bc || !err || !nrm) return MQ_ENOMEM;
  MQ_CUDA(c, cudaMemsetAsync(err, 0, sizeof(int), c->stream));
  // scale factors from rigorous bounds (FP16 only; BF16 has the FP32 range):
  // |XX| <= max_P (sqrt max (ab|ab))^2 (Schwarz), |Y_k| <= |Y_{k-1}| * max column 1-norm of C_k
  double sX = 1, sI = 1, sA = 1, sJ = 1, sB = 1, s1 = 1, s2 = 1, s3 = 1;
  if (fp16) {
    MQ_TRY(eri_schwarz(c));
    MQ_TRY(sync_check(c, "schwarz"));
    max_kernel<<<1, 256, 0, c->stream>>>(c->pt.schwarz, c->pt.npairs, nrm);
    col_norms_kernel<<<1, 256, 0, c->stream>>>(Ci, (int)n, no1, nrm + 2);
    col_norms_kernel<<<1, 256, 0, c->stream>>>(Ca, (int)n, nv1, nrm + 4);
    col_norms_kernel<<<1, 256, 0, c->stream>>>(Cj, (int)n, no2, nrm + 6);
    col_norms_kernel<<<1, 256, 0, c->stream>>>(Cb, (int)n, nv2, nrm + 8);
    c->stats.launches += 5;
    MQ_TRY(sync_check(c, "norms"));
    double h[10];
    MQ_CUDA(c, cudaMemcpyAsync(h, nrm, sizeof h, cudaMemcpyDeviceToHost, c->stream));
    MQ_CUDA(c, cudaStreamSynchronize(c->stream));
    const double bX = h[0] * h[0];
    sX = pow2_scale(bX);
    sI = pow2_scale(h[2]);
    sA = pow2_scale(h[4]);
    sJ = pow2_scale(h[6]);
    sB = pow2_scale(h[8]);
    const double b1 = bX * h[9], b2 = b1 * h[7], b3 = b2 * h[5];
    s1 = pow2_scale(b1);
    s2 = pow2_scale(b2);
    s3 = pow2_scale(b3);
  }
  SplitOperand X{bx, bx + eX}, Y1{b1, b1 + e1}, Y2{b2, b2 + e2}, Y3{b1, b1 + e3};  // Y3 reuses Y1's space
  SplitOperand Bi{bc, bc + eC}, Ba{Bi.hi + (size_t)no1 * Kp, Bi.lo + (size_t)no1 * Kp};
  SplitOperand Bj{Ba.hi + (size_t)nv1 * Kp, Ba.lo + (size_t)nv1 * Kp}, Bb{Bj.hi + (size_t)no2 * Kp, Bj.lo + (size_t)no2 * Kp};
  // coefficient blocks: column p of C (n contiguous) becomes row p of B (K-major)
  MQ_TRY(split_rows(c, Ci, no1, (int)n, n, Kp, (float)sI, fp16, Bi));
  MQ_TRY(split_rows(c, Ca, nv1, (int)n, n, Kp, (float)sA, fp16, Ba));
  MQ_TRY(split_rows(c, Cj, no2, (int)n, n, Kp, (float)sJ, fp16, Bj));
  MQ_TRY(split_rows(c, Cb, nv2, (int)n, n, Kp, (float)sB, fp16, Bb));
  // XX(d,l,u,v) at d + n*((l,u,v)): rows (l,u,v) with K = d
  MQ_TRY(split_rows(c, c->d_XX, n3, (int)n, n, Kp, (float)sX, fp16, X));
  GemmArgs g{};
  g.err = err;
  g.fp16 = fp16;
  // 1: Y1[b][(u,v)][l] = sum_d XX(d,l,u,v) Cb(d,b);   row m = l + n*(u + n*v)
  g.out_f64 = 0;
  g.out_scale = (float)(s1 / (sX * sB));
  g.out_hi = Y1.hi;
  g.out_lo = Y1.lo;
  g.mdiv = n;
  g.s_m0 = 1;
  g.s_m1 = Kp;
  g.s_n = n2 * Kp;
  g.s_b = 0;
  MQ_TRY(split_gemm(c, X, n3, 1, 0, Bb, nv2, Kp, g));
  // 2: batch b; rows m = u + n*v, K = l -> Y2[j,b][v][u]
  g.out_scale = (float)(s2 / (s1 * sJ));
  g.out_hi = Y2.hi;
  g.out_lo = Y2.lo;
  g.mdiv = n;
  g.s_m0 = 1;
  g.s_m1 = Kp;
  g.s_n = n * Kp;
  g.s_b = (long long)no2 * n * Kp;
  MQ_TRY(split_gemm(c, Y1, n2, nv2, n2 * Kp, Bj, no2, Kp, g));
  // 3: batch (j + no2*b); rows v, K = u -> Y3[a + nv1*(j + no2*b)][v]
  g.out_scale = (float)(s3 / (s2 * sA));
  g.out_hi = Y3.hi;
  g.out_lo = Y3.lo;
  g.mdiv = 1ll << 62;
  g.s_m0 = 1;
  g.s_m1 = 0;
  g.s_n = Kp;
  g.s_b = (long long)nv1 * Kp;
  MQ_TRY(split_gemm(c, Y2, n, no2 * nv2, n * Kp, Ba, nv1, Kp, g));
  // 4: rows (a, j, b), K = v -> Om(i, a, j, b) = D[m][i] at i + no1*m
  g.out_f64 = 1;
  g.out_scale = (float)(1.0 / (s3 * sI));
  g.out = d_out;
  g.mdiv = 1ll << 62;
  g.s_m0 = no1;
  g.s_m1 = 0;
  g.s_n = 1;
  g.s_b = 0;
  MQ_TRY(split_gemm(c, Y3, (long long)nv1 * no2 * nv2, 1, 0, Bi, no1, Kp, g));
  int h = 0;
  MQ_CUDA(c, cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  MQ_CUDA(c, cudaStreamSynchronize(c->stream));
  if (h) return set_err(c, MQ_ETIMEOUT, "split GEMM pipeline wait timed out");
  return MQ_OK;
}

}  // namespace mq
