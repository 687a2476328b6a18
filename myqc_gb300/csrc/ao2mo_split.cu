// ao2mo_split.cu -- (ia|jb) on the 5th-generation tensor cores with split
// BF16 operands and FP32 accumulation (the precision option of the four-index
// transform that src/ao2mo/ao2mo.f90:1306-1439 does in FP64).
//
// Each FP64/FP32 operand x is stored as P BF16 planes (x ~ hi + lo, or
// hi + mid + lo), each plane the BF16 rounding of what the previous ones left;
// the products of plane pairs above the FP32 accumulator's resolution are
// accumulated (3 MMAs per K step for P = 2, 6 for P = 3).
//
// One GEMM kernel serves all four quarter transforms:
//     D[m][n] = sum_k A[m][k] * B[n][k]      (A, B K-major BF16 planes)
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

#include "internal.h"

namespace mq {

typedef __nv_bfloat16 bf16;

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
// An operand is stored as P BF16 planes (P = 2: hi, lo; P = 3: hi, mid, lo),
// x ~ sum of planes.  The products accumulated per K step are all plane pairs
// whose combined weight is above the FP32 accumulator's resolution:
//   P = 2: hh, hl, lh          (~16-bit operands)
//   P = 3: hh, hm, mh, hl, mm, lh   (~24-bit operands)
template <int P>
struct PlaneProducts;
template <>
struct PlaneProducts<2> {
  static constexpr int n = 3;
  __device__ static constexpr int a(int i) { return i == 2 ? 1 : 0; }
  __device__ static constexpr int b(int i) { return i == 1 ? 1 : 0; }
};
template <>
struct PlaneProducts<3> {
  static constexpr int n = 6;
  __device__ static constexpr int a(int i) { return i == 0 ? 0 : i == 1 ? 0 : i == 2 ? 1 : i == 3 ? 0 : i == 4 ? 1 : 2; }
  __device__ static constexpr int b(int i) { return i == 0 ? 0 : i == 1 ? 1 : i == 2 ? 0 : i == 3 ? 2 : i == 4 ? 1 : 0; }
};

struct GemmArgs {
  int M, N, K, batch;       // logical sizes (K is the padded K)
  int ntile;                // N rounded up to a multiple of 16
  int tmem_cols;            // power of two >= ntile
  int out_f64;              // 1: FP64 output; 0: split BF16 output (P planes)
  long long mdiv, s_m0, s_m1, s_n, s_b;  // out index = (m%mdiv)*s_m0 + (m/mdiv)*s_m1 + n*s_n + batch*s_b
  long long out_plane;      // elements between output planes
  double *out;
  bf16 *out16;
  int *err;
};

// x ~ p[0] + p[1] (+ p[2]) in BF16, each part the rounding of the remainder
template <int P>
__device__ __forceinline__ void split_planes(float x, bf16 (&p)[P]) {
#pragma unroll
  for (int k = 0; k < P; ++k) {
    p[k] = __float2bfloat16_rn(x);
    x = x - __bfloat162float(p[k]);
  }
}

struct Maps {
  CUtensorMap a[3];
  CUtensorMap b[3];
};

template <int P, int STAGES>
__global__ void __launch_bounds__(GEMM_THREADS, 1) split_gemm_kernel(const __grid_constant__ Maps maps, GemmArgs g) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  // 1024-byte aligned base for the swizzled tiles
  uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  const int ntile = g.ntile;
  const uint32_t a_bytes = UM * UK * 2, b_bytes = (uint32_t)ntile * UK * 2;
  const uint32_t stage_bytes = P * (a_bytes + b_bytes);
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
#pragma unroll
          for (int pl = 0; pl < P; ++pl) {
            tma_load_3d(st + pl * a_bytes, &maps.a[pl], full + s, kc * UK, mt * UM, bt);
            tma_load_3d(st + P * a_bytes + pl * b_bytes, &maps.b[pl], full + s, kc * UK, 0, 0);
          }
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
      // D = F32 (bits 4-5 = 1); A, B = BF16 (bits 7-9, 10-12 = 1); both K-major; N >> 3; M >> 4
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
            const uint32_t off = kk * 32;  // 16 BF16 = 32 bytes along the swizzled row
#pragma unroll
            for (int pr = 0; pr < PlaneProducts<P>::n; ++pr) {
              const uint64_t ad = sdesc(base + PlaneProducts<P>::a(pr) * a_bytes + off);
              const uint64_t bd = sdesc(base + P * a_bytes + PlaneProducts<P>::b(pr) * b_bytes + off);
              umma(tmem, ad, bd, idesc, (kc | kk | pr) != 0);
            }
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
            g.out[o] = (double)v[i];
          } else {
            bf16 p[P];
            split_planes<P>(v[i], p);
#pragma unroll
            for (int k = 0; k < P; ++k) g.out16[o + k * g.out_plane] = p[k];
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

// FP64 -> FP32 without FP64 arithmetic: exponent rebias and the top 23 mantissa
// bits with integer operations (values below the FP32 normal range become 0).
__device__ __forceinline__ float f64_to_f32_bits(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
  const int e = (int)((hi >> 20) & 0x7ff) - 1023 + 127;
  if (e <= 0) return 0.0f;
  if (e >= 255) return __uint_as_float((hi & 0x80000000u) | 0x7f800000u);
  const unsigned m = ((hi & 0xfffffu) << 3) | (lo >> 29);
  return __uint_as_float((hi & 0x80000000u) | ((unsigned)e << 23) | m);
}

// plane k of out holds part k of in[k' + ld*r] at r*Kp + k' (zero for kvalid <= k' < Kp)
template <int P>
__global__ void split_rows_kernel(const double *__restrict__ in, long long rows, int kvalid, long long ld, int Kp,
                                  long long plane, bf16 *__restrict__ out) {
  const long long tot = rows * Kp;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < tot; i += (long long)gridDim.x * blockDim.x) {
    const long long r = i / Kp;
    const int k = (int)(i - r * Kp);
    const float x = k < kvalid ? f64_to_f32_bits(__ldcs(in + k + ld * r)) : 0.0f;
    bf16 p[P];
    split_planes<P>(x, p);
#pragma unroll
    for (int q = 0; q < P; ++q) out[i + q * plane] = p[q];
  }
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

// rank-3 map of a K-major BF16 operand [batch][rows][Kp] (Kp % 8 == 0), box (64, box_rows, 1)
static int make_map(mq_ctx *c, CUtensorMap *m, const bf16 *ptr, int Kp, long long rows, long long batch,
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
  CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, (void *)ptr, dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return set_err(c, MQ_ECUDA, "cuTensorMapEncodeTiled failed");
  return MQ_OK;
}

// a split operand: P planes of `plane` elements each, starting at `base`
struct SplitOperand {
  bf16 *base;
  long long plane;
};

template <int P>
static int split_gemm(mq_ctx *c, SplitOperand A, long long M, int batch, long long a_batch_stride, SplitOperand B,
                      int N, int Kp, GemmArgs g) {
  if (N <= 0 || M <= 0 || batch <= 0) return MQ_OK;
  if (N > 256) return set_err(c, MQ_EINVAL, "split GEMM: N > 256");
  if (M > 2147483647LL) return set_err(c, MQ_EINVAL, "split GEMM: M too large");
  Maps maps;
  const int ntile = (N + 15) / 16 * 16;
  for (int p = 0; p < P; ++p) {
    MQ_TRY(make_map(c, &maps.a[p], A.base + p * A.plane, Kp, M, batch, a_batch_stride, UM));
    MQ_TRY(make_map(c, &maps.b[p], B.base + p * B.plane, Kp, N, 1, 0, ntile));
  }
  g.M = (int)M;
  g.N = N;
  g.K = Kp;
  g.batch = batch;
  g.ntile = ntile;
  int cols = 32;
  while (cols < ntile) cols <<= 1;
  g.tmem_cols = cols;
  const size_t stage = (size_t)P * ((size_t)UM * UK * 2 + (size_t)ntile * UK * 2);
  const size_t limit = 227 * 1024 - 1024 - 256;
  const int stages = limit >= 4 * stage ? 4 : (limit >= 3 * stage ? 3 : 2);
  if (limit < 2 * stage) return set_err(c, MQ_EINVAL, "split GEMM: shared memory");
  const size_t smem = stages * stage + 1024 + 256;
  int sms = 148;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
  const long long tiles = (M + UM - 1) / UM * batch;
  const int grid = (int)std::min<long long>(tiles, sms);
  auto kern = stages == 4 ? split_gemm_kernel<P, 4> : (stages == 3 ? split_gemm_kernel<P, 3> : split_gemm_kernel<P, 2>);
  MQ_CUDA(c, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  kern<<<grid, GEMM_THREADS, smem, c->stream>>>(maps, g);
  c->stats.launches += 1;
  MQ_CUDA(c, cudaGetLastError());
  return sync_check(c, "split_gemm");
}

template <int P>
static int split_rows(mq_ctx *c, const double *in, long long rows, int kvalid, long long ld, int Kp, SplitOperand o) {
  const long long tot = rows * Kp;
  const int tb = 256;
  const long long blocks = std::max<long long>(1, std::min<long long>((tot + tb - 1) / tb, 1 << 20));
  split_rows_kernel<P><<<(unsigned)blocks, tb, 0, c->stream>>>(in, rows, kvalid, ld, Kp, o.plane, o.base);
  c->stats.launches += 1;
  MQ_CUDA(c, cudaGetLastError());
  return sync_check(c, "split_rows");
}

template <int P>
static int ao2mo_split_planes(mq_ctx *c, const double *Ci, int no1, const double *Ca, int nv1, const double *Cj,
                              int no2, const double *Cb, int nv2, double *d_out) {
  const long long n = c->nao;
  const int Kp = (int)((n + 7) / 8 * 8);
  if (no1 > 256 || nv1 > 256 || no2 > 256 || nv2 > 256)
    return set_err(c, MQ_EINVAL, "split transform: orbital blocks above 256 are not supported");
  const long long n2 = n * n, n3 = n2 * n;
  // plane sizes (BF16 elements)
  const long long eX = n3 * Kp, e1 = (long long)nv2 * n2 * Kp, e2 = (long long)no2 * nv2 * n * Kp,
                  e3 = (long long)nv1 * no2 * nv2 * Kp;
  const long long eC[4] = {(long long)no1 * Kp, (long long)nv1 * Kp, (long long)no2 * Kp, (long long)nv2 * Kp};
  bf16 *bx = (bf16 *)buf(c, "split_xx", P * eX * sizeof(bf16));
  bf16 *b1 = (bf16 *)buf(c, "split_y1", P * std::max(e1, e3) * sizeof(bf16));
  bf16 *b2 = (bf16 *)buf(c, "split_y2", P * e2 * sizeof(bf16));
  bf16 *bc = (bf16 *)buf(c, "split_c", P * (eC[0] + eC[1] + eC[2] + eC[3]) * sizeof(bf16));
  int *err = (int *)buf(c, "split_err", 64);
  if (!bx || !b1 || !b2 || !bc || !err) return MQ_ENOMEM;
  MQ_CUDA(c, cudaMemsetAsync(err, 0, sizeof(int), c->stream));
  SplitOperand X{bx, eX}, Y1{b1, e1}, Y2{b2, e2}, Y3{b1, e3};  // Y3 reuses Y1's space
  SplitOperand Bi{bc, eC[0]}, Ba{bc + P * eC[0], eC[1]}, Bj{Ba.base + P * eC[1], eC[2]},
      Bb{Bj.base + P * eC[2], eC[3]};
  // coefficient blocks: column p of C (n contiguous) becomes row p of B (K-major)
  MQ_TRY(split_rows<P>(c, Ci, no1, (int)n, n, Kp, Bi));
  MQ_TRY(split_rows<P>(c, Ca, nv1, (int)n, n, Kp, Ba));
  MQ_TRY(split_rows<P>(c, Cj, no2, (int)n, n, Kp, Bj));
  MQ_TRY(split_rows<P>(c, Cb, nv2, (int)n, n, Kp, Bb));
  // XX(d,l,u,v) at d + n*((l,u,v)): rows (l,u,v) with K = d
  MQ_TRY(split_rows<P>(c, c->d_XX, n3, (int)n, n, Kp, X));
  GemmArgs g{};
  g.err = err;
  // 1: Y1[b][(u,v)][l] = sum_d XX(d,l,u,v) Cb(d,b);   row m = l + n*(u + n*v)
  g.out_f64 = 0;
  g.out16 = Y1.base;
  g.out_plane = Y1.plane;
  g.mdiv = n;
  g.s_m0 = 1;
  g.s_m1 = Kp;
  g.s_n = n2 * Kp;
  g.s_b = 0;
  MQ_TRY(split_gemm<P>(c, X, n3, 1, 0, Bb, nv2, Kp, g));
  // 2: batch b; rows m = u + n*v, K = l -> Y2[j,b][v][u]
  g.out16 = Y2.base;
  g.out_plane = Y2.plane;
  g.mdiv = n;
  g.s_m0 = 1;
  g.s_m1 = Kp;
  g.s_n = n * Kp;
  g.s_b = (long long)no2 * n * Kp;
  MQ_TRY(split_gemm<P>(c, Y1, n2, nv2, n2 * Kp, Bj, no2, Kp, g));
  // 3: batch (j + no2*b); rows v, K = u -> Y3[a + nv1*(j + no2*b)][v]
  g.out16 = Y3.base;
  g.out_plane = Y3.plane;
  g.mdiv = 1ll << 62;
  g.s_m0 = 1;
  g.s_m1 = 0;
  g.s_n = Kp;
  g.s_b = (long long)nv1 * Kp;
  MQ_TRY(split_gemm<P>(c, Y2, n, no2 * nv2, n * Kp, Ba, nv1, Kp, g));
  // 4: rows (a, j, b), K = v -> Om(i, a, j, b) = D[m][i] at i + no1*m
  g.out_f64 = 1;
  g.out = d_out;
  g.mdiv = 1ll << 62;
  g.s_m0 = no1;
  g.s_m1 = 0;
  g.s_n = 1;
  g.s_b = 0;
  MQ_TRY(split_gemm<P>(c, Y3, (long long)nv1 * no2 * nv2, 1, 0, Bi, no1, Kp, g));
  int h = 0;
  MQ_CUDA(c, cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  MQ_CUDA(c, cudaStreamSynchronize(c->stream));
  if (h) return set_err(c, MQ_ETIMEOUT, "split GEMM pipeline wait timed out");
  return MQ_OK;
}

int ao2mo_split_device(mq_ctx *c, const double *Ci, int no1, const double *Ca, int nv1, const double *Cj, int no2,
                       const double *Cb, int nv2, double *d_out, int planes) {
  if (planes == 3) return ao2mo_split_planes<3>(c, Ci, no1, Ca, nv1, Cj, no2, Cb, nv2, d_out);
  return ao2mo_split_planes<2>(c, Ci, no1, Ca, nv1, Cj, no2, Cb, nv2, d_out);
}

}  // namespace mq
