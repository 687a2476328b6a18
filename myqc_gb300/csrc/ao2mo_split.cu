// ao2mo_split.cu -- (ia|jb) on the 5th-generation tensor cores with split
// BF16 operands and FP32 accumulation (the precision option of the four-index
// transform that src/ao2mo/ao2mo.f90:1306-1439 does in FP64).
//
// Each operand row is scaled by a power of two and cut into S integer slices
// that BF16 holds exactly (S = 2: hi+lo, S = 3: hi+mid+lo); slice products
// are accumulated exactly in FP32 TMEM (see "kernels" below).
//
// One GEMM kernel serves all four quarter transforms:
//     D[m][n] = sum_k A[m][k] * B[n][k]      (A, B K-major BF16 slices)
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
// step's A with coalesced stores (with the quartet store instead of XX, the
// first step is a sparse FP32 product on the CUDA cores, store_first_quarter
// below: its operand is mostly screened-out zeros):
//   1  Y1[b][(l,p)]     = sum_d XX(d,l,u,v) Cb(d,b)       A1 rows (l,p),   K = d
//   2  Y2[j,b][p]       = sum_l Y1[b][(l,p)] Cj(l,j)       A2 rows p,       K = l
//   3  Y3[a,j,b][v]     = sum_u Y2[j,b][(u,v)] Ca(u,a)     A3 rows v,       K = u
//   4  Om(i,a,j,b)      = sum_v Y3[a,j,b][v] Ci(v,i)       A4 rows (a,j,b), K = v
// where p runs over the AO pairs u <= v only ((uv|ld) = (vu|ld)): steps 1 and
// 2 do half the rows, and step 3's slicing reads (u,v) and (v,u) from the same
// packed element of Y2.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include "internal.h"
#include "tc.cuh"

namespace mq {

// ------------------------------------------------------------------ kernels
// Operands are cut into S exact BF16 slices with one power-of-two scale per
// row (per row of A over K, per row of B over K):
//     x = 2^(e - 8S + 1) * (s0 * 2^(8(S-1)) + ... + s_{S-1}),   s_k integers, |s_k| <= 128
// Each slice is an integer that BF16 holds exactly, so a slice product is an
// integer below 2^14 and, for one output element and one slice pair, every
// partial sum over K is an integer too.  Products are grouped by level
// L = k + l (L < S) into S TMEM accumulators; with at most 3 pairs per level
// and K <= 340, every partial sum stays below 2^24 and the FP32 accumulation
// is exact in any order and rounding mode.  Only the slicing itself rounds
// (to nearest, unbiased), at 2^-8S of the row maximum.  Levels >= S (pairs
// of weight below 2^-8S) are not formed.
//   S = 2: levels {00}, {01,10}                 3 MMAs per K step (~16-bit)
//   S = 3: levels {00}, {01,10}, {02,11,20}     6 MMAs per K step (~24-bit)
constexpr int SLICE_KMAX = 340;  // 3 * 340 * 128^2 < 2^24

template <int S>
struct Levels;
template <>
struct Levels<2> {
  static constexpr int n = 3;
  __device__ static constexpr int a(int i) { return i == 2 ? 1 : 0; }
  __device__ static constexpr int b(int i) { return i == 1 ? 1 : 0; }
  __device__ static constexpr int lev(int i) { return i == 0 ? 0 : 1; }
};
template <>
struct Levels<3> {
  static constexpr int n = 6;
  __device__ static constexpr int a(int i) { return i < 2 ? 0 : i == 2 ? 1 : i == 3 ? 0 : i == 4 ? 1 : 2; }
  __device__ static constexpr int b(int i) { return i == 0 ? 0 : i == 1 ? 1 : i == 2 ? 0 : i == 3 ? 2 : i == 4 ? 1 : 0; }
  __device__ static constexpr int lev(int i) { return i == 0 ? 0 : i < 3 ? 1 : 2; }
};

struct GemmArgs {
  int M, N, K, batch;       // logical sizes (K is the padded K)
  int ntile;                // N rounded up to a multiple of 16
  int tmem_cols;            // power of two >= S * ntile
  int out_f64;              // 1: FP64 output; 0: FP32 output
  long long mdiv, s_m0, s_m1, s_n, s_b;  // out index = (m%mdiv)*s_m0 + (m/mdiv)*s_m1 + n*s_n + batch*s_b
  const int *eA;            // row exponents of A, [batch][M]
  const int *eB;            // row exponents of B, [N]
  double *out64;
  float *out32;
  int *err;
};

struct Maps {
  CUtensorMap a[3];
  CUtensorMap b[3];
};

__device__ __forceinline__ float pow2f(int e) {  // 2^e for e in the FP32 normal range, 0 below
  return e < -126 ? 0.0f : __int_as_float((min(e, 127) + 127) << 23);
}

template <int S, int STAGES>
__global__ void __launch_bounds__(GEMM_THREADS, 1) slice_gemm_kernel(const __grid_constant__ Maps maps, GemmArgs g) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  // 1024-byte aligned base for the swizzled tiles
  uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  const int ntile = g.ntile;
  const uint32_t a_bytes = UM * UK * 2, b_bytes = (uint32_t)ntile * UK * 2;
  const uint32_t stage_bytes = S * (a_bytes + b_bytes);
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
          for (int pl = 0; pl < S; ++pl) {
            tma_load_3d(st + pl * a_bytes, &maps.a[pl], full + s, kc * UK, mt * UM, bt);
            tma_load_3d(st + S * a_bytes + pl * b_bytes, &maps.b[pl], full + s, kc * UK, 0, 0);
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
            for (int pr = 0; pr < Levels<S>::n; ++pr) {
              const int L = Levels<S>::lev(pr);
              const uint64_t ad = sdesc(base + Levels<S>::a(pr) * a_bytes + off);
              const uint64_t bd = sdesc(base + S * a_bytes + Levels<S>::b(pr) * b_bytes + off);
              // the first product of each level in a tile overwrites its accumulator
              const bool first = kc == 0 && kk == 0 && (pr == 0 || Levels<S>::lev(pr - 1) != L);
              umma(tmem + (uint32_t)(L * ntile), ad, bd, idesc, first ? 0u : 1u);
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
      const int ea = live ? g.eA[(long long)bt * g.M + m] : 0;
      for (int c0 = 0; c0 < ntile; c0 += 16) {
        float v[S][16];
#pragma unroll
        for (int L = 0; L < S; ++L) tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(L * ntile + c0), v[L]);
        if (!live) continue;
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          const int n = c0 + i;
          if (n >= g.N) break;
          // exact integer levels combined once, rounding to nearest
          float x = v[S - 1][i];
#pragma unroll
          for (int L = S - 2; L >= 0; --L) x = fmaf(x, 0.00390625f, v[L][i]);
          x *= pow2f(ea + g.eB[n] - 14);
          const long long o = base + (long long)n * g.s_n;
          if (g.out_f64) g.out64[o] = (double)x;
          else g.out32[o] = x;
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

// Row exponent and fixed-point digits with integer operations only.
// A value |x| < 2^e becomes q = round(x * 2^(8S-1-e)), |q| < 2^(8S-1), split in
// balanced base-256 digits s_0 .. s_{S-1} (|s_0| <= 128, others in [-128, 127]).
__device__ __forceinline__ int exp_field(double x) {
  return (int)((unsigned long long)__double_as_longlong(x) >> 52) & 0x7ff;
}
__device__ __forceinline__ int exp_field(float x) { return (__float_as_int(x) >> 23) & 0xff; }
// value = mant * 2^(ex) with mant the full integer significand (implicit bit set)
__device__ __forceinline__ void decompose(double x, long long &mant, int &ex) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int E = (int)(b >> 52) & 0x7ff;
  if (E == 0) {  // zero (subnormals are far below any slice)
    mant = 0;
    ex = 0;
    return;
  }
  mant = (long long)((b & 0xfffffffffffffull) | 0x10000000000000ull);
  if (b >> 63) mant = -mant;
  ex = E - 1075;
}
__device__ __forceinline__ void decompose(float x, long long &mant, int &ex) {
  const unsigned b = (unsigned)__float_as_int(x);
  const int E = (int)(b >> 23) & 0xff;
  if (E == 0) {
    mant = 0;
    ex = 0;
    return;
  }
  mant = (long long)((b & 0x7fffffu) | 0x800000u);
  if (b >> 31) mant = -mant;
  ex = E - 150;
}

// One warp per row: the r-th row at in + r*ld (kvalid values) becomes S planes
// of `plane` elements at out + r*Kp, its exponent e[r].  Lane l owns the
// 8-element chunks l and l+32 of the row (Kp <= 512): the row is read once into
// registers (16-byte loads when `vec`), and each plane gets one 16-byte store per
// chunk.  `vec` requires 16-byte aligned rows and kvalid a multiple of the
// elements per 16 bytes.
template <class T>
__device__ __forceinline__ void load_chunk(const T *__restrict__ x, int k0, int kvalid, bool vec, T (&v)[8]) {
  if (vec && k0 + 8 <= kvalid) {
    if (sizeof(T) == 8) {
      const double2 *p = reinterpret_cast<const double2 *>(x + k0);
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const double2 t = __ldg(p + j);
        v[2 * j] = (T)t.x;
        v[2 * j + 1] = (T)t.y;
      }
    } else {
      const float4 *p = reinterpret_cast<const float4 *>(x + k0);
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        const float4 t = __ldg(p + j);
        v[4 * j] = (T)t.x;
        v[4 * j + 1] = (T)t.y;
        v[4 * j + 2] = (T)t.z;
        v[4 * j + 3] = (T)t.w;
      }
    }
  } else {
#pragma unroll
    for (int j = 0; j < 8; ++j) v[j] = (k0 + j < kvalid) ? __ldg(x + k0 + j) : (T)0;
  }
}

// Where row r of a sliced operand comes from (RowSrc):
//   ROW_PLAIN  in + r * ld;
//   ROW_PAIRS  rows (l, p) of XX restricted to the pairs p = (u <= v): source row
//              l + n (u + n v) of XX (rows of n values), l = r mod n;
//   ROW_SYMM   row (v, jb) of the pair-packed Y2: element u is
//              in[jb * npairs + pidx(min(u, v), max(u, v))], pidx(u, v) = u + v (v + 1) / 2.
//   ROW_TRANS  row (b, p) of the [p][l][b] array the store's first quarter
//              writes: element l at in[(p n + l) nb + b]; the rows are visited
//              with b fastest, so the warps reading one p share its sectors
enum { ROW_PLAIN = 0, ROW_PAIRS = 1, ROW_SYMM = 2, ROW_TRANS = 3 };
struct StoreView {
  const double *X;
  const int4 *pinfo;  // [S1 * nsh + S2]: pair, class, rank, bit 0: stored as (S2, S1), bit 1: S1 = S2
  const int *ao_shell, *ao0;
  const long long *off[6];
  const int *len[6];
  long long base[6];
  int nsh;
  const double *pbound;  // Schwarz bound of each pair
  const double *qmax;    // per shell: the largest bound of a pair containing it
  const int *partners;   // per shell S: the shells D by the bound of the pair (D, S), descending
  double thr;            // the store's threshold
};
struct RowSrc {
  const int2 *pairs;  // (u, v) of each pair p, u <= v
  long long n, npairs;
  long long nb;  // ROW_TRANS: the columns b of the [p][l][b] source
};

__host__ __device__ constexpr int sv_nfa(int cls) { return cls >= 1 ? 4 : 1; }
__host__ __device__ constexpr int sv_nfb(int cls) { return cls == 2 ? 4 : 1; }

// The S planes and the exponent of one row whose values a warp holds in
// registers: lane owns the 8-element chunks lane + 32 h (h < H) of the row.
template <int S, class T, int H>
__device__ __forceinline__ void slice_row_regs(T (&v)[H][8], long long r, int nchunk, int Kp, long long plane,
                                               bf16 *__restrict__ out, int *__restrict__ e) {
  const int lane = threadIdx.x & 31;
  int emax = 0;
#pragma unroll
  for (int h = 0; h < H; ++h)
    if (lane + 32 * h < nchunk)
#pragma unroll
      for (int j = 0; j < 8; ++j) emax = max(emax, exp_field(v[h][j]));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, o));
  // |x| < 2^erow with erow = unbiased exponent of the largest element + 1
  const int erow = emax == 0 ? -200 : emax - (sizeof(T) == 8 ? 1022 : 126);
  if (lane == 0) e[r] = erow;
#pragma unroll
  for (int h = 0; h < H; ++h) {
    const int c = lane + 32 * h;
    if (c >= nchunk) continue;
    unsigned packed[S][4];
#pragma unroll
    for (int j = 0; j < 8; j += 2) {
      float dig[2][S];
#pragma unroll
      for (int t = 0; t < 2; ++t) {
        long long mant;
        int ex;
        decompose(v[h][j + t], mant, ex);
        // q = round(mant * 2^(ex + 8S - 1 - erow)); the shift is negative for every nonzero x
        const int sh = -(ex + 8 * S - 1 - erow);
        int q = 0;
        if (mant != 0 && sh < 62) q = (int)(sh > 0 ? ((mant + (1ll << (sh - 1))) >> sh) : (mant << -sh));
#pragma unroll
        for (int d = S - 1; d > 0; --d) {
          const int hi = (q + 128) >> 8;  // balanced digit: q = hi*256 + lo, lo in [-128, 127]
          dig[t][d] = (float)(q - hi * 256);
          q = hi;
        }
        dig[t][0] = (float)q;
      }
#pragma unroll
      for (int d = 0; d < S; ++d) {
        const __nv_bfloat162 b2 = __floats2bfloat162_rn(dig[0][d], dig[1][d]);
        packed[d][j >> 1] = *reinterpret_cast<const unsigned *>(&b2);
      }
    }
#pragma unroll
    for (int d = 0; d < S; ++d)
      *reinterpret_cast<uint4 *>(out + d * plane + r * Kp + 8 * c) =
          make_uint4(packed[d][0], packed[d][1], packed[d][2], packed[d][3]);
  }
}

template <int S, class T, int H, int MODE>
__global__ void __launch_bounds__(256, 4) slice_rows_kernel(const T *__restrict__ in, long long rows, int kvalid,
                                                         long long ld, int Kp, long long plane, bf16 *__restrict__ out,
                                                         int *__restrict__ e, int vec, RowSrc rs) {
  const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
  const int lane = threadIdx.x & 31;
  const int nchunk = Kp >> 3;
  for (long long ri = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); ri < rows; ri += warps) {
    long long r = ri;
    const T *x = in + r * ld;
    long long jb = 0;
    int vrow = 0;
    if (MODE == ROW_TRANS) {
      const long long p = ri / rs.nb, b = ri - p * rs.nb;
      r = b * rs.npairs + p;
      x = in + p * rs.n * rs.nb + b;
    } else if (MODE == ROW_PAIRS) {
      const long long pidx = r / rs.n;
      const int2 uv = rs.pairs[pidx];
      x = in + ((r - pidx * rs.n) + rs.n * (uv.x + rs.n * (long long)uv.y)) * ld;
    } else if (MODE == ROW_SYMM) {
      jb = r / rs.n;
      vrow = (int)(r - jb * rs.n);
      x = in + jb * rs.npairs;
    }
    T v[H][8];
#pragma unroll
    for (int h = 0; h < H; ++h) {
      const int c = lane + 32 * h;
      if (c < nchunk) {
        if (MODE == ROW_SYMM) {
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const int u = 8 * c + j, lo = min(u, vrow), hi = max(u, vrow);
            v[h][j] = u < kvalid ? __ldg(x + lo + (long long)hi * (hi + 1) / 2) : (T)0;
          }
        } else if (MODE == ROW_TRANS) {
#pragma unroll
          for (int j = 0; j < 8; ++j) v[h][j] = 8 * c + j < kvalid ? __ldg(x + (8 * c + j) * rs.nb) : (T)0;
        } else {
          load_chunk(x, 8 * c, kvalid, vec != 0, v[h]);
        }
      }
    }
    slice_row_regs<S, T, H>(v, r, nchunk, Kp, plane, out, e);
  }
}

// ---- Stored blocks of a row group (L; U <= V) of the first step: the rows
// (l, p = (u <= v)) with l in shell L and (u, v) the AO pairs u <= v of the
// shells U, V, element (d l|u v) at column d.  Every row of a group reads the
// same blocks -- (D L|U V) for the shells D whose pair (D, L) passes the
// screen with (U, V), a prefix of L's partner list (ordered by the bound of
// (D, L)), cut by the same bound product test as the store's staircase.
struct LiveBlock {
  long long off;  // the block in the store
  int a0;         // first AO of D
  int flags;      // bit0: (D, L) stored as (L, D); bit1: D = L; bit2: (D, L) is the bra; bit3: (D, L) = (U, V);
                  // bits 4, 5, 6: 4 functions in the block's second, third, fourth shell; bits 8-11: AOs of D
};

// the store offset of the element (d l|u v) of a listed block; (i2, f2) and
// (j2, g2): the AOs of (u, v) and their function indices, in the stored
// orientation of (U, V)
__device__ __forceinline__ long long live_offset(const LiveBlock &b, int d, int fd, int l, int fl, int i2, int f2,
                                                 int j2, int g2, int n) {
  int i1 = d, fi1 = fd, j1 = l, fj1 = fl;
  if (b.flags & 1) {
    i1 = l, fi1 = fl, j1 = d, fj1 = fd;
  }
  if ((b.flags & 2) && i1 < j1) {  // A = B: the canonical element has i >= j
    const int t = i1, ft = fi1;
    i1 = j1, fi1 = fj1, j1 = t, fj1 = ft;
  }
  const bool bra1 = b.flags & 4;
  int ia = bra1 ? i1 : i2, fa = bra1 ? fi1 : f2, ja = bra1 ? j1 : j2, fb = bra1 ? fj1 : g2;
  int ka = bra1 ? i2 : i1, fc = bra1 ? f2 : fi1, la = bra1 ? j2 : j1, fdd = bra1 ? g2 : fj1;
  if ((b.flags & 8) && (long long)ia * n + ja < (long long)ka * n + la) {  // P = Q: ij >= kl
    int t = fa;
    fa = fc, fc = t;
    t = fb;
    fb = fdd, fdd = t;
  }
  const int NB = (b.flags & 16) ? 4 : 1, NC = (b.flags & 32) ? 4 : 1, ND = (b.flags & 64) ? 4 : 1;
  return b.off + ((fa * NB + fb) * NC + fc) * ND + fdd;
}

// ---- The first quarter transform straight from the quartet store.
// Y1[p][l][b] = sum_d (d l|u v) C(d, b) for the AO pairs p = (u <= v): b
// fastest, so that each row's columns are one coalesced store (the second
// step's slicing reads it transposed, ROW_TRANS).
// Over (l, p) x d the operand (d l|u v) is mostly zeros -- shell quartets that
// fail the Schwarz screen -- so instead of cutting it into BF16 planes for a
// dense tensor-core product, each warp takes one row group (L; U <= V), lists
// the stored blocks (D L|U V) and their AOs d once, and works through the
// group's rows (u, v, l) in passes of up to FQ_ROWS: it gathers the stored
// elements (d l|u v) of the pass into shared memory (FP32, each by one lane)
// and forms the products with C in FP32 on the CUDA cores -- lane k owns the
// columns b = k + 32 j, and each gathered element is one shared-memory
// broadcast for KB multiply-adds per lane.  Every lane is busy whatever the
// row count, and only stored elements are visited.
constexpr int FQ_ROWS = 8;
constexpr int FQ_KCHUNK = 64;  // listed AOs gathered at a time
constexpr int FQ_LCH = 16;      // shells L per group
constexpr int FQ_GATHER = 2;    // gathered elements in flight per lane

// row f of a group: AO pair (u, v) number f / nl of the shells U <= V (u <= v),
// l = l0 + f % nl
__device__ __forceinline__ void fq_row(int f, int nl, int u0, int nu, int v0, int nv, bool same, int &u, int &v,
                                       int &l) {
  const int pi = f / nl;
  l = f - pi * nl;
  if (!same) {
    u = u0 + pi / nv;
    v = v0 + pi % nv;
  } else {  // pairs u <= v within one shell, v outer
    int vv = 0;
    while ((vv + 1) * (vv + 2) / 2 <= pi) ++vv;
    u = u0 + (pi - vv * (vv + 1) / 2);
    v = v0 + vv;
  }
}

// rows f0 .. f0 + nr - 1 of the group (nr <= R; the others of the pass are zeros, not written).
// Not inlined: the three pass widths would otherwise triple the kernel's code,
// and its instruction fetches were a leading stall.
template <int KB, int R>
__device__ __noinline__ void fq_pass(const StoreView &sv, int n, int Kp, const float *Cf, int nvb,
                                        float *__restrict__ Y1, long long np, const int *dl, const LiveBlock *tab,
                                        int nd, float *Vs, int f0, int nr, int nl, int l0, int u0, int nu, int v0,
                                        int nv, bool same, int4 e2) {
  const int lane = threadIdx.x & 31;
  float acc[R][KB];
#pragma unroll
  for (int rr = 0; rr < R; ++rr)
#pragma unroll
    for (int j = 0; j < KB; ++j) acc[rr][j] = 0.f;
  // the listed AOs in chunks of FQ_KCHUNK: gather the chunk's elements, then
  // its products
  for (int kc = 0; kc < nd; kc += FQ_KCHUNK) {
    const int kn = min(FQ_KCHUNK, nd - kc);
    // gather: element (k, rr) by lane (k * R + rr) mod 32; FQ_GATHER
    // elements per lane at a time -- their offsets first, then every load in
    // flight together, then the shared-memory stores
    for (int base = 0; base < kn * R; base += 32 * FQ_GATHER) {
      long long off[FQ_GATHER];
#pragma unroll
      for (int t = 0; t < FQ_GATHER; ++t) {
        off[t] = -1;
        const int idx = base + lane + 32 * t;
        if (idx >= kn * R) continue;
        const int k = idx / R, rr = idx - k * R;
        if (rr >= nr) continue;
        int u, v, l;
        fq_row(f0 + rr, nl, u0, nu, v0, nv, same, u, v, l);
        int i2 = u, f2 = u - u0, j2 = v, g2 = v - v0;
        if (e2.w & 1) {
          i2 = v, f2 = v - v0, j2 = u, g2 = u - u0;
        }
        if ((e2.w & 2) && i2 < j2) {
          const int tt = i2, ft = f2;
          i2 = j2, f2 = g2, j2 = tt, g2 = ft;
        }
        const int e = dl[kc + k], d = e & 0xffff;
        const LiveBlock b = tab[e >> 16];
        off[t] = live_offset(b, d, d - b.a0, l0 + l, l, i2, f2, j2, g2, n);
      }
      double x[FQ_GATHER];
#pragma unroll
      for (int t = 0; t < FQ_GATHER; ++t) x[t] = off[t] >= 0 ? __ldg(sv.X + off[t]) : 0.0;
#pragma unroll
      for (int t = 0; t < FQ_GATHER; ++t) {
        const int idx = base + lane + 32 * t;
        if (idx < kn * R) {
          const int k = idx / R, rr = idx - k * R;
          Vs[k * FQ_ROWS + rr] = (float)x[t];
        }
      }
    }
    __syncwarp();
#pragma unroll 2
    for (int k = 0; k < kn; ++k) {
      const float *crow = Cf + (size_t)(dl[kc + k] & 0xffff) * nvb;
      float cv[KB];
#pragma unroll
      for (int j = 0; j < KB; ++j) cv[j] = lane + 32 * j < nvb ? crow[lane + 32 * j] : 0.f;
      const float *x = Vs + k * FQ_ROWS;
      if constexpr (R >= 4) {
#pragma unroll
        for (int r4 = 0; r4 < R; r4 += 4) {
          const float4 x4 = *reinterpret_cast<const float4 *>(x + r4);
#pragma unroll
          for (int j = 0; j < KB; ++j) {
            acc[r4][j] = fmaf(cv[j], x4.x, acc[r4][j]);
            acc[r4 + 1][j] = fmaf(cv[j], x4.y, acc[r4 + 1][j]);
            acc[r4 + 2][j] = fmaf(cv[j], x4.z, acc[r4 + 2][j]);
            acc[r4 + 3][j] = fmaf(cv[j], x4.w, acc[r4 + 3][j]);
          }
        }
      } else {
#pragma unroll
        for (int rr = 0; rr < R; ++rr)
#pragma unroll
          for (int j = 0; j < KB; ++j) acc[rr][j] = fmaf(cv[j], x[rr], acc[rr][j]);
      }
    }
    __syncwarp();  // Vs is read before the next chunk's gather
  }
#pragma unroll
  for (int rr = 0; rr < R; ++rr) {
    if (rr >= nr) break;
    int u, v, l;
    fq_row(f0 + rr, nl, u0, nu, v0, nv, same, u, v, l);
    const long long p = (long long)u + (long long)v * (v + 1) / 2;
#pragma unroll
    for (int j = 0; j < KB; ++j) {
      const int bb = lane + 32 * j;
      if (bb < nvb) Y1[((size_t)p * n + l0 + l) * nvb + bb] = acc[rr][j];
    }
  }
}

template <int KB>
__global__ void __launch_bounds__(256, 2) store_first_quarter_kernel(const StoreView sv, int n, int Kp,
                                                                   const float *Cf, int nvb, int cs_floats,
                                                                   float *__restrict__ Y1, long long np,
                                                                   long long ngroups) {
  extern __shared__ __align__(16) unsigned char fq_sm_raw[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int nsh = sv.nsh;
  // C in shared memory when it fits (cs_floats > 0), then per warp: gathered
  // elements [FQ_KCHUNK][FQ_ROWS] floats, listed blocks [nsh], listed AOs [n]
  float *Cs = reinterpret_cast<float *>(fq_sm_raw);
  if (cs_floats > 0) {
    for (int i = threadIdx.x; i < cs_floats; i += blockDim.x) Cs[i] = __ldg(Cf + i);
    __syncthreads();
    Cf = Cs;
  }
  // (the per-warp regions start on a 16-byte boundary: Vs is read as float4)
  unsigned char *fq_sm = fq_sm_raw + (size_t)((cs_floats + 3) & ~3) * sizeof(float);
  constexpr int VSZ = FQ_KCHUNK * FQ_ROWS;
  float *Vs = reinterpret_cast<float *>(fq_sm) + (size_t)w * VSZ;
  LiveBlock *tab = reinterpret_cast<LiveBlock *>(reinterpret_cast<float *>(fq_sm) + (size_t)nw * VSZ) +
                   (size_t)w * nsh;
  int *dl = reinterpret_cast<int *>(reinterpret_cast<LiveBlock *>(reinterpret_cast<float *>(fq_sm) +
                                                                  (size_t)nw * VSZ) +
                                    (size_t)nw * nsh) +
            (size_t)w * n;
  const long long warps = (long long)gridDim.x * nw;
  // group g: shell pair q = U + V (V + 1) / 2 (U <= V) and the chunk of FQ_LCH
  // consecutive shells L; the warp's rows then cover whole runs of l for each
  // (u, v), so the sectors of Y1 it writes are completed while in L2
  const int nch = (nsh + FQ_LCH - 1) / FQ_LCH;
  for (long long g = (long long)blockIdx.x * nw + w; g < ngroups; g += warps) {
    const long long q = g / nch;
    const int Lc = (int)(g - q * nch);
    int V1 = (int)((sqrt(8.0 * (double)q + 1.0) - 1.0) * 0.5);
    while ((long long)V1 * (V1 + 1) / 2 > q) --V1;
    while ((long long)(V1 + 1) * (V1 + 2) / 2 <= q) ++V1;
    const int U = (int)(q - (long long)V1 * (V1 + 1) / 2), Vs1 = V1;
    const int u0 = sv.ao0[U], u1 = U + 1 < nsh ? sv.ao0[U + 1] : n, nu = u1 - u0;
    const int v0 = sv.ao0[Vs1], v1 = Vs1 + 1 < nsh ? sv.ao0[Vs1 + 1] : n, nv = v1 - v0;
    const bool same = U == Vs1;
    const int4 e2 = sv.pinfo[U * nsh + Vs1];
    const double quv = sv.pbound[e2.x];
    for (int L = Lc * FQ_LCH; L < min(nsh, (Lc + 1) * FQ_LCH); ++L) {
    const int l0 = sv.ao0[L], l1 = L + 1 < nsh ? sv.ao0[L + 1] : n, nl = l1 - l0;
    // the stored blocks of the group, then their AOs d
    int cnt = 0;
    if (sv.qmax[L] * quv >= sv.thr) {
      const int *ptn = sv.partners + (size_t)L * nsh;
      for (int base = 0; base < nsh; base += 32) {
        const int k = base + lane;
        bool ok = false, live = false;
        LiveBlock b{};
        if (k < nsh) {
          const int D = ptn[k];
          const int4 e1 = sv.pinfo[D * nsh + L];
          ok = sv.pbound[e1.x] * quv >= sv.thr;
          if (ok) {
            const bool first_bra = e1.y > e2.y || (e1.y == e2.y && e1.z >= e2.z);
            const int4 eb = first_bra ? e1 : e2, ek = first_bra ? e2 : e1;
            const int K = eb.y * (eb.y + 1) / 2 + ek.y;
            live = ek.z < sv.len[K][eb.z];
            const int NB = sv_nfb(eb.y), NC = sv_nfa(ek.y), ND = sv_nfb(ek.y), NOUT = sv_nfa(eb.y) * NB * NC * ND;
            const int a0 = sv.ao0[D], a1 = D + 1 < nsh ? sv.ao0[D + 1] : n;
            b.off = sv.base[K] + (sv.off[K][eb.z] + ek.z) * NOUT;
            b.a0 = a0;
            b.flags = (e1.w & 3) | (first_bra ? 4 : 0) | (eb.x == ek.x ? 8 : 0) | (NB == 4 ? 16 : 0) |
                      (NC == 4 ? 32 : 0) | (ND == 4 ? 64 : 0) | ((a1 - a0) << 8);
          }
        }
        const unsigned lv = __ballot_sync(0xffffffffu, live);
        if (live) tab[cnt + __popc(lv & ((1u << lane) - 1))] = b;
        cnt += __popc(lv);
        if (!__all_sync(0xffffffffu, ok)) break;
      }
    }
    __syncwarp();
    int nd = 0;  // listed AOs: dl[k] = d | (block << 16)
    for (int base = 0; base < cnt; base += 32) {
      const int t = base + lane;
      const int na = t < cnt ? (tab[t].flags >> 8) : 0;
      int incl = na;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
      }
      const int pos = nd + incl - na;
      for (int i = 0; i < na; ++i) dl[pos + i] = (tab[t].a0 + i) | (t << 16);
      nd += __shfl_sync(0xffffffffu, incl, 31);
    }
    __syncwarp();
    const int rows = (same ? nu * (nu + 1) / 2 : nu * nv) * nl;
    for (int f0 = 0; f0 < rows;) {
      const int left = rows - f0;
      if (left >= 5 && KB <= 2) {
        const int nr = min(left, 8);
        fq_pass<KB, 8>(sv, n, Kp, Cf, nvb, Y1, np, dl, tab, nd, Vs, f0, nr, nl, l0, u0, nu, v0, nv, same, e2);
        f0 += nr;
      } else if (left >= 2) {
        const int nr = min(left, 4);
        fq_pass<KB, 4>(sv, n, Kp, Cf, nvb, Y1, np, dl, tab, nd, Vs, f0, nr, nl, l0, u0, nu, v0, nv, same, e2);
        f0 += nr;
      } else {
        fq_pass<KB, 1>(sv, n, Kp, Cf, nvb, Y1, np, dl, tab, nd, Vs, f0, 1, nl, l0, u0, nu, v0, nv, same, e2);
        f0 += 1;
      }
    }
    __syncwarp();  // the tables are read before the next shell L's
    }
  }
}

// C(d, b) as FP32, b fastest
__global__ void coef_f32_kernel(const double *__restrict__ C, int n, int nvb, float *__restrict__ Cf) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n * nvb) return;
  const int d = i / nvb, b = i % nvb;
  Cf[i] = (float)C[d + (size_t)n * b];
}

// ------------------------------------------------------------------ host side
// a sliced operand: S planes of `plane` elements from `base`, row exponents `e`
struct Sliced {
  bf16 *base;
  long long plane;
  int *e;
};

template <int S>
static int slice_gemm(mq_ctx *c, Sliced A, long long M, int batch, long long a_batch_stride, Sliced B, int N, int Kp,
                      GemmArgs g) {
  if (N <= 0 || M <= 0 || batch <= 0) return MQ_OK;
  if (N > 256) return set_err(c, MQ_EINVAL, "split GEMM: N > 256");
  if (M > 2147483647LL) return set_err(c, MQ_EINVAL, "split GEMM: M too large");
  Maps maps;
  const int ntile = (N + 15) / 16 * 16;
  for (int p = 0; p < S; ++p) {
    MQ_TRY(make_map(c, &maps.a[p], A.base + p * A.plane, Kp, M, batch, a_batch_stride, UM));
    MQ_TRY(make_map(c, &maps.b[p], B.base + p * B.plane, Kp, N, 1, 0, ntile));
  }
  g.M = (int)M;
  g.N = N;
  g.K = Kp;
  g.batch = batch;
  g.ntile = ntile;
  g.eA = A.e;
  g.eB = B.e;
  int cols = 32;
  while (cols < S * ntile) cols <<= 1;
  if (cols > 512) return set_err(c, MQ_EINVAL, "split GEMM: accumulators exceed TMEM");
  g.tmem_cols = cols;
  const size_t stage = (size_t)S * ((size_t)UM * UK * 2 + (size_t)ntile * UK * 2);
  const size_t limit = 227 * 1024 - 1024 - 256;
  if (limit < 2 * stage) return set_err(c, MQ_EINVAL, "split GEMM: shared memory");
  const int stages = limit >= 4 * stage ? 4 : (limit >= 3 * stage ? 3 : 2);
  const size_t smem = stages * stage + 1024 + 256;
  int sms = 148;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
  const long long tiles = (M + UM - 1) / UM * batch;
  const int grid = (int)std::min<long long>(tiles, sms);
  auto kern = stages == 4 ? slice_gemm_kernel<S, 4> : (stages == 3 ? slice_gemm_kernel<S, 3> : slice_gemm_kernel<S, 2>);
  MQ_CUDA(c, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  kern<<<grid, GEMM_THREADS, smem, c->stream>>>(maps, g);
  c->stats.launches += 1;
  MQ_CUDA(c, cudaGetLastError());
  return sync_check(c, "slice_gemm");
}

template <int S, int MODE = ROW_PLAIN, class T>
static int slice_rows(mq_ctx *c, const T *in, long long rows, int kvalid, long long ld, int Kp, Sliced o,
                      RowSrc rs = RowSrc{nullptr, 1, 0, 1}) {
  if (Kp % 8 || Kp > 512) return set_err(c, MQ_EINVAL, "slice_rows: Kp must be a multiple of 8 up to 512");
  const int tb = 256;
  const long long blocks = std::max<long long>(1, std::min<long long>((rows + 7) / 8, 1 << 20));
  const int per16 = 16 / (int)sizeof(T);
  const int vec = MODE != ROW_SYMM && MODE != ROW_TRANS && ((uintptr_t)in % 16 == 0) && (ld % per16 == 0) &&
                  (kvalid % per16 == 0);
  if (Kp <= 256)
    slice_rows_kernel<S, T, 1, MODE><<<(unsigned)blocks, tb, 0, c->stream>>>(in, rows, kvalid, ld, Kp, o.plane,
                                                                             o.base, o.e, vec, rs);
  else
    slice_rows_kernel<S, T, 2, MODE><<<(unsigned)blocks, tb, 0, c->stream>>>(in, rows, kvalid, ld, Kp, o.plane,
                                                                             o.base, o.e, vec, rs);
  c->stats.launches += 1;
  MQ_CUDA(c, cudaGetLastError());
  return sync_check(c, "slice_rows");
}

// (u, v) of every AO pair u <= v at p = u + v (v + 1) / 2
__global__ void pair_table_kernel(int n, int2 *__restrict__ pairs) {
  const int u = blockIdx.x * blockDim.x + threadIdx.x, v = blockIdx.y;
  if (u <= v && v < n) pairs[u + (long long)v * (v + 1) / 2] = make_int2(u, v);
}

static int pair_table(mq_ctx *c, int n, const int2 **out) {
  const long long np = (long long)n * (n + 1) / 2;
  int2 *d = (int2 *)buf(c, "ao2mo_pairs", np * sizeof(int2));
  if (!d) return MQ_ENOMEM;
  pair_table_kernel<<<dim3((n + 127) / 128, n), 128, 0, c->stream>>>(n, d);
  c->stats.launches += 1;
  MQ_CUDA(c, cudaGetLastError());
  *out = d;
  return MQ_OK;
}

// The quartet store as the first step's slicing reads it.
static StoreView store_view(mq_ctx *c) {
  const QStore &qs = c->qs;
  StoreView v{};
  v.X = qs.X;
  v.pinfo = qs.pinfo;
  v.ao_shell = qs.ao_shell;
  v.ao0 = qs.shell_ao0;
  for (int k = 0; k < 6; ++k) {
    v.off[k] = qs.combo[k].off;
    v.len[k] = qs.combo[k].len;
    v.base[k] = qs.combo[k].base;
  }
  v.nsh = c->nshell;
  v.pbound = c->pt.schwarz;
  v.qmax = qs.shell_qmax;
  v.partners = qs.partners;
  v.thr = qs.thr;
  return v;
}

// A operand of the first step -- XX(d, l, u, v), rows (l, u <= v), K = d --
// cut into S planes from the n^4 array
template <int S>
static int slice_xx(mq_ctx *c, long long n, int Kp, Sliced A, const int2 *pairs) {
  const long long np = n * (n + 1) / 2;
  if (c->nparts > 1) return set_err(c, MQ_EINVAL, "the transform needs every integral: reset the partition first");
  MQ_TRY(ensure_xx_full(c));
  return slice_rows<S, ROW_PAIRS>(c, c->d_XX, n * np, (int)n, n, Kp, A, RowSrc{pairs, n, np, 1});
}

// Y1[p][l][b] from the quartet store and C(:, b), b < nvb
static int store_first_quarter(mq_ctx *c, long long n, int Kp, const double *Cb, int nvb, float *y1, long long np) {
  const int nsh = c->nshell, nw = 256 / 32;
  float *Cf = (float *)buf(c, "fq_coef", sizeof(float) * (size_t)n * std::max(nvb, 1));
  if (!Cf) return MQ_ENOMEM;
  coef_f32_kernel<<<(unsigned)((n * nvb + 255) / 256), 256, 0, c->stream>>>(Cb, (int)n, nvb, Cf);
  const long long groups = (long long)nsh * (nsh + 1) / 2 * ((nsh + FQ_LCH - 1) / FQ_LCH);
  size_t sm = (size_t)nw * ((size_t)FQ_KCHUNK * FQ_ROWS * sizeof(float) + (size_t)n * sizeof(int) +
                            (size_t)nsh * sizeof(LiveBlock));
  // C in shared memory when the CTA still fits twice per SM
  const int cs_floats = sm + (size_t)n * nvb * sizeof(float) <= 110 * 1024 ? (int)(n * nvb) : 0;
  sm += (size_t)((cs_floats + 3) & ~3) * sizeof(float);
  if (sm > 200 * 1024) return set_err(c, MQ_EINVAL, "split transform: too many shells for the store transform");
  if (n > 0xffff || nsh > 0xffff) return set_err(c, MQ_EINVAL, "split transform: too many AOs for the store transform");
  auto kern = nvb <= 32 ? store_first_quarter_kernel<1>
                        : (nvb <= 64 ? store_first_quarter_kernel<2>
                                     : (nvb <= 128 ? store_first_quarter_kernel<4> : store_first_quarter_kernel<8>));
  // (with KB >= 4, passes of at most 4 rows keep the accumulators in registers)
  MQ_CUDA(c, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
  const long long blocks = std::max<long long>(1, std::min<long long>((groups + nw - 1) / nw, (long long)sms * 16));
  kern<<<(unsigned)blocks, 256, sm, c->stream>>>(store_view(c), (int)n, Kp, Cf, nvb, cs_floats, y1, np, groups);
  c->stats.launches += 2;
  MQ_CUDA(c, cudaGetLastError());
  return sync_check(c, "store_first_quarter");
}

template <int S>
static int ao2mo_slices(mq_ctx *c, const double *Ci, int no1, const double *Ca, int nv1, const double *Cj, int no2,
                        const double *Cb, int nv2, double *d_out) {
  const long long n = c->nao;
  const int Kp = (int)((n + 7) / 8 * 8);
  if (no1 > 256 || nv1 > 256 || no2 > 256 || nv2 > 256)
    return set_err(c, MQ_EINVAL, "split transform: orbital blocks above 256 are not supported");
  if (Kp > SLICE_KMAX) return set_err(c, MQ_EINVAL, "split transform: more than 340 basis functions");
  MQ_TRY(join_side(c));  // a prefetch of the XX slices, before any buffer is touched
  const long long n2 = n * n, n3 = n2 * n;
  // A operand rows per step, and the FP32 intermediates [rows][Kp]
  // the first step reads the quartet store directly when there is no n^4 array
  const bool from_store = !c->xx_valid && c->qs.valid;
  if (from_store && c->nparts > 1)
    return set_err(c, MQ_EINVAL, "the transform needs every integral: reset the partition first");
  const long long rX = from_store ? 0 : n3, r1 = (long long)nv2 * n2, r2 = (long long)no2 * nv2 * n,
                  r3 = (long long)nv1 * no2 * nv2;
  const long long rB = (long long)no1 + nv1 + no2 + nv2;
  const long long rmax = std::max(std::max(rX, r1), std::max(r2, r3));
  bf16 *pa = (bf16 *)buf(c, "slice_a", S * rmax * Kp * sizeof(bf16));
  int *ea = (int *)buf(c, "slice_ea", rmax * sizeof(int));
  bf16 *pb = (bf16 *)buf(c, "slice_b", S * rB * Kp * sizeof(bf16));
  int *eb = (int *)buf(c, "slice_eb", rB * sizeof(int));
  float *y1 = (float *)buf(c, "slice_y1", std::max(r1, r3) * Kp * sizeof(float));
  float *y2 = (float *)buf(c, "slice_y2", r2 * Kp * sizeof(float));
  int *err = (int *)buf(c, "split_err", 64);
  if (!pa || !ea || !pb || !eb || !y1 || !y2 || !err) return MQ_ENOMEM;
  MQ_CUDA(c, cudaMemsetAsync(err, 0, sizeof(int), c->stream));
  // the padding columns Kp > n of the intermediates are never read: slicing reads n values per row
  // coefficient blocks: column p of C (n contiguous) becomes row p of B (K-major)
  const long long plB = rB * Kp;
  Sliced Bi{pb, plB, eb}, Ba{pb + (long long)no1 * Kp, plB, eb + no1};
  Sliced Bj{Ba.base + (long long)nv1 * Kp, plB, Ba.e + nv1}, Bb{Bj.base + (long long)no2 * Kp, plB, Bj.e + no2};
  MQ_TRY(slice_rows<S>(c, Ci, no1, (int)n, n, Kp, Bi));
  MQ_TRY(slice_rows<S>(c, Ca, nv1, (int)n, n, Kp, Ba));
  MQ_TRY(slice_rows<S>(c, Cj, no2, (int)n, n, Kp, Bj));
  MQ_TRY(slice_rows<S>(c, Cb, nv2, (int)n, n, Kp, Bb));
  GemmArgs g{};
  g.err = err;
  // (uv|ld) = (vu|ld): the first two steps run over the AO pairs p = (u <= v)
  // only, half of the rows; the third reads (u, v) and (v, u) from the same
  // packed element.
  const long long np = n * (n + 1) / 2, rXp = n * np;
  const int2 *pairs = nullptr;
  MQ_TRY(pair_table(c, (int)n, &pairs));
  const RowSrc rs{pairs, n, np, 1};
  // 1: XX(d,l,u,v) at d + n*((l,u,v)): rows (l,p), K = d -> Y1[b][p][l]:
  // from the quartet store on the CUDA cores (FP32), else from the n^4 array
  // by the tensor cores (its slices already cut on the side stream when the
  // SCF prefetched them)
  Sliced A{pa, rX * Kp, ea};
  c->stats.ms_ao2mo_first = 0;
  if (from_store) {
    StageTimer t1;
    t1.start(c->stream);
    MQ_TRY(store_first_quarter(c, n, Kp, Cb, nv2, y1, np));
    t1.stop(c->stream);
    t1.collect_sync();
    c->stats.ms_ao2mo_first = t1.total;
  } else {
    if (c->xx_sliced != S) MQ_TRY(slice_xx<S>(c, n, Kp, A, pairs));
    c->xx_sliced = 0;  // step 2 overwrites the slices
    g.out_f64 = 0;
    g.out32 = y1;
    g.mdiv = n;
    g.s_m0 = 1;
    g.s_m1 = Kp;
    g.s_n = np * Kp;
    g.s_b = 0;
    MQ_TRY(slice_gemm<S>(c, A, rXp, 1, 0, Bb, nv2, Kp, g));
  }
  // 2: batch b; rows p, K = l -> Y2[j,b][p] (packed pairs)
  const long long r1p = (long long)nv2 * np;
  A = Sliced{pa, r1p * Kp, ea};
  if (from_store)  // Y1 as [p][l][b]
    MQ_TRY((slice_rows<S, ROW_TRANS>(c, y1, r1p, (int)n, 0, Kp, A, RowSrc{nullptr, n, np, nv2})));
  else
    MQ_TRY(slice_rows<S>(c, y1, r1p, (int)n, Kp, Kp, A));
  g.out32 = y2;
  g.mdiv = 1ll << 62;
  g.s_m0 = 1;
  g.s_m1 = 0;
  g.s_n = np;
  g.s_b = (long long)no2 * np;
  MQ_TRY(slice_gemm<S>(c, A, np, nv2, np * Kp, Bj, no2, Kp, g));
  // 3: batch (j + no2*b); rows v, K = u (gathered from the packed pairs) -> Y3[a + nv1*(j + no2*b)][v]
  A = Sliced{pa, r2 * Kp, ea};
  MQ_TRY((slice_rows<S, ROW_SYMM>(c, y2, r2, (int)n, 0, Kp, A, rs)));
  g.out32 = y1;  // Y1 is dead
  g.mdiv = 1ll << 62;
  g.s_m0 = 1;
  g.s_m1 = 0;
  g.s_n = Kp;
  g.s_b = (long long)nv1 * Kp;
  MQ_TRY(slice_gemm<S>(c, A, n, no2 * nv2, n * Kp, Ba, nv1, Kp, g));
  // 4: rows (a, j, b), K = v -> Om(i, a, j, b) = D[m][i] at i + no1*m
  A = Sliced{pa, r3 * Kp, ea};
  MQ_TRY(slice_rows<S>(c, y1, r3, (int)n, Kp, Kp, A));
  g.out_f64 = 1;
  g.out64 = d_out;
  g.mdiv = 1ll << 62;
  g.s_m0 = no1;
  g.s_m1 = 0;
  g.s_n = 1;
  g.s_b = 0;
  MQ_TRY(slice_gemm<S>(c, A, r3, 1, 0, Bi, no1, Kp, g));
  int h = 0;
  MQ_CUDA(c, cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  MQ_CUDA(c, cudaStreamSynchronize(c->stream));
  if (h) return set_err(c, MQ_ETIMEOUT, "split GEMM pipeline wait timed out");
  return MQ_OK;
}

int join_side(mq_ctx *c) {
  if (!c->side_pending) return MQ_OK;
  MQ_CUDA(c, cudaStreamWaitEvent(c->stream, c->ev_side, 0));
  c->side_pending = 0;
  return MQ_OK;
}

// The first step's A operand -- XX cut into S planes, rows (l,u,v), K = d --
// depends on XX alone, so it can be formed before the orbitals exist: on the
// side stream (lowest priority) while the main stream finishes the SCF.  The
// buffers are the ones ao2mo_slices uses, at the sizes it asks for (the
// largest A operand of the four steps is XX itself: n^3 rows).
template <int S>
static int preslice(mq_ctx *c) {
  const long long n = c->nao;
  const int Kp = (int)((n + 7) / 8 * 8);
  // nothing to cut ahead without the n^4 array: the first step then reads the
  // quartet store itself, after the SCF (and a transform of more than 340
  // functions is rejected anyway)
  if (Kp > SLICE_KMAX || !c->xx_valid) return MQ_OK;
  const long long rX = n * n * n;
  bf16 *pa = (bf16 *)buf(c, "slice_a", S * rX * Kp * sizeof(bf16));
  int *ea = (int *)buf(c, "slice_ea", rX * sizeof(int));
  if (!pa || !ea) return MQ_ENOMEM;
  if (!c->side) {
    int lo = 0, hi = 0;
    MQ_CUDA(c, cudaDeviceGetStreamPriorityRange(&lo, &hi));
    MQ_CUDA(c, cudaStreamCreateWithPriority(&c->side, cudaStreamNonBlocking, lo));
    MQ_CUDA(c, cudaEventCreateWithFlags(&c->ev_main, cudaEventDisableTiming));
    MQ_CUDA(c, cudaEventCreateWithFlags(&c->ev_side, cudaEventDisableTiming));
  }
  const int2 *pairs = nullptr;
  MQ_TRY(pair_table(c, (int)n, &pairs));  // on the main stream, before the event below
  MQ_CUDA(c, cudaEventRecord(c->ev_main, c->stream));
  MQ_CUDA(c, cudaStreamWaitEvent(c->side, c->ev_main, 0));
  cudaStream_t main = c->stream;
  c->stream = c->side;  // the slicing launches on c->stream
  const int rc = slice_xx<S>(c, n, Kp, Sliced{pa, rX * Kp, ea}, pairs);
  c->stream = main;
  MQ_TRY(rc);
  MQ_CUDA(c, cudaEventRecord(c->ev_side, c->side));
  c->side_pending = 1;
  c->xx_sliced = S;
  return MQ_OK;
}

int ao2mo_preslice_xx(mq_ctx *c) {
  if (c->ao2mo_prefetch == 3) return preslice<3>(c);
  if (c->ao2mo_prefetch == 2) return preslice<2>(c);
  return MQ_OK;
}

int ao2mo_split_device(mq_ctx *c, const double *Ci, int no1, const double *Ca, int nv1, const double *Cj, int no2,
                       const double *Cb, int nv2, double *d_out, int planes) {
  if (planes == 3) return ao2mo_slices<3>(c, Ci, no1, Ca, nv1, Cj, no2, Cb, nv2, d_out);
  return ao2mo_slices<2>(c, Ci, no1, Ca, nv1, Cj, no2, Cb, nv2, d_out);
}

}  // namespace mq
