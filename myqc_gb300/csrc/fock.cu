// fock.cu -- two-electron Fock matrix from the device-resident full XX.
//
// Replaces RHFI2G (src/I2G/RHFI2G.f90:80-90) and UHFI2G (src/I2G/UHFI2G.f90:80-93).
// For symmetric densities the reference's
//   G_ij = sum_kl D_kl [(ij|kl) - 1/4 (ik|jl) - 1/4 (il|jk)]
// is J - K/2 with J_ij = sum_kl (ij|kl) D_kl and K_ij = sum_kl (ik|jl) D_kl; UHF
// uses G^a = J[Da+Db] - K[Da], G^b = J[Da+Db] - K[Db].
//
// One streaming pass over XX.  The slab S = XX(:,:,i,j) (n^2 contiguous
// doubles, (kl|ij) for all k,l) gives J_ij = <S, Dt> and adds S . D(:,j) to
// column i of K.  A CTA owns one i and a chunk of j: J_ij is complete inside
// the CTA, and the chunk's partial K column goes to a scratch slice; a second
// kernel sums the slices in a fixed order.  No atomics, deterministic.
#include <algorithm>
#include <cstring>
#include <mutex>

#include "internal.h"

namespace mq {

constexpr int FOCK_THREADS = 256;

// ---- double-float arithmetic on the FP32 pipes ----------------------------
// GB300 issues FP32 at many times its FP64 rate, so the digestion keeps its
// sums as unevaluated float pairs (hi + lo, ~48-bit significand).  An integral
// x is split into hi + lo floats with integer operations only: hi takes the
// top 24 significand bits, lo the next 24 of the remainder (both truncated;
// |x - hi - lo| < 2^-47 |x|; values below the FP32 normal range become 0).
__device__ __forceinline__ float2 split_f64(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned hi32 = (unsigned)(b >> 32);
  const unsigned sign = hi32 & 0x80000000u;
  const int E = (int)((hi32 >> 20) & 0x7ff);
  const int e8 = E - 896;  // FP32 biased exponent of x
  if (e8 <= 0 || e8 >= 255) return make_float2(0.f, 0.f);
  const unsigned long long frac = b & 0xfffffffffffffull;
  const float h = __uint_as_float(sign | ((unsigned)e8 << 23) | (unsigned)(frac >> 29));
  const unsigned rem = (unsigned)(frac & 0x1fffffffu);  // value rem * 2^(E - 1075)
  float l = 0.f;
  if (rem) {
    const int msb = 31 - __clz(rem);  // 0..28
    const int el = msb + E - 948;     // FP32 biased exponent of the remainder
    if (el > 0) {
      const unsigned mant = msb >= 23 ? (rem >> (msb - 23)) : (rem << (23 - msb));
      l = __uint_as_float(sign | ((unsigned)el << 23) | (mant & 0x7fffffu));
    }
  }
  return make_float2(h, l);
}

// s += x * d in double-float: exact hi product (FMA), cross terms, two-sum
__device__ __forceinline__ void dfma(float2 &s, float2 x, float2 d) {
  const float ph = x.x * d.x;
  const float pe = fmaf(x.x, d.x, -ph);
  const float cr = fmaf(x.x, d.y, x.y * d.x);
  const float t = s.x + ph;
  const float bb = t - s.x;
  const float err = (s.x - (t - bb)) + (ph - bb);
  s.x = t;
  s.y += err + (pe + cr);
}

// density hi/lo pairs: DJ from Da (+ Db), DKa from Da, DKb from Db (UHF)
__global__ void split_density_kernel(const double *__restrict__ Da, const double *__restrict__ Db, size_t n2,
                                     float2 *__restrict__ DJ, float2 *__restrict__ DKa, float2 *__restrict__ DKb) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n2) return;
  const double a = Da[i];
  if (Db) {
    const double b = Db[i];
    DJ[i] = split_f64(a + b);
    DKa[i] = split_f64(a);
    DKb[i] = split_f64(b);
  } else {
    DJ[i] = split_f64(a);
  }
}

template <bool UHF>
__global__ void __launch_bounds__(FOCK_THREADS) fock_slab_kernel(const double *__restrict__ XX,
                                                                 const float2 *__restrict__ DJ,
                                                                 const float2 *__restrict__ DKa,
                                                                 const float2 *__restrict__ DKb, int n, int jchunk,
                                                                 double *__restrict__ J, double *__restrict__ Kpa,
                                                                 double *__restrict__ Kpb) {
  const int i = blockIdx.x, chunk = blockIdx.y;
  const int j0 = chunk * jchunk, j1 = min(n, j0 + jchunk);
  const size_t N = n, n2 = N * N;
  __shared__ double red[FOCK_THREADS / 32];
  // each thread owns rows k = tid, tid + 256, ... (at most 4 rows: n <= 1024)
  double ka[4] = {0, 0, 0, 0}, kb[4] = {0, 0, 0, 0};
  for (int j = j0; j < j1; ++j) {
    const double *S = XX + n2 * ((size_t)i + N * j);
    double jsum = 0.0;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int k = threadIdx.x + r * FOCK_THREADS;
      if (k >= n) break;
      float2 sa = make_float2(0.f, 0.f), sb = sa, sj = sa;
#pragma unroll 4
      for (int l = 0; l < n; ++l) {
        const float2 x = split_f64(__ldcs(S + k + N * l));  // streamed once: do not keep in L2
        dfma(sj, x, DJ[k + N * l]);
        dfma(sa, x, DKa[l + N * j]);
        if (UHF) dfma(sb, x, DKb[l + N * j]);
      }
      jsum += (double)sj.x + (double)sj.y;
      ka[r] += (double)sa.x + (double)sa.y;
      if (UHF) kb[r] += (double)sb.x + (double)sb.y;
    }
    // block reduction of J_ij
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) jsum += __shfl_xor_sync(0xffffffffu, jsum, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = jsum;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (int w = 0; w < FOCK_THREADS / 32; ++w) t += red[w];
      J[i + N * j] = t;
    }
    __syncthreads();
  }
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int k = threadIdx.x + r * FOCK_THREADS;
    if (k >= n) break;
    Kpa[n2 * chunk + k + N * i] = ka[r];
    if (UHF) Kpb[n2 * chunk + k + N * i] = kb[r];
  }
}

// G = J - f*K_total with K_total the sum of the chunk slices (fixed order),
// symmetrised as (K_ij + K_ji)/2.  J_ij and J_ji come from identical slabs in
// the same order and are equal bit for bit; K_ij and K_ji come from different
// slabs and differ by rounding, which the eigensolver must not see as an
// off-diagonal residue it cannot rotate away.
__global__ void fock_combine_kernel(const double *__restrict__ J, const double *__restrict__ Kp, int nchunk, int n,
                                    double f, double *__restrict__ G) {
  const size_t N = n, n2 = N * N;
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n2) return;
  const size_t tdx = (idx % N) * N + idx / N;
  double k = 0.0, kt = 0.0;
  for (int c = 0; c < nchunk; ++c) {
    k += Kp[n2 * c + idx];
    kt += Kp[n2 * c + tdx];
  }
  G[idx] = J[idx] - f * (0.5 * (k + kt));
}

int fock_stored_device(mq_ctx *c, const double *d_Da, const double *d_Db, double *d_Ga, double *d_Gb) {
  const int n = c->nao;
  if (!c->d_XX) return set_err(c, MQ_ESTATE, "no integrals on the device (call mq_eri_store or mq_eri_upload)");
  if (n > 4 * FOCK_THREADS) return set_err(c, MQ_EINVAL, "stored Fock build supports n <= 1024");
  const bool uhf = d_Db != nullptr;
  // chunks of j so that the grid covers the GPU about 4 times
  int sms = 148;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
  int nchunk = std::max(1, std::min(n, (4 * sms + n - 1) / n));
  const int jchunk = (n + nchunk - 1) / nchunk;
  nchunk = (n + jchunk - 1) / jchunk;
  const size_t n2 = (size_t)n * n;
  double *J = (double *)buf(c, "fock_partials", sizeof(double) * n2 * (1 + nchunk * (uhf ? 2 : 1)));
  float2 *DJ = (float2 *)buf(c, "fock_dsplit", sizeof(float2) * n2 * (uhf ? 3 : 1));
  if (!J || !DJ) return MQ_ENOMEM;
  double *Kpa = J + n2, *Kpb = uhf ? Kpa + n2 * nchunk : nullptr;
  float2 *DKa = uhf ? DJ + n2 : DJ, *DKb = uhf ? DJ + 2 * n2 : nullptr;
  const int tb = 256;
  const unsigned gb = (unsigned)((n2 + tb - 1) / tb);
  split_density_kernel<<<gb, tb, 0, c->stream>>>(d_Da, d_Db, n2, DJ, DKa, DKb);
  dim3 grid(n, nchunk);
  if (uhf)
    fock_slab_kernel<true><<<grid, FOCK_THREADS, 0, c->stream>>>(c->d_XX, DJ, DKa, DKb, n, jchunk, J, Kpa, Kpb);
  else
    fock_slab_kernel<false><<<grid, FOCK_THREADS, 0, c->stream>>>(c->d_XX, DJ, DKa, nullptr, n, jchunk, J, Kpa,
                                                                  nullptr);
  MQ_CUDA(c, cudaGetLastError());
  fock_combine_kernel<<<gb, tb, 0, c->stream>>>(J, Kpa, nchunk, n, uhf ? 1.0 : 0.5, d_Ga);
  if (uhf) fock_combine_kernel<<<gb, tb, 0, c->stream>>>(J, Kpb, nchunk, n, 1.0, d_Gb);
  c->stats.launches += uhf ? 4 : 3;
  MQ_CUDA(c, cudaGetLastError());
  return MQ_OK;
}

// ---------------------------------------------------------------------------
// Allocation-free RHF Fock build (mq_fock_rhf_noalloc).
//
// For callers that may not allocate device memory themselves -- a Fortran or
// C host whose device arrays are owned by an OpenACC / OpenMP-offload runtime
// or by a preallocated pool, or code that must not call cudaMalloc while it
// runs -- the same two kernels as fock_stored_device run on caller-owned
// device buffers, with their scratch (J and the per-chunk K columns) in the
// fixed array below instead of a context buffer.  The array is part of the
// loaded library: every GPU that loads libmyqc holds its 16 MiB until the
// process exits.  Host code cannot use the array's name as a device address;
// the first call on each device looks the address up with
// cudaGetSymbolAddress (with that device current) and keeps it.
constexpr size_t NOALLOC_SCRATCH_DOUBLES = (size_t)2 << 20;  // 16 MiB
static __device__ __align__(256) double g_fock_noalloc_scratch[NOALLOC_SCRATCH_DOUBLES];
constexpr int NOALLOC_MAX_DEVICES = 64;
static double *g_fock_noalloc_addr[NOALLOC_MAX_DEVICES];
static std::mutex g_fock_noalloc_mu;

static int noalloc_fail(char *msg, int len, int code, const char *what) {
  if (msg && len > 0) {
    strncpy(msg, what, len - 1);
    msg[len - 1] = 0;
  }
  return code;
}

}  // namespace mq

extern "C" int mq_fock_rhf_noalloc(int n, const double *d_XX, const double *d_D, double *d_G, void *stream,
                                   char *msg, int msglen) {
  using namespace mq;
  if (n <= 0 || !d_XX || !d_D || !d_G) return noalloc_fail(msg, msglen, MQ_EINVAL, "null pointer or n <= 0");
  if (n > 4 * FOCK_THREADS) return noalloc_fail(msg, msglen, MQ_EINVAL, "n > 1024 is not supported");
  const size_t n2 = (size_t)n * n;
  // J, the split density (one float pair per element) and at least one K
  // slice must fit the fixed scratch: 3 n^2 <= 2 Mi doubles (n <= 836)
  if (3 * n2 > NOALLOC_SCRATCH_DOUBLES)
    return noalloc_fail(msg, msglen, MQ_EINVAL, "scratch too small: 3 n^2 must not exceed 2097152 doubles (n <= 836)");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NOALLOC_MAX_DEVICES)
    return noalloc_fail(msg, msglen, MQ_ECUDA, "cudaGetDevice failed");
  double *scr = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_fock_noalloc_mu);
    if (!g_fock_noalloc_addr[dev]) {
      void *p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_fock_noalloc_scratch);
      if (e != cudaSuccess || !p) return noalloc_fail(msg, msglen, MQ_ECUDA, cudaGetErrorString(e));
      g_fock_noalloc_addr[dev] = (double *)p;
    }
    scr = g_fock_noalloc_addr[dev];
  }
  int sms = 148;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int nmax = (int)(NOALLOC_SCRATCH_DOUBLES / n2) - 2;  // K slices that fit beside J and the density
  int nchunk = std::max(1, std::min({n, (4 * sms + n - 1) / n, nmax}));
  const int jchunk = (n + nchunk - 1) / nchunk;
  nchunk = (n + jchunk - 1) / jchunk;
  // every split-density, J and K-slice element is written by an earlier
  // kernel before a later one reads it, so nothing needs clearing between calls
  double *J = scr;
  float2 *Ds = (float2 *)(scr + n2);
  double *Kp = scr + 2 * n2;
  cudaStream_t s = (cudaStream_t)stream;
  split_density_kernel<<<(unsigned)((n2 + 255) / 256), 256, 0, s>>>(d_D, nullptr, n2, Ds, Ds, nullptr);
  fock_slab_kernel<false><<<dim3(n, nchunk), FOCK_THREADS, 0, s>>>(d_XX, Ds, Ds, nullptr, n, jchunk, J, Kp, nullptr);
  fock_combine_kernel<<<(unsigned)((n2 + 255) / 256), 256, 0, s>>>(J, Kp, nchunk, n, 0.5, d_G);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return noalloc_fail(msg, msglen, MQ_ECUDA, cudaGetErrorString(e));
  return MQ_OK;
}
