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

template <bool UHF>
__global__ void __launch_bounds__(FOCK_THREADS) fock_slab_kernel(const double *__restrict__ XX,
                                                                 const double *__restrict__ Da,
                                                                 const double *__restrict__ Db, int n, int jchunk,
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
      double sa = 0.0, sb = 0.0, sj = 0.0;
      for (int l = 0; l < n; ++l) {
        const double x = __ldcs(S + k + N * l);  // streamed once: do not keep in L2
        const double dal = __ldg(Da + l + N * j);
        const double dkl = UHF ? __ldg(Da + k + N * l) + __ldg(Db + k + N * l) : __ldg(Da + k + N * l);
        sj = fma(x, dkl, sj);
        sa = fma(x, dal, sa);
        if (UHF) sb = fma(x, __ldg(Db + l + N * j), sb);
      }
      jsum += sj;
      ka[r] += sa;
      if (UHF) kb[r] += sb;
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

// G = J - f*K_total with K_total the sum of the chunk slices (fixed order)
__global__ void fock_combine_kernel(const double *__restrict__ J, const double *__restrict__ Kp, int nchunk,
                                    size_t n2, double f, double *__restrict__ G) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n2) return;
  double k = 0.0;
  for (int c = 0; c < nchunk; ++c) k += Kp[n2 * c + idx];
  G[idx] = J[idx] - f * k;
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
  if (!J) return MQ_ENOMEM;
  double *Kpa = J + n2, *Kpb = uhf ? Kpa + n2 * nchunk : nullptr;
  dim3 grid(n, nchunk);
  if (uhf)
    fock_slab_kernel<true><<<grid, FOCK_THREADS, 0, c->stream>>>(c->d_XX, d_Da, d_Db, n, jchunk, J, Kpa, Kpb);
  else
    fock_slab_kernel<false><<<grid, FOCK_THREADS, 0, c->stream>>>(c->d_XX, d_Da, nullptr, n, jchunk, J, Kpa, nullptr);
  MQ_CUDA(c, cudaGetLastError());
  const int tb = 256;
  const unsigned gb = (unsigned)((n2 + tb - 1) / tb);
  fock_combine_kernel<<<gb, tb, 0, c->stream>>>(J, Kpa, nchunk, n2, uhf ? 1.0 : 0.5, d_Ga);
  if (uhf) fock_combine_kernel<<<gb, tb, 0, c->stream>>>(J, Kpb, nchunk, n2, 1.0, d_Gb);
  c->stats.launches += uhf ? 3 : 2;
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
  // J plus at least one K slice must fit the fixed scratch: 2 n^2 <= 2 Mi doubles
  if (2 * n2 > NOALLOC_SCRATCH_DOUBLES)
    return noalloc_fail(msg, msglen, MQ_EINVAL, "scratch too small: 2 n^2 must not exceed 2097152 doubles");
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
  const int nmax = (int)(NOALLOC_SCRATCH_DOUBLES / n2) - 1;  // K slices that fit beside J
  int nchunk = std::max(1, std::min({n, (4 * sms + n - 1) / n, nmax}));
  const int jchunk = (n + nchunk - 1) / nchunk;
  nchunk = (n + jchunk - 1) / jchunk;
  // every J element and every K slice element is written by the first kernel
  // before the second reads it, so nothing needs clearing between calls
  double *J = scr, *Kp = scr + n2;
  cudaStream_t s = (cudaStream_t)stream;
  fock_slab_kernel<false><<<dim3(n, nchunk), FOCK_THREADS, 0, s>>>(d_XX, d_D, nullptr, n, jchunk, J, Kp, nullptr);
  fock_combine_kernel<<<(unsigned)((n2 + 255) / 256), 256, 0, s>>>(J, Kp, nchunk, n2, 0.5, d_G);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return noalloc_fail(msg, msglen, MQ_ECUDA, cudaGetErrorString(e));
  return MQ_OK;
}
