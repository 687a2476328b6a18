// eri.cu -- launches of the integral kernels (eri_impl.cuh): the full XX
// array, the Schwarz bounds, the direct Fock build, batches.  The quartet
// store's pass is in eri_store.cu.
#include <algorithm>
#include <string>
#include <vector>

#include "eri_impl.cuh"

namespace mq {

// Schwarz compaction of one class combination: every quartet index whose bound
// passes goes to `list`.  Each CTA writes its survivors, in index order, to
// its own slot of `part` (blockDim entries) and their number to `counts`; a
// second kernel packs the slots in CTA order, so the list is ascending and the
// same on every run.
__global__ void quartet_screen_kernel(EriArgs g, long long *__restrict__ part, int *__restrict__ counts) {
  __shared__ int warp_cnt[32], warp_off[33];
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long qd = q;
  int P = 0, Q = 0, m = 0;
  EriArgs h = g;
  h.list = nullptr;
  const bool keep = q < g.nq && decode(h, qd, P, Q, m);
  const unsigned bal = __ballot_sync(0xffffffffu, keep);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) warp_cnt[w] = __popc(bal);
  __syncthreads();
  if (threadIdx.x == 0) {
    warp_off[0] = 0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) warp_off[k + 1] = warp_off[k] + warp_cnt[k];
    counts[blockIdx.x] = warp_off[blockDim.x >> 5];
  }
  __syncthreads();
  if (keep) part[(size_t)blockIdx.x * blockDim.x + warp_off[w] + __popc(bal & ((1u << lane) - 1))] = q;
}

// exclusive prefix sum of the CTA counts (one CTA) and the total
__global__ void __launch_bounds__(1024) quartet_scan_kernel(const int *__restrict__ counts, long long nb,
                                                            long long *__restrict__ offs, long long *__restrict__ total) {
  __shared__ long long warp_sum[32];
  __shared__ long long carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (long long base = 0; base < nb; base += blockDim.x) {
    const long long i = base + threadIdx.x;
    long long v = i < nb ? counts[i] : 0, x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const long long y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) warp_sum[w] = x;
    __syncthreads();
    if (w == 0) {
      long long t = lane < (int)(blockDim.x >> 5) ? warp_sum[lane] : 0;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const long long y = __shfl_up_sync(0xffffffffu, t, o);
        if (lane >= o) t += y;
      }
      warp_sum[lane] = t;  // inclusive sums of the warps
    }
    __syncthreads();
    const long long incl = x + (w ? warp_sum[w - 1] : 0) + carry;
    if (i < nb) offs[i] = incl - v;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = incl;
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = carry;
}

__global__ void quartet_pack_kernel(const long long *__restrict__ part, const int *__restrict__ counts,
                                    const long long *__restrict__ offs, int block, long long *__restrict__ list) {
  const int b = blockIdx.x;
  for (int k = threadIdx.x; k < counts[b]; k += blockDim.x) list[offs[b] + k] = part[(size_t)b * block + k];
}

// all unique (bra class >= ket class) combinations
// The surviving quartet indices of launch h (Schwarz screen) into a context
// buffer; h.list / h.nq are set to the compacted list.  Warps of the integral
// kernel then hold only quartets that compute, instead of mostly screened
// lanes that idle while the others loop over their primitives.
static int compact_quartets(mq_ctx *c, EriArgs &h, int slot) {
  const int block = 256;
  const long long nb = (h.nq + block - 1) / block;
  if (nb == 0) return MQ_OK;
  // one buffer per class combination: the lists of all six stay alive until
  // their integral launches have run (nothing here waits for the device)
  const std::string name = "eri_screen" + std::to_string(slot);
  char *w = (char *)buf(c, name.c_str(), (size_t)nb * block * sizeof(long long) + (size_t)nb * (sizeof(int) + sizeof(long long)) +
                                             (size_t)h.nq * sizeof(long long) + 256);
  if (!w) return MQ_ENOMEM;
  long long *part = (long long *)w;
  long long *list = part + (size_t)nb * block;
  long long *offs = list + h.nq;
  long long *total = offs + nb;
  int *counts = (int *)(total + 1);
  quartet_screen_kernel<<<(unsigned)nb, block, 0, c->stream>>>(h, part, counts);
  quartet_scan_kernel<<<1, 1024, 0, c->stream>>>(counts, nb, offs, total);
  quartet_pack_kernel<<<(unsigned)nb, 128, 0, c->stream>>>(part, counts, offs, block, list);
  c->stats.launches += 3;
  MQ_CUDA(c, cudaGetLastError());
  h.list = list;
  h.list_n = total;  // h.nq stays the bound: the grid covers every quartet, idle past *total
  return MQ_OK;
}

template <int EPI>
static int run_all(mq_ctx *c, EriArgs g) {
  const int *off = c->pt.class_off;
  for (int cP = 0; cP < 3; ++cP)
    for (int cQ = 0; cQ <= cP; ++cQ) {
      const int nP = off[cP + 1] - off[cP], nQ = off[cQ + 1] - off[cQ];
      if (nP == 0 || nQ == 0) continue;
      EriArgs h = g;
      h.pOff = off[cP];
      h.nP = nP;
      h.qOff = off[cQ];
      h.nQ = nQ;
      h.tri = cP == cQ;
      h.diag = 0;
      h.nq = h.tri ? (long long)nP * (nP + 1) / 2 : (long long)nP * nQ;
      h.list = nullptr;
      h.list_n = nullptr;
      const int slot = cP * (cP + 1) / 2 + cQ;
      if constexpr (EPI == EPI_XX) {
        if (g.boys_f && c->eri_f32_tau > h.thr) {
          // mixed precision: bounds >= tau in FP64, [thr, tau) in FP32
          EriArgs h64 = h, h32 = h;
          h64.thr = c->eri_f32_tau;
          h64.thr_hi = 0.0;
          MQ_TRY(compact_quartets(c, h64, slot));
          MQ_TRY(launch_class<EPI>(c, h64, cP, cQ));
          h32.thr = std::max(h.thr, 1e-300);
          h32.thr_hi = c->eri_f32_tau;
          h32.counters = h.counters ? h.counters + 2 : nullptr;
          MQ_TRY(compact_quartets(c, h32, slot + 8));
          MQ_TRY((launch_class<EPI, float>(c, h32, cP, cQ)));
          continue;
        }
      }
      if (h.thr > 0.0) MQ_TRY(compact_quartets(c, h, slot));
      MQ_TRY(launch_class<EPI>(c, h, cP, cQ));
    }
  return MQ_OK;
}

int eri_schwarz(mq_ctx *c) {
  EriArgs g = base_args(c);
  g.sch = (unsigned long long *)c->pt.schwarz;
  MQ_CUDA(c, cudaMemsetAsync(c->pt.schwarz, 0, sizeof(double) * std::max(1, c->pt.npairs), c->stream));
  const int *off = c->pt.class_off;
  for (int cl = 0; cl < 3; ++cl) {
    const int np = off[cl + 1] - off[cl];
    if (!np) continue;
    EriArgs h = g;
    h.pOff = h.qOff = off[cl];
    h.nP = h.nQ = np;
    h.diag = 1;
    h.nq = np;
    MQ_TRY(launch_class<EPI_SCHWARZ>(c, h, cl, cl));
  }
  c->schwarz_valid = 1;
  return MQ_OK;
}

// The bounds depend only on the system (geometry, basis, Boys mode): computed
// once per mq_set_system, on the first call that needs them.
int ensure_schwarz(mq_ctx *c) { return c->schwarz_valid ? MQ_OK : eri_schwarz(c); }

// largest Schwarz bound (one CTA)
__global__ void schwarz_max_kernel(const double *__restrict__ sch, int npairs, double *__restrict__ out) {
  __shared__ double red[32];
  double m = 0.0;
  for (int p = threadIdx.x; p < npairs; p += blockDim.x) m = fmax(m, sch[p]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = fmax(m, red[w]);
    out[0] = fmax(m, red[0]);
  }
}

// live[i + n j] for the AO pairs of shell pair P: Q_P * max_Q Q_Q >= thr, the
// condition for some quartet of the slab to pass the integral screen
// (Q_P Q_Q >= thr); counts the live slabs in cnt
__global__ void slab_live_kernel(PairTable t, int n, double thr, const double *__restrict__ qmax,
                                 unsigned char *__restrict__ live, unsigned long long *__restrict__ cnt) {
  const int P = blockIdx.x * blockDim.x + threadIdx.x;
  if (P >= t.npairs) return;
  const int nA = P >= t.class_off[1] ? 4 : 1, nB = P >= t.class_off[2] ? 4 : 1;
  const unsigned char v = t.schwarz[P] * qmax[0] >= thr ? 1 : 0;
  const size_t N = n;
  unsigned long long c = 0;
  for (int a = 0; a < nA; ++a)
    for (int b = 0; b < nB; ++b) {
      const size_t i = t.aoA[P] + a, j = t.aoB[P] + b;
      live[i + N * j] = v;
      live[j + N * i] = v;
      c += v ? (i == j ? 1 : 2) : 0;
    }
  if (c) atomicAdd(cnt, c);
}

int eri_full_device(mq_ctx *c, double *d_XX) {
  const size_t n = (size_t)c->nao;
  MQ_TRY(join_side(c));  // a slicing of the previous XX may still read it
  c->xx_sliced = 0;
  MQ_CUDA(c, cudaMemsetAsync(d_XX, 0, n * n * n * n * sizeof(double), c->stream));
  EriArgs g = base_args(c);
  g.XX = d_XX;
  g.thr = c->schwarz_thr;
  const bool mixed = c->eri_f32_tau > 0.0 && c->mode == MQ_MODE_TIGHT && c->d_boys_f32;
  if (mixed) g.boys_f = c->d_boys_f32;
  if (g.thr > 0 || mixed) MQ_TRY(ensure_schwarz(c));
  unsigned long long *cnt = (unsigned long long *)buf(c, "eri_counters", 4 * sizeof(unsigned long long));
  if (!cnt) return MQ_ENOMEM;
  MQ_CUDA(c, cudaMemsetAsync(cnt, 0, 4 * sizeof(unsigned long long), c->stream));
  g.counters = cnt;
  MQ_TRY(run_all<EPI_XX>(c, g));
  c->d_eri_counters = cnt;  // read when the quartet statistics are asked for
  c->slab_live_valid = 0;
  if (g.thr > 0) {  // zero slabs of XX for the digestion to skip
    const size_t n2 = n * n;
    char *w = (char *)buf(c, "slab_live", n2 + 64);
    if (!w) return MQ_ENOMEM;
    double *qmax = (double *)w;
    unsigned long long *lc = (unsigned long long *)(w + 8);
    MQ_CUDA(c, cudaMemsetAsync(lc, 0, 8, c->stream));
    schwarz_max_kernel<<<1, 1024, 0, c->stream>>>(c->pt.schwarz, c->pt.npairs, qmax);
    slab_live_kernel<<<(c->pt.npairs + 127) / 128, 128, 0, c->stream>>>(c->pt, (int)n, g.thr, qmax,
                                                                        (unsigned char *)(w + 64), lc);
    c->stats.launches += 2;
    MQ_CUDA(c, cudaGetLastError());
    c->d_slab_live = (unsigned char *)(w + 64);
    c->d_slab_live_count = lc;
    c->slab_live_valid = 1;
  }
  return MQ_OK;
}

// Batch: the full XX of every molecule into the packed XX (offset
// MolDesc::xx), one launch per class combination for all molecules.  qcount
// holds, per combination (cP, cQ) with cQ <= cP at index cP*(cP+1)/2 + cQ,
// the device prefix of the molecules' quartet counts and its total.
int eri_batch_device(mq_ctx *c, const PairTable &t, const MolDesc *d_mols, int nmol, const int *d_pstart,
                     const int *d_pcount, const long long *const d_mq_off[6], const long long total[6], double *d_XX,
                     size_t xx_total) {
  MQ_CUDA(c, cudaMemsetAsync(d_XX, 0, xx_total * sizeof(double), c->stream));
  EriArgs g{};
  g.t = t;
  g.boys = c->d_boys;
  g.mode = MQ_MODE_TIGHT;
  g.XX = d_XX;
  g.nmol = nmol;
  g.pstart = d_pstart;
  g.pcount = d_pcount;
  g.mols = d_mols;
  for (int cP = 0; cP < 3; ++cP)
    for (int cQ = 0; cQ <= cP; ++cQ) {
      const int k = cP * (cP + 1) / 2 + cQ;
      if (total[k] == 0) continue;
      EriArgs h = g;
      h.cP = cP;
      h.cQ = cQ;
      h.tri = cP == cQ;
      h.nq = total[k];
      h.mq_off = d_mq_off[k];
      MQ_TRY(eri_batch_launch(c, h, cP, cQ));
    }
  return MQ_OK;
}

int fock_direct_device(mq_ctx *c, const double *d_Da, const double *d_Db, double *d_J, double *d_Ka, double *d_Kb) {
  const size_t n = (size_t)c->nao;
  MQ_CUDA(c, cudaMemsetAsync(d_J, 0, n * n * sizeof(double), c->stream));
  MQ_CUDA(c, cudaMemsetAsync(d_Ka, 0, n * n * sizeof(double), c->stream));
  if (d_Kb) MQ_CUDA(c, cudaMemsetAsync(d_Kb, 0, n * n * sizeof(double), c->stream));
  EriArgs g = base_args(c);
  g.thr = c->schwarz_thr;
  g.Da = d_Da;
  g.Db = d_Db;
  g.J = d_J;
  g.Ka = d_Ka;
  g.Kb = d_Kb;
  g.uhf = d_Db != nullptr;
  return run_all<EPI_FOCK>(c, g);
}

// G = (J + J^T)/2 - f (K + K^T)/2: the direct kernel accumulates each unique
// integral into one of the two mirror elements only
__global__ void direct_combine_kernel(const double *J, const double *K, double f, int n, double *G) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (size_t)n * n) return;
  const size_t r = idx % n, col = idx / n, t = col + (size_t)n * r;
  G[idx] = 0.5 * (J[idx] + J[t]) - f * 0.5 * (K[idx] + K[t]);
}

int direct_combine(mq_ctx *c, const double *J, const double *Ka, const double *Kb, double *Ga, double *Gb) {
  const int n = c->nao;
  const unsigned grid = (unsigned)(((size_t)n * n + 255) / 256);
  direct_combine_kernel<<<grid, 256, 0, c->stream>>>(J, Ka, Kb ? 1.0 : 0.5, n, Ga);
  if (Kb) direct_combine_kernel<<<grid, 256, 0, c->stream>>>(J, Kb, 1.0, n, Gb);
  c->stats.launches += Kb ? 2 : 1;
  MQ_CUDA(c, cudaGetLastError());
  return MQ_OK;
}

}  // namespace mq
