// eri_store.cu -- the quartet store's integral pass (qstore.cu builds its
// tables): one launch per class combination over the staircase of surviving
// quartets; the split classes share their per-primitive work across warps.
// Also the launch-order binning of the integral launches and the autotuner
// that picks, per class combination and size, whether to bin, whether the
// warps take their quartets from a persistent work queue, and the CTA size.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <string>

#include "eri_impl.cuh"

namespace mq {

// ---------------------------------------------------------------- binning
// A warp's time in an integral launch is set by its lane with the most
// surviving primitive quartets (quartet() visits exactly the survivors).
// Binning orders a launch's quartets by that count, largest first, so that the
// 32 quartets of a warp have nearly equal counts; the heavy warps also start
// first, which shortens the tail.  A quartet's count is the sum over its bra
// primitive pairs of the ket prefix passing Kab*Kcd >= 1e-14, found by one
// two-pointer walk over the K-descending lists (in FP32: the count only orders
// the launch; the kernels screen in the launch's own arithmetic).  Counting
// sort over BIN_N keys; within one warp's quartets of equal key the order of q
// is kept.
constexpr int BIN_N = 256;
constexpr unsigned char BIN_SKIP = 0xFF;  // quartet that does not decode (screened out): not listed

__device__ __forceinline__ float pp_K(const PairTable &t, int ip) { return __ldg(&t.pf[4 * ip]).z; }

__global__ void bin_cost_kernel(EriArgs g, unsigned char *__restrict__ key, unsigned *__restrict__ hist) {
  __shared__ unsigned h[BIN_N];
  for (int k = threadIdx.x; k < BIN_N; k += blockDim.x) h[k] = 0;
  __syncthreads();
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q < g.nq) {
    long long qd = q;
    int P = 0, Q = 0, m = 0;
    unsigned char k = BIN_SKIP;
    if (decode(g, qd, P, Q, m)) {
      const PairTable &t = g.t;
      const int p0 = t.pp_off[P], p1 = t.pp_off[P + 1], q0 = t.pp_off[Q];
      int len = t.pp_off[Q + 1] - q0, S = 0;
      for (int i = p0; i < p1 && len > 0; ++i) {
        const float Ki = pp_K(t, i);
        while (len > 0 && Ki * pp_K(t, q0 + len - 1) < 1.0e-14f) --len;
        S += len;
      }
      k = (unsigned char)(BIN_N - 2 - min(S, BIN_N - 2));  // largest count first; key < BIN_SKIP
      atomicAdd(&h[k], 1u);
    }
    key[q] = k;
  }
  __syncthreads();
  for (int k = threadIdx.x; k < BIN_N; k += blockDim.x)
    if (h[k]) atomicAdd(&hist[k], h[k]);
}

// exclusive prefix of the key histogram (one CTA of BIN_N threads) and the total
__global__ void __launch_bounds__(BIN_N) bin_scan_kernel(const unsigned *__restrict__ hist,
                                                         unsigned long long *__restrict__ cursor,
                                                         long long *__restrict__ total) {
  __shared__ unsigned long long s[BIN_N];
  const int k = threadIdx.x;
  s[k] = hist[k];
  __syncthreads();
  for (int o = 1; o < BIN_N; o <<= 1) {
    const unsigned long long v = k >= o ? s[k - o] : 0;
    __syncthreads();
    s[k] += v;
    __syncthreads();
  }
  cursor[k] = s[k] - hist[k];
  if (k == BIN_N - 1) *total = (long long)s[k];
}

// each quartet to its key's next slot: one atomic per (warp, key)
__global__ void bin_scatter_kernel(long long nq, const unsigned char *__restrict__ key,
                                   unsigned long long *__restrict__ cursor, long long *__restrict__ list) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned char k = q < nq ? key[q] : BIN_SKIP;
  const unsigned act = __ballot_sync(0xffffffffu, k != BIN_SKIP);
  if (k == BIN_SKIP) return;
  const unsigned peers = __match_any_sync(act, (unsigned)k);
  const int lane = threadIdx.x & 31, leader = __ffs(peers) - 1;
  unsigned long long base = 0;
  if (lane == leader) base = atomicAdd(&cursor[k], (unsigned long long)__popc(peers));
  base = __shfl_sync(peers, base, leader);
  list[base + __popc(peers & ((1u << lane) - 1))] = q;
}

int bin_quartets(mq_ctx *c, EriArgs &h, int slot) {
  const long long nq = h.nq;
  if (nq <= 0) return MQ_OK;
  const std::string name = "eri_bin" + std::to_string(slot);
  const size_t keyb = ((size_t)nq + 255) & ~(size_t)255;
  char *w = (char *)buf(c, name.c_str(), keyb + (size_t)nq * sizeof(long long) + BIN_N * (4 + 8) + 256);
  if (!w) return MQ_ENOMEM;
  unsigned char *key = (unsigned char *)w;
  long long *list = (long long *)(w + keyb);
  unsigned long long *cursor = (unsigned long long *)(list + nq);
  unsigned *hist = (unsigned *)(cursor + BIN_N);
  long long *total = (long long *)(hist + BIN_N);
  EriArgs g = h;
  g.list = nullptr;
  g.list_n = nullptr;
  const unsigned nb = (unsigned)((nq + 255) / 256);
  MQ_CUDA(c, cudaMemsetAsync(hist, 0, BIN_N * sizeof(unsigned), c->stream));
  bin_cost_kernel<<<nb, 256, 0, c->stream>>>(g, key, hist);
  bin_scan_kernel<<<1, BIN_N, 0, c->stream>>>(hist, cursor, total);
  bin_scatter_kernel<<<nb, 256, 0, c->stream>>>(nq, key, cursor, list);
  c->stats.launches += 3;
  MQ_CUDA(c, cudaGetLastError());
  h.list = list;
  h.list_n = total;  // h.nq stays the bound: the grid covers every quartet, idle past *total
  return MQ_OK;
}

// ---------------------------------------------------------------- autotuner
// Launches of fewer quartets are not tuned: they take microseconds, and the
// defaults (binned, 128 threads) serve them.
constexpr long long TUNE_MIN_QUARTETS = 1 << 16;

static unsigned long long tune_key(int epi, int combo, long long nq) {
  int b = 0;
  while ((1LL << (b + 1)) <= nq) ++b;  // floor(log2 nq): launches within a factor 2 share a choice
  return ((unsigned long long)epi << 40) | ((unsigned long long)combo << 32) | (unsigned long long)b;
}

// One class combination's launch with a candidate (binned, block,
// persistent); the binning kernels count towards its time, since every pass
// repeats them.  `slot` names the launch's binning buffers.
template <int EPI>
static int run_candidate(mq_ctx *c, const EriArgs &h0, int cP, int cQ, int slot, const EriTune &t) {
  EriArgs h = h0;
  if (t.binned) MQ_TRY(bin_quartets(c, h, slot));
  return launch_class<EPI>(c, h, cP, cQ, t.block, t.persistent != 0);
}

// The choice for this launch: cached per (epilogue, combination, size class);
// otherwise every candidate runs once (timed with events after one untimed
// run of the default) and the fastest is kept.  Every candidate writes the
// same integrals (each to its own place), so the output is complete whichever
// ran last.
template <int EPI>
static int tuned_launch(mq_ctx *c, const EriArgs &h, int cP, int cQ, int combo, int slot) {
  // the split classes of the quartet store run their CTA-shared kernel: its
  // shape is fixed by the warp count, only the order is a choice
  const bool fixed_shape = EPI == EPI_STORE && nsplit_of(cP, cQ) > 1;
  EriTune def;
  if (c->eri_tune_mode == 0 || h.nq < TUNE_MIN_QUARTETS) return run_candidate<EPI>(c, h, cP, cQ, slot, def);
  const unsigned long long key = tune_key(EPI, combo, h.nq);
  auto it = c->eri_tune.find(key);
  if (it != c->eri_tune.end()) return run_candidate<EPI>(c, h, cP, cQ, slot, it->second);
  std::vector<EriTune> cand;
  for (int binned = 1; binned >= 0; --binned)
    for (int persistent = 0; persistent <= (fixed_shape ? 0 : 1); ++persistent)
      for (int block : {64, 128, 256}) {
        if ((fixed_shape || nsplit_of(cP, cQ) > 1) && block != 128) continue;
        EriTune t;
        t.binned = binned;
        t.block = block;
        t.persistent = persistent;
        cand.push_back(t);
      }
  cudaEvent_t e0, e1;
  MQ_CUDA(c, cudaEventCreate(&e0));
  MQ_CUDA(c, cudaEventCreate(&e1));
  int rc = run_candidate<EPI>(c, h, cP, cQ, slot, def);  // untimed: first-touch of buffers and code
  EriTune best;
  best.ms = 1e30f;
  for (size_t k = 0; rc == MQ_OK && k < cand.size(); ++k) {
    cudaEventRecord(e0, c->stream);
    rc = run_candidate<EPI>(c, h, cP, cQ, slot, cand[k]);
    cudaEventRecord(e1, c->stream);
    if (rc != MQ_OK) break;
    if (cudaEventSynchronize(e1) != cudaSuccess) {
      rc = cuda_check(c, cudaGetLastError(), "eri autotuner");
      break;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cand[k].ms = ms;
    if (ms < best.ms) best = cand[k];
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc != MQ_OK) return rc;
  c->eri_tune[key] = best;
  c->eri_tune_log.push_back({key, cand});
  return MQ_OK;
}

// One tuned pass of a class combination: while its signature is untuned the
// tuning runs (counters off) and then the chosen shape runs once more, so the
// counters count one pass.
template <int EPI>
static int tuned_pass(mq_ctx *c, const EriArgs &h, int cP, int cQ, int combo, int slot) {
  if (c->eri_tune_mode != 0 && h.nq >= TUNE_MIN_QUARTETS && !c->eri_tune.count(tune_key(EPI, combo, h.nq))) {
    EriArgs ht = h;
    ht.counters = nullptr;
    MQ_TRY(tuned_launch<EPI>(c, ht, cP, cQ, combo, slot));
  }
  return tuned_launch<EPI>(c, h, cP, cQ, combo, slot);
}

// The batch's integral pass (eri.cu builds the launches): the autotuned
// shape per class combination.
int eri_batch_launch(mq_ctx *c, const EriArgs &h, int cP, int cQ) {
  const int combo = cP * (cP + 1) / 2 + cQ;
  return tuned_pass<EPI_XX>(c, h, cP, cQ, combo, 16 + combo);
}

// The quartet store's integral blocks: one launch per class combination over
// its staircase of surviving quartets (qstore.cu builds the tables first).
int eri_store_quartets(mq_ctx *c) {
  QStore &qs = c->qs;
  unsigned long long *cnt = (unsigned long long *)buf(c, "eri_counters", 4 * sizeof(unsigned long long));
  if (!cnt) return MQ_ENOMEM;
  MQ_CUDA(c, cudaMemsetAsync(cnt, 0, 4 * sizeof(unsigned long long), c->stream));
  EriArgs g = base_args(c);
  g.counters = cnt;
  for (int k = 0; k < 6; ++k) {
    const QCombo &cb = qs.combo[k];
    if (cb.total == 0) continue;
    EriArgs h = g;
    h.nq = cb.total;
    h.st_off = cb.off;
    h.st_n = cb.nP;
    h.permP = qs.perm + qs.cls_off[cb.cP];
    h.permQ = qs.perm + qs.cls_off[cb.cQ];
    h.store = qs.X + cb.base;
    MQ_TRY(tuned_pass<EPI_STORE>(c, h, cb.cP, cb.cQ, k, k));
  }
  c->d_eri_counters = cnt;
  return MQ_OK;
}

// Text report of the autotuner's choices and timings (one line per launch
// signature: the candidates in the order run, the chosen one marked).
std::string eri_tune_report(const mq_ctx *c) {
  std::string out;
  static const char *const CLS[6] = {"(ss|ss)", "(sps|ss)", "(sps|sps)", "(spsp|ss)", "(spsp|sps)", "(spsp|spsp)"};
  for (const auto &e : c->eri_tune_log) {
    const int combo = (int)((e.first >> 32) & 0xff), b = (int)(e.first & 0xffffffff);
    const int epi = (int)(e.first >> 40);
    const EriTune &ch = c->eri_tune.at(e.first);
    char line[1024];
    int len = std::snprintf(line, sizeof line, "%s %s 2^%d quartets:", epi == EPI_STORE ? "store" : "batch",
                            combo < 6 ? CLS[combo] : "?", b);
    for (const EriTune &t : e.second)
      len += std::snprintf(line + len, sizeof line - len, " %s/%s%d %.3fms%s", t.binned ? "binned" : "plain",
                           t.persistent ? "queue/" : "", t.block, t.ms,
                           (t.binned == ch.binned && t.block == ch.block && t.persistent == ch.persistent) ? "*"
                                                                                                             : "");
    out += line;
    out += "\n";
  }
  return out;
}

}  // namespace mq
