// eri_store.cu -- the quartet store's integral pass (qstore.cu builds its
// tables): one launch per class combination over the staircase of surviving
// quartets; the split classes share their per-primitive work across warps.
#include "eri_impl.cuh"

namespace mq {

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
    MQ_TRY(launch_class<EPI_STORE>(c, h, cb.cP, cb.cQ));
  }
  c->d_eri_counters = cnt;
  return MQ_OK;
}

}  // namespace mq
