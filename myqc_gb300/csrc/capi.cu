#include <algorithm>
// capi.cu -- the extern "C" entry points of libmyqc (include/myqc.h).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "internal.h"

namespace mq {

int set_err(mq_ctx *c, int code, const std::string &msg) {
  if (c) c->err = msg;
  return code;
}

int cuda_check(mq_ctx *c, cudaError_t e, const char *what) {
  char b[512];
  snprintf(b, sizeof b, "%s: %s", what, cudaGetErrorString(e));
  return set_err(c, e == cudaErrorMemoryAllocation ? MQ_ENOMEM : MQ_ECUDA, b);
}

void *buf(mq_ctx *c, const char *name, size_t bytes) {
  DeviceBuf &b = c->bufs[name];
  if (b.bytes >= bytes && b.ptr) return b.ptr;
  if (b.ptr) {
    cudaStreamSynchronize(c->stream);
    cudaFree(b.ptr);
    b.ptr = nullptr;
    b.bytes = 0;
  }
  void *p = nullptr;
  const size_t want = std::max<size_t>(bytes, 256);
  if (cudaMalloc(&p, want) != cudaSuccess) {
    cudaGetLastError();
    set_err(c, MQ_ENOMEM, std::string("device allocation failed: ") + name);
    return nullptr;
  }
  b.ptr = p;
  b.bytes = want;
  return p;
}

int sync_check(mq_ctx *c, const char *label) {
  static int on = -1;
  if (on < 0) {
    const char *e = getenv("MYQC_SYNC_CHECK");
    on = e && e[0] == '1';
  }
  if (!on) return MQ_OK;
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) {
    char b[512];
    snprintf(b, sizeof b, "stage %s: %s", label, cudaGetErrorString(e));
    return set_err(c, MQ_ECUDA, b);
  }
  return MQ_OK;
}

static int need_system(mq_ctx *c) {
  if (!c) return MQ_EINVAL;
  if (!c->have_system) return set_err(c, MQ_ESTATE, "no system: call mq_set_system first");
  return MQ_OK;
}

// device copy of a host matrix into buffer `name`
static double *to_dev(mq_ctx *c, const char *name, const double *h, size_t count) {
  double *d = (double *)buf(c, name, count * sizeof(double));
  if (!d) return nullptr;
  if (cudaMemcpyAsync(d, h, count * sizeof(double), cudaMemcpyHostToDevice, c->stream) != cudaSuccess) {
    set_err(c, MQ_ECUDA, "host to device copy failed");
    return nullptr;
  }
  return d;
}

int ensure_xx_alloc(mq_ctx *c) {
  const size_t n = c->nao, n4 = n * n * n * n;
  if (c->d_XX && c->XX_elems == n4) return MQ_OK;
  if (c->d_XX) cudaFree(c->d_XX);
  c->d_XX = nullptr;
  c->XX_elems = 0;
  if (cudaMalloc((void **)&c->d_XX, n4 * sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    return set_err(c, MQ_ENOMEM, "cannot allocate the n^4 integral array on the device");
  }
  c->XX_elems = n4;
  return MQ_OK;
}

// The full n^4 array of the current system: already there, or filled from the
// quartet store (on c->stream).
int ensure_xx_full(mq_ctx *c) {
  if (c->xx_valid) return MQ_OK;
  if (!c->qs.valid) return set_err(c, MQ_ESTATE, "no integrals on the device (call mq_eri_store or mq_eri_upload)");
  if (c->nparts > 1) return set_err(c, MQ_EINVAL, "the full integral array needs every quartet: reset the partition first");
  MQ_TRY(ensure_xx_alloc(c));
  MQ_TRY(qstore_expand(c, c->d_XX));
  c->xx_valid = 1;
  return MQ_OK;
}

int ensure_aux(mq_ctx *c) {
  if (!c->aux) {
    int lo = 0, hi = 0;
    MQ_CUDA(c, cudaDeviceGetStreamPriorityRange(&lo, &hi));
    MQ_CUDA(c, cudaStreamCreateWithPriority(&c->aux, cudaStreamNonBlocking, hi));
  }
  if (!c->ev_early) MQ_CUDA(c, cudaEventCreateWithFlags(&c->ev_early, cudaEventDisableTiming));
  return MQ_OK;
}

}  // namespace mq

using namespace mq;

extern "C" {

const char *mq_version(void) { return "myqc-gb300 0.1 sm_103a"; }

int mq_init(mq_ctx **ctx, int device) {
  if (!ctx) return MQ_EINVAL;
  *ctx = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return MQ_ECUDA;
  }
  if (device < 0 || device >= ndev) return MQ_EINVAL;
  if (cudaSetDevice(device) != cudaSuccess) return MQ_ECUDA;
  mq_ctx *c = new mq_ctx();
  c->device = device;
  // priorities (lower is higher): the aux stream's short network passes, then
  // the main stream, then the side stream's overlapping slicing
  int prio_lo = 0, prio_hi = 0;
  cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi);
  const int prio_main = prio_hi < prio_lo ? prio_hi + 1 : prio_hi;
  if (cudaStreamCreateWithPriority(&c->stream, cudaStreamNonBlocking, prio_main) != cudaSuccess) {
    delete c;
    return MQ_ECUDA;
  }
  *ctx = c;
  return MQ_OK;
}

int mq_free(mq_ctx *c) {
  if (!c) return MQ_OK;
  cudaSetDevice(c->device);
  if (c->side) cudaStreamSynchronize(c->side);
  if (c->aux) cudaStreamSynchronize(c->aux);
  cudaStreamSynchronize(c->stream);
  free_pairs(c);
  batch_clear(c);
  mlp_free(c);
  if (c->d_boys_tight) cudaFree(c->d_boys_tight);
  for (auto &kv : c->bufs)
    if (kv.second.ptr) cudaFree(kv.second.ptr);
  if (c->d_XX) cudaFree(c->d_XX);
  if (c->d_boys_f32) cudaFree(c->d_boys_f32);
  if (c->d_boys) cudaFree(c->d_boys);
  if (c->d_nuc) cudaFree(c->d_nuc);
  if (c->pin) cudaFreeHost(c->pin);
  cudaStreamDestroy(c->stream);
  if (c->side) cudaStreamDestroy(c->side);
  if (c->aux) cudaStreamDestroy(c->aux);
  if (c->ev_params) cudaEventDestroy(c->ev_params);
  if (c->ev_early) cudaEventDestroy(c->ev_early);
  if (c->ev_main) cudaEventDestroy(c->ev_main);
  if (c->ev_side) cudaEventDestroy(c->ev_side);
  delete c;
  return MQ_OK;
}

int mq_last_error(const mq_ctx *c, char *out, int len) {
  if (!out || len <= 0) return MQ_EINVAL;
  const char *m = c ? c->err.c_str() : "no context";
  strncpy(out, m, len - 1);
  out[len - 1] = 0;
  return MQ_OK;
}

int mq_set_system(mq_ctx *c, int nnuc, const int *Z, const double *xyz, const double *bas, const double *set,
                  const int *basinfo, const int *setinfo, const double *ftab, int mode) {
  if (!c) return MQ_EINVAL;
  if (mode != MQ_MODE_REFERENCE && mode != MQ_MODE_TIGHT) return set_err(c, MQ_EINVAL, "bad mode");
  if (mode == MQ_MODE_REFERENCE && !ftab) return set_err(c, MQ_EINVAL, "reference mode needs the Ftab table");
  cudaSetDevice(c->device);
  MQ_TRY(join_side(c));  // the side stream may still read the previous system's XX
  c->xx_sliced = 0;
  c->have_system = 0;
  c->mode = mode;
  MQ_TRY(build_shells(c, nnuc, Z, xyz, bas, set, basinfo, setinfo));
  MQ_TRY(build_pairs(c));
  // Boys table (+ its grid values Tk/10, as the reference computes them); the
  // tight table is a constant and stays on the device once uploaded
  if (mode == MQ_MODE_REFERENCE || c->boys_loaded != MQ_MODE_TIGHT) {
    std::vector<double> tab;
    if (mode == MQ_MODE_REFERENCE) {
      tab.assign(ftab, ftab + FTAB_NT * FTAB_NM);
      for (int k = 0; k < FTAB_NT; ++k) tab.push_back(k / 10.0);
    } else {
      tight_boys_device_table(tab);
    }
    c->boys_loaded = -1;
    if (c->d_boys) cudaFree(c->d_boys);
    c->d_boys = nullptr;
    if (c->d_boys_f32) cudaFree(c->d_boys_f32);
    c->d_boys_f32 = nullptr;
    if (mode == MQ_MODE_TIGHT) {  // single-precision copy for the mixed-precision integral pass
      std::vector<float> tf(tab.begin(), tab.end());
      MQ_CUDA(c, cudaMalloc((void **)&c->d_boys_f32, tf.size() * sizeof(float)));
      MQ_CUDA(c, cudaMemcpy(c->d_boys_f32, tf.data(), tf.size() * sizeof(float), cudaMemcpyHostToDevice));
    }
    MQ_CUDA(c, cudaMalloc((void **)&c->d_boys, tab.size() * sizeof(double)));
    MQ_CUDA(c, cudaMemcpy(c->d_boys, tab.data(), tab.size() * sizeof(double), cudaMemcpyHostToDevice));
    c->boys_loaded = mode;
  }
  if (mode != MQ_MODE_TIGHT) c->eri_f32_tau = 0.0;
  std::vector<double> nuc(4 * (size_t)nnuc);
  for (int a = 0; a < nnuc; ++a) {
    for (int k = 0; k < 3; ++k) nuc[4 * a + k] = c->xyz[3 * a + k];
    nuc[4 * a + 3] = Z[a];
  }
  if (nnuc > c->nuc_cap) {
    if (c->d_nuc) cudaFree(c->d_nuc);
    c->d_nuc = nullptr;
    c->nuc_cap = 0;
    MQ_CUDA(c, cudaMalloc((void **)&c->d_nuc, nuc.size() * sizeof(double)));
    c->nuc_cap = nnuc;
  }
  MQ_CUDA(c, cudaMemcpy(c->d_nuc, nuc.data(), nuc.size() * sizeof(double), cudaMemcpyHostToDevice));
  // integrals of a previous system are stale
  c->slab_live_valid = 0;
  c->schwarz_valid = 0;
  c->xx_valid = 0;  // the allocation stays for the next mq_eri_store of the same order
  c->qs.valid = 0;
  c->have_system = 1;
  if (c->schwarz_thr > 0) MQ_TRY(ensure_schwarz(c));
  return MQ_OK;
}

int mq_norb(const mq_ctx *c, int *norb) {
  if (!c || !norb) return MQ_EINVAL;
  if (!c->have_system) return MQ_ESTATE;
  *norb = c->nao;
  return MQ_OK;
}

int mq_set_schwarz(mq_ctx *c, double threshold) {
  if (!c || threshold < 0) return MQ_EINVAL;
  c->schwarz_thr = threshold;
  c->qs.valid = 0;
  c->qs.tables_valid = 0;
  if (c->have_system && threshold > 0) {  // bounds of the current system, recomputed
    c->schwarz_valid = 0;
    return ensure_schwarz(c);
  }
  return MQ_OK;
}

int mq_set_eri_mixed(mq_ctx *c, double tau) {
  if (!c || !(tau >= 0)) return MQ_EINVAL;
  if (tau > 0 && c->have_system && c->mode != MQ_MODE_TIGHT)
    return set_err(c, MQ_EINVAL, "mixed-precision integrals need MQ_MODE_TIGHT (reference mode reproduces the "
                                 "reference's FP64 Boys table)");
  c->eri_f32_tau = tau;
  return MQ_OK;
}

int mq_int1e(mq_ctx *c, double *S, double *H) {
  MQ_TRY(need_system(c));
  if (!S || !H) return set_err(c, MQ_EINVAL, "null output");
  cudaSetDevice(c->device);
  const size_t n2 = (size_t)c->nao * c->nao;
  double *d = (double *)buf(c, "int1e_out", 2 * n2 * sizeof(double));
  if (!d) return MQ_ENOMEM;
  MQ_TRY(int1e_device(c, d, d + n2));
  MQ_CUDA(c, cudaMemcpyAsync(S, d, n2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  MQ_CUDA(c, cudaMemcpyAsync(H, d + n2, n2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  MQ_CUDA(c, cudaStreamSynchronize(c->stream));
  return MQ_OK;
}

int mq_int1p(mq_ctx *c, double *Px) {
  MQ_TRY(need_system(c));
  if (!Px) return set_err(c, MQ_EINVAL, "null output");
  cudaSetDevice(c->device);
  const size_t n2 = (size_t)c->nao * c->nao;
  double *d = (double *)buf(c, "int1p_out", 3 * n2 * sizeof(double));
  if (!d) return MQ_ENOMEM;
  MQ_TRY(int1p_device(c, d));
  MQ_CUDA(c, cudaMemcpyAsync(Px, d, 3 * n2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  MQ_CUDA(c, cudaStreamSynchronize(c->stream));
  return MQ_OK;
}

static int eri_store_full(mq_ctx *c) {
  MQ_TRY(ensure_xx_alloc(c));
  // queued on the context's stream; the call returns without waiting (later
  // calls on the context order after it)
  c->t_eri.collect_sync();
  c->t_eri.total = 0;
  c->t_eri.start(c->stream);
  const int rc = eri_full_device(c, c->d_XX);
  c->t_eri.stop(c->stream);
  c->xx_valid = rc == MQ_OK;
  return rc;
}

int mq_eri_store(mq_ctx *c) {
  MQ_TRY(need_system(c));
  cudaSetDevice(c->device);
  MQ_TRY(join_side(c));
  c->qs.valid = 0;
  c->xx_valid = 0;
  c->xx_sliced = 0;
  c->slab_live_valid = 0;
  if (c->eri_storage != MQ_STORE_QUARTETS) {
    if (c->nparts > 1) return set_err(c, MQ_EINVAL, "a partition of the quartets needs MQ_STORE_QUARTETS");
    return eri_store_full(c);
  }
  if (!(c->schwarz_thr > 0.0))
    return set_err(c, MQ_EINVAL, "MQ_STORE_QUARTETS needs a Schwarz threshold > 0 (mq_set_schwarz)");
  if (c->eri_f32_tau > 0.0) return set_err(c, MQ_EINVAL, "MQ_STORE_QUARTETS stores FP64 integrals only");
  c->t_eri.collect_sync();
  c->t_eri.total = 0;
  c->t_eri.start(c->stream);
  const int rc = qstore_build(c);
  c->t_eri.stop(c->stream);
  return rc;
}

int mq_set_partition(mq_ctx *c, int part, int nparts) {
  if (!c || nparts < 1 || part < 0 || part >= nparts) return MQ_EINVAL;
  c->part = part;
  c->nparts = nparts;
  c->qs.valid = 0;
  c->qs.tables_valid = 0;
  return MQ_OK;
}

int mq_set_eri_storage(mq_ctx *c, int storage) {
  if (!c || (storage != MQ_STORE_FULL && storage != MQ_STORE_QUARTETS)) return MQ_EINVAL;
  c->eri_storage = storage;
  return MQ_OK;
}

int mq_set_eri_tuning(mq_ctx *c, int mode) {
  if (!c || (mode != 0 && mode != 1)) return MQ_EINVAL;
  c->eri_tune_mode = mode;
  return MQ_OK;
}

int mq_eri_tuning_report(const mq_ctx *c, char *out, int len) {
  if (!c || !out || len <= 0) return MQ_EINVAL;
  const std::string r = eri_tune_report(c);
  strncpy(out, r.c_str(), len - 1);
  out[len - 1] = 0;
  return MQ_OK;
}

int mq_eri_full(mq_ctx *c, double *XX) {
  if (!XX) return set_err(c, MQ_EINVAL, "null output");
  MQ_TRY(need_system(c));
  cudaSetDevice(c->device);
  MQ_TRY(join_side(c));
  c->qs.valid = 0;
  c->xx_sliced = 0;
  MQ_TRY(eri_store_full(c));
  MQ_CUDA(c, cudaMemcpyAsync(XX, c->d_XX, c->XX_elems * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  MQ_CUDA(c, cudaStreamSynchronize(c->stream));
  return MQ_OK;
}

int mq_eri_upload(mq_ctx *c, const double *XX) {
  MQ_TRY(need_system(c));
  if (!XX) return set_err(c, MQ_EINVAL, "null input");
  cudaSetDevice(c->device);
  MQ_TRY(join_side(c));
  MQ_TRY(ensure_xx_alloc(c));
  MQ_CUDA(c, cudaMemcpyAsync(c->d_XX, XX, c->XX_elems * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  MQ_CUDA(c, cudaStreamSynchronize(c->stream));
  c->slab_live_valid = 0;  // any slab of the uploaded integrals may be nonzero
  c->xx_sliced = 0;
  c->xx_valid = 1;
  c->qs.valid = 0;
  return MQ_OK;
}

static int fock_common(mq_ctx *c, const double *Da, const double *Db, double *Ga, double *Gb, bool direct) {
  MQ_TRY(need_system(c));
  if (!Da || !Ga || (Db && !Gb)) return set_err(c, MQ_EINVAL, "null matrix");
  cudaSetDevice(c->device);
  const size_t n2 = (size_t)c->nao * c->nao;
  const int ns = Db ? 2 : 1;
  double *dD = to_dev(c, "fock_in", Da, n2 * ns);
  if (!dD) return MQ_ENOMEM;
  if (Db) MQ_CUDA(c, cudaMemcpyAsync(dD + n2, Db, n2 * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  double *dG = (double *)buf(c, "fock_out", n2 * (ns + 3) * sizeof(double));
  if (!dG) return MQ_ENOMEM;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, c->stream);
  c->t_fock_kernel.collect();
  c->t_fock_kernel.total = 0;
  c->stats.fock_kernel_launches = 0;
  int rc;
  if (direct && !Db && !c->fock_df32) {  // RHF: integral blocks recomputed into the store, digested from it
    rc = fock_direct_store_rhf(c, dD, dG);
  } else if (c->nparts > 1 && (Db || c->fock_df32)) {
    rc = set_err(c, MQ_EINVAL, "a partition of the quartets serves RHF FP64 builds only");
  } else if (direct) {
    double *J = dG + n2 * ns, *Ka = J + n2, *Kb = Db ? Ka + n2 : nullptr;
    rc = fock_direct_device(c, dD, Db ? dD + n2 : nullptr, J, Ka, Kb);
    if (rc == MQ_OK) rc = direct_combine(c, J, Ka, Kb, dG, Db ? dG + n2 : nullptr);
  } else {
    rc = fock_stored_device(c, dD, Db ? dD + n2 : nullptr, dG, Db ? dG + n2 : nullptr);
  }
  cudaEventRecord(e1, c->stream);
  cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  c->stats.ms_fock = ms;
  c->t_fock_kernel.collect();
  c->stats.ms_fock_kernel = c->t_fock_kernel.total;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc != MQ_OK) return rc;
  MQ_CUDA(c, cudaMemcpyAsync(Ga, dG, n2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  if (Db) MQ_CUDA(c, cudaMemcpyAsync(Gb, dG + n2, n2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  MQ_CUDA(c, cudaStreamSynchronize(c->stream));
  return MQ_OK;
}

int mq_fock(mq_ctx *c, const double *Da, const double *Db, double *Ga, double *Gb) {
  return fock_common(c, Da, Db, Ga, Gb, false);
}

int mq_fock_direct(mq_ctx *c, const double *Da, const double *Db, double *Ga, double *Gb) {
  return fock_common(c, Da, Db, Ga, Gb, true);
}

int mq_scf(mq_ctx *c, const double *S, const double *H, const mq_scf_opts *o, double *C, double *eps, double *D,
           double *energy, int *iters, double *history) {
  MQ_TRY(need_system(c));
  if (!S || !H || !o || !C || !eps || !energy || !iters) return set_err(c, MQ_EINVAL, "null argument");
  cudaSetDevice(c->device);
  return scf_device(c, S, H, o, C, eps, D, energy, iters, history);
}

int mq_ao2mo_iajb(mq_ctx *c, const double *Ci, int no1, const double *Ca, int nv1, const double *Cj, int no2,
                  const double *Cb, int nv2, int precision, double *out) {
  MQ_TRY(need_system(c));
  if (!Ci || !Ca || !Cj || !Cb || no1 < 0 || nv1 < 0 || no2 < 0 || nv2 < 0)
    return set_err(c, MQ_EINVAL, "bad ao2mo arguments");
  if (precision < MQ_PREC_FP64 || precision > MQ_PREC_SPLIT_BF16X3) return set_err(c, MQ_EINVAL, "bad precision");
  cudaSetDevice(c->device);
  const size_t n = c->nao;
  // pack all four coefficient blocks into one buffer
  double *dCc = (double *)buf(c, "ao2mo_C", n * (size_t)(no1 + nv1 + no2 + nv2) * sizeof(double));
  if (!dCc) return MQ_ENOMEM;
  double *dCi = dCc, *dCa = dCi + n * no1, *dCj = dCa + n * nv1, *dCb = dCj + n * no2;
  MQ_CUDA(c, cudaMemcpyAsync(dCi, Ci, n * no1 * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  MQ_CUDA(c, cudaMemcpyAsync(dCa, Ca, n * nv1 * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  MQ_CUDA(c, cudaMemcpyAsync(dCj, Cj, n * no2 * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  MQ_CUDA(c, cudaMemcpyAsync(dCb, Cb, n * nv2 * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  const size_t cnt = (size_t)no1 * nv1 * no2 * nv2;
  if (c->iajb_elems < cnt) {
    if (c->d_iajb) cudaFree(c->d_iajb);
    c->d_iajb = nullptr;
    c->iajb_elems = 0;
    MQ_CUDA(c, cudaMalloc((void **)&c->d_iajb, std::max<size_t>(cnt, 1) * sizeof(double)));
    c->iajb_elems = cnt;
  }
  c->iajb_dims[0] = no1;
  c->iajb_dims[1] = nv1;
  c->iajb_dims[2] = no2;
  c->iajb_dims[3] = nv2;
  c->iajb_precision = precision;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, c->stream);
  int rc = ao2mo_device(c, dCi, no1, dCa, nv1, dCj, no2, dCb, nv2, precision, c->d_iajb);
  cudaEventRecord(e1, c->stream);
  cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  c->stats.ms_ao2mo = ms;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc != MQ_OK) return rc;
  if (out) {
    MQ_CUDA(c, cudaMemcpyAsync(out, c->d_iajb, cnt * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    MQ_CUDA(c, cudaStreamSynchronize(c->stream));
  }
  return MQ_OK;
}

int mq_mp2_rhf(mq_ctx *c, const double *eig, int nocc, int nvir, double *e_out) {
  MQ_TRY(need_system(c));
  if (!eig || !e_out) return set_err(c, MQ_EINVAL, "null argument");
  if (c->iajb_dims[0] != nocc || c->iajb_dims[1] != nvir || c->iajb_dims[2] != nocc || c->iajb_dims[3] != nvir)
    return set_err(c, MQ_ESTATE, "the device (ia|jb) block does not match nocc/nvir");
  cudaSetDevice(c->device);
  double *de = to_dev(c, "mp2_eig", eig, (size_t)nocc + nvir);
  if (!de) return MQ_ENOMEM;
  return mp2_rhf_device(c, c->d_iajb, de, nocc, nvir, e_out);
}

int mq_mp2_uhf(mq_ctx *c, const double *CA, const double *CB, const double *eA, const double *eB, int noA, int noB,
               int precision, double *e_out) {
  MQ_TRY(need_system(c));
  if (!CA || !CB || !eA || !eB || !e_out) return set_err(c, MQ_EINVAL, "null argument");
  const int n = c->nao, nvA = n - noA, nvB = n - noB;
  if (noA < 0 || noB < 0 || nvA < 0 || nvB < 0) return set_err(c, MQ_EINVAL, "bad occupation");
  double *de = to_dev(c, "mp2_eig", eA, (size_t)2 * n);
  if (!de) return MQ_ENOMEM;
  MQ_CUDA(c, cudaMemcpyAsync(de + n, eB, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  double s[2], out[3];
  // alpha-alpha, beta-beta, alpha-beta blocks as slow_ao2mo_MP2_UHF builds them (ao2mo.f90:614-904)
  const double *Cs[3][2] = {{CA, CA}, {CB, CB}, {CA, CB}};
  const int no[3][2] = {{noA, noA}, {noB, noB}, {noA, noB}};
  for (int blk = 0; blk < 3; ++blk) {
    const double *C1 = Cs[blk][0], *C2 = Cs[blk][1];
    const int o1 = no[blk][0], o2 = no[blk][1], v1 = n - o1, v2 = n - o2;
    MQ_TRY(mq_ao2mo_iajb(c, C1, o1, C1 + (size_t)n * o1, v1, C2, o2, C2 + (size_t)n * o2, v2, precision, nullptr));
    const double *e1 = blk == 1 ? de + n : de, *e2 = blk == 0 ? de : de + n;
    // mp2_pair_sums takes eo = e[0:no], ev = e[no:] for each side
    MQ_TRY(mp2_pair_sums(c, c->d_iajb, o1, v1, o2, v2, e1, e2, blk < 2, s));
    out[blk] = blk < 2 ? s[1] : s[0];
  }
  e_out[0] = out[0];
  e_out[1] = out[1];
  e_out[2] = out[2];
  e_out[3] = out[0] + out[1] + out[2];
  return MQ_OK;
}

int mq_mp2_pairs(mq_ctx *c, const double *iajb, int no1, int nv1, int no2, int nv2, const double *e1,
                 const double *e2, int same_spin, double *e_out) {
  if (!c) return MQ_EINVAL;
  const size_t nel = (size_t)no1 * nv1 * no2 * nv2;
  if ((nel && !iajb) || !e1 || !e2 || !e_out || no1 < 0 || nv1 < 0 || no2 < 0 || nv2 < 0)
    return set_err(c, MQ_EINVAL, "bad mp2 pair arguments");
  if (nel == 0) {  // no occupied or no virtual orbitals on one side: no pairs
    e_out[0] = e_out[1] = 0.0;
    return MQ_OK;
  }
  cudaSetDevice(c->device);
  double *d = to_dev(c, "mp2_pairs_in", iajb, nel);
  if (!d) return MQ_ENOMEM;
  double *de = (double *)buf(c, "mp2_pairs_eig", sizeof(double) * ((size_t)no1 + nv1 + no2 + nv2 + 2));
  if (!de) return MQ_ENOMEM;
  MQ_CUDA(c, cudaMemcpyAsync(de, e1, sizeof(double) * (no1 + nv1), cudaMemcpyHostToDevice, c->stream));
  MQ_CUDA(c, cudaMemcpyAsync(de + no1 + nv1, e2, sizeof(double) * (no2 + nv2), cudaMemcpyHostToDevice, c->stream));
  double s[2] = {0.0, 0.0};
  MQ_TRY(mp2_pair_sums(c, d, no1, nv1, no2, nv2, de, de + no1 + nv1, same_spin, s));
  e_out[0] = s[0];
  e_out[1] = s[1];
  return MQ_OK;
}

int mq_syev_batched(mq_ctx *c, int n, int batch, double *A, double *w, double *V) {
  if (!c || !A || !w || !V || n <= 0 || batch <= 0) return MQ_EINVAL;
  cudaSetDevice(c->device);
  const size_t n2 = (size_t)n * n;
  double *dA = to_dev(c, "syev_A", A, n2 * batch);
  double *dV = (double *)buf(c, "syev_V", (n2 + n) * batch * sizeof(double));
  if (!dA || !dV) return MQ_ENOMEM;
  double *dw = dV + n2 * batch;
  MQ_TRY(syev_batched_device(c, n, batch, dA, dw, dV));
  MQ_CUDA(c, cudaMemcpyAsync(V, dV, n2 * batch * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  MQ_CUDA(c, cudaMemcpyAsync(w, dw, (size_t)n * batch * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  MQ_CUDA(c, cudaStreamSynchronize(c->stream));
  return MQ_OK;
}

int mq_dgemm(mq_ctx *c, char transa, char transb, int m, int n, int k, double alpha, const double *A, int lda,
             const double *B, int ldb, double beta, double *C, int ldc) {
  if (!c || !A || !B || !C || m <= 0 || n <= 0 || k <= 0) return MQ_EINVAL;
  const bool ta = transa == 'T' || transa == 't', tb = transb == 'T' || transb == 't';
  if ((!ta && transa != 'N' && transa != 'n') || (!tb && transb != 'N' && transb != 'n'))
    return set_err(c, MQ_EINVAL, "mq_dgemm: trans must be N or T");
  if (lda < (ta ? k : m) || ldb < (tb ? n : k) || ldc < m) return set_err(c, MQ_EINVAL, "mq_dgemm: leading dimension");
  cudaSetDevice(c->device);
  const size_t na = (size_t)lda * (ta ? m : k), nb = (size_t)ldb * (tb ? k : n), nc = (size_t)ldc * n;
  double *dA = to_dev(c, "dgemm_A", A, na), *dB = to_dev(c, "dgemm_B", B, nb), *dC = to_dev(c, "dgemm_C", C, nc);
  if (!dA || !dB || !dC) return MQ_ENOMEM;
  MQ_TRY(gemm(c, transa, transb, m, n, k, alpha, dA, lda, dB, ldb, beta, dC, ldc));
  MQ_CUDA(c, cudaMemcpyAsync(C, dC, nc * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  MQ_CUDA(c, cudaStreamSynchronize(c->stream));
  return MQ_OK;
}

int mq_sygv(mq_ctx *c, int n, const double *F, const double *S, double *w, double *C) {
  if (!c || !F || !S || !w || !C || n <= 0) return MQ_EINVAL;
  cudaSetDevice(c->device);
  const size_t n2 = (size_t)n * n;
  // S = U s U^T, X = U s^-1/2 U^T, F' = X^T F X = V w V^T, C = X V
  std::vector<double> hs(n), U(n2), X(n2, 0.0), T(n2), Fp(n2, 0.0), V(n2);
  std::vector<double> Sc(S, S + n2);
  MQ_TRY(mq_syev_batched(c, n, 1, Sc.data(), hs.data(), U.data()));
  if (hs[0] <= 0) return set_err(c, MQ_EINVAL, "S not positive definite");
  double *d = (double *)buf(c, "sygv", 4 * n2 * sizeof(double));
  if (!d) return MQ_ENOMEM;
  double *dU = d, *dX = d + n2, *dT = d + 2 * n2, *dF = d + 3 * n2;
  for (size_t i = 0; i < n2; ++i) T[i] = U[i] / std::sqrt(hs[i / n]);
  MQ_CUDA(c, cudaMemcpyAsync(dU, U.data(), n2 * 8, cudaMemcpyHostToDevice, c->stream));
  MQ_CUDA(c, cudaMemcpyAsync(dT, T.data(), n2 * 8, cudaMemcpyHostToDevice, c->stream));
  MQ_TRY(gemm(c, 'N', 'T', n, n, n, 1.0, dT, n, dU, n, 0.0, dX, n));
  MQ_CUDA(c, cudaMemcpyAsync(dF, F, n2 * 8, cudaMemcpyHostToDevice, c->stream));
  MQ_TRY(gemm(c, 'T', 'N', n, n, n, 1.0, dX, n, dF, n, 0.0, dT, n));
  MQ_TRY(gemm(c, 'N', 'N', n, n, n, 1.0, dT, n, dX, n, 0.0, dU, n));
  MQ_CUDA(c, cudaMemcpyAsync(Fp.data(), dU, n2 * 8, cudaMemcpyDeviceToHost, c->stream));
  MQ_CUDA(c, cudaMemcpyAsync(X.data(), dX, n2 * 8, cudaMemcpyDeviceToHost, c->stream));
  MQ_CUDA(c, cudaStreamSynchronize(c->stream));
  MQ_TRY(mq_syev_batched(c, n, 1, Fp.data(), w, V.data()));
  MQ_CUDA(c, cudaMemcpyAsync(dT, V.data(), n2 * 8, cudaMemcpyHostToDevice, c->stream));
  MQ_CUDA(c, cudaMemcpyAsync(dX, X.data(), n2 * 8, cudaMemcpyHostToDevice, c->stream));
  MQ_TRY(gemm(c, 'N', 'N', n, n, n, 1.0, dX, n, dT, n, 0.0, dF, n));
  MQ_CUDA(c, cudaMemcpyAsync(C, dF, n2 * 8, cudaMemcpyDeviceToHost, c->stream));
  MQ_CUDA(c, cudaStreamSynchronize(c->stream));
  return MQ_OK;
}

int mq_set_fock_precision(mq_ctx *c, int precision) {
  if (!c) return MQ_EINVAL;
  if (precision != MQ_FOCK_FP64 && precision != MQ_FOCK_DF32) return set_err(c, MQ_EINVAL, "bad Fock precision");
  c->fock_df32 = precision == MQ_FOCK_DF32;
  return MQ_OK;
}

int mq_set_ao2mo_prefetch(mq_ctx *c, int planes) {
  if (!c) return MQ_EINVAL;
  if (planes != 0 && planes != 2 && planes != 3) return set_err(c, MQ_EINVAL, "prefetch planes must be 0, 2 or 3");
  c->ao2mo_prefetch = planes;
  return MQ_OK;
}

int mq_set_fock_incremental(mq_ctx *c, double tau) {
  if (!c || !(tau >= 0.0) || tau > 1e-2) return c ? set_err(c, MQ_EINVAL, "incremental Fock threshold must be in [0, 1e-2]") : MQ_EINVAL;
  c->fock_inc_tau = tau;
  return MQ_OK;
}

int mq_set_fock_screened_increments(mq_ctx *c, double tau) {
  if (!c) return MQ_EINVAL;
  if (!(tau >= 0.0) || tau > 1e-6) return set_err(c, MQ_EINVAL, "screened-increment threshold must be in [0, 1e-6]");
  c->fock_inc_screen = tau;
  return MQ_OK;
}

int mq_batch_clear(mq_ctx *c) {
  if (!c) return MQ_EINVAL;
  return batch_clear(c);
}

int mq_batch_add(mq_ctx *c, int nnuc, const int *Z, const double *xyz, const double *bas, const double *set,
                 const int *basinfo, const int *setinfo, int nocc) {
  if (!c) return MQ_EINVAL;
  if (nnuc <= 0 || !Z || !xyz || !bas || !set || !basinfo || !setinfo) return set_err(c, MQ_EINVAL, "null argument");
  return batch_add(c, nnuc, Z, xyz, bas, set, basinfo, setinfo, nocc);
}

int mq_batch_info(const mq_ctx *c, int *nmol, int *norb) {
  if (!c || !nmol) return MQ_EINVAL;
  *nmol = (int)c->bmols.size();
  if (norb)
    for (size_t m = 0; m < c->bmols.size(); ++m) norb[m] = c->bmols[m].n;
  return MQ_OK;
}

int mq_batch_scf(mq_ctx *c, const mq_batch_opts *o, double *energy, int *iters, int *converged, double *D,
                 double *eps) {
  if (!c) return MQ_EINVAL;
  if (!o || !energy) return set_err(c, MQ_EINVAL, "null argument");
  cudaSetDevice(c->device);
  return batch_scf(c, o, energy, iters, converged, D, eps);
}

int mq_mlp_init(mq_ctx *c, int nin, int width, int nout) {
  if (!c) return MQ_EINVAL;
  cudaSetDevice(c->device);
  return mlp_init(c, nin, width, nout);
}

int mq_mlp_param_count(mq_ctx *c, int *n) {
  if (!c || !n) return MQ_EINVAL;
  if (!c->mlp) return set_err(c, MQ_ESTATE, "no MLP (mq_mlp_init)");
  *n = mlp_param_count(c);
  return MQ_OK;
}

int mq_mlp_set_params(mq_ctx *c, const float *params) {
  if (!c || !params) return MQ_EINVAL;
  cudaSetDevice(c->device);
  return mlp_set_params(c, params);
}

int mq_mlp_get_params(mq_ctx *c, float *params) {
  if (!c || !params) return MQ_EINVAL;
  cudaSetDevice(c->device);
  return mlp_get_params(c, params);
}

int mq_mlp_forward(mq_ctx *c, int rows, const float *X, float *Y) {
  if (!c || rows < 0 || (rows && (!X || !Y))) return MQ_EINVAL;
  cudaSetDevice(c->device);
  return mlp_forward(c, rows, X, Y);
}

int mq_mlp_grad(mq_ctx *c, int rows, const float *X, const float *T, const float *W, float *grads, double *loss) {
  if (!c || rows <= 0 || !X || !T || !W || !grads || !loss) return MQ_EINVAL;
  cudaSetDevice(c->device);
  return mlp_grad(c, rows, X, T, W, grads, loss);
}

int mq_mlp_set_data(mq_ctx *c, long long n, const float *X, const float *T, const float *W) {
  if (!c || n <= 0 || !X || !T || !W) return MQ_EINVAL;
  cudaSetDevice(c->device);
  return mlp_set_data(c, n, X, T, W);
}

int mq_mlp_train_epoch(mq_ctx *c, const int *perm, int batch, float lr, double *loss) {
  if (!c || !perm || !loss) return MQ_EINVAL;
  cudaSetDevice(c->device);
  return mlp_train_epoch(c, perm, batch, lr, loss);
}

int mq_stat(const mq_ctx *c, const char *key, double *value) {
  if (!c || !key || !value) return MQ_EINVAL;
  const Stats &s = c->stats;
  mq_ctx *mut = const_cast<mq_ctx *>(c);  // lazily collected device timings and counters
  if (!strcmp(key, "eri")) {
    mut->t_eri.collect_sync();
    *value = c->t_eri.total;
  } else if (!strcmp(key, "eri_kernel")) {  // quartet store: the integral kernels alone (0 otherwise)
    mut->t_eri_kernel.collect_sync();
    *value = c->qs.valid ? c->t_eri_kernel.total : 0.0;
  }
  else if (!strcmp(key, "fock")) *value = s.ms_fock;
  else if (!strcmp(key, "diag")) *value = s.ms_diag;
  else if (!strcmp(key, "ao2mo")) *value = s.ms_ao2mo;
  else if (!strcmp(key, "ao2mo_first")) *value = s.ms_ao2mo_first;
  else if (!strcmp(key, "mp2")) *value = s.ms_mp2;
  else if (!strcmp(key, "scf")) *value = s.ms_scf;
  else if (!strcmp(key, "fock_calls")) *value = s.fock_calls;
  else if (!strcmp(key, "scf_iters")) *value = s.scf_iters;
  else if (!strcmp(key, "diag_calls")) *value = s.diag_calls;
  else if (!strcmp(key, "purify_steps")) *value = s.purify_steps;
  else if (!strcmp(key, "purify_persistent")) *value = s.purify_persistent;
  else if (!strcmp(key, "purify_stepwise")) *value = s.purify_stepwise;
  else if (!strcmp(key, "guesses_taken")) *value = s.guesses_taken;
  else if (!strcmp(key, "fock_jc")) *value = s.fock_jc;
  else if (!strcmp(key, "graph_launches")) *value = s.graph_launches;
  else if (!strcmp(key, "eig_cluster")) *value = s.eig_cluster;
  else if (!strcmp(key, "eig_final")) *value = s.ms_eig_final;
  else if (!strcmp(key, "eig_f32_sweeps")) *value = s.eig_f32_sweeps;
  else if (!strcmp(key, "eig_f32_off")) *value = s.eig_f32_off;
  else if (!strcmp(key, "eig_f32")) *value = s.ms_eig_f32;
  else if (!strcmp(key, "eig_refine")) *value = s.ms_eig_refine;
  else if (!strcmp(key, "eig_jacobi")) *value = s.ms_eig_jacobi;
  else if (!strcmp(key, "eig_jacobi_sweeps")) *value = s.eig_jacobi_sweeps;
  else if (!strcmp(key, "fock_precision")) *value = c->fock_df32;
  else if (!strcmp(key, "fock_inc_builds")) *value = s.fock_inc_builds;
  else if (!strcmp(key, "fock_screened_builds")) *value = s.fock_screened_builds;
  else if (!strcmp(key, "fock_full_builds")) *value = s.fock_full_builds;
  else if (!strcmp(key, "fock_full")) *value = s.ms_fock_full;
  else if (!strcmp(key, "eig_early")) *value = s.eig_early;
  else if (!strcmp(key, "fock_kernel")) *value = s.ms_fock_kernel;
  else if (!strcmp(key, "fock_kernel_launches")) *value = s.fock_kernel_launches;
  else if (!strcmp(key, "tune_fock_ms")) *value = s.tune_fock_ms;
  else if (!strcmp(key, "lib_launches")) *value = s.lib_launches;
  else if (!strcmp(key, "launches")) *value = s.launches;
  else if (!strcmp(key, "quartets") || !strcmp(key, "prim_quartets") || !strcmp(key, "quartets_f32") ||
           !strcmp(key, "prim_quartets_f32")) {
    // [0], [1]: all quartets and primitive quartets; [2], [3]: those computed in FP32
    unsigned long long h[4] = {0, 0, 0, 0};
    if (c->d_eri_counters) {
      cudaMemcpyAsync(h, c->d_eri_counters, sizeof(h), cudaMemcpyDeviceToHost, mut->stream);
      cudaStreamSynchronize(mut->stream);
    }
    const bool f32 = strstr(key, "f32") != nullptr, prim = key[0] == 'p';
    *value = (double)(f32 ? h[prim ? 3 : 2] : h[prim ? 1 : 0] + h[prim ? 3 : 2]);
  }
  else if (!strcmp(key, "eri_f32_tau")) *value = c->eri_f32_tau;
  else if (!strcmp(key, "store_unique")) *value = c->qs.valid ? c->qs.unique : 0.0;
  else if (!strcmp(key, "store_quartets")) *value = c->qs.valid ? c->qs.quartets : 0.0;
  else if (!strcmp(key, "store_bytes")) *value = c->qs.valid ? 8.0 * (double)c->qs.X_elems : 0.0;
  else if (!strcmp(key, "live_slabs")) {  // fraction of XX slabs the digestion reads (1: all)
    unsigned long long h = 0;
    if (c->slab_live_valid && c->d_slab_live_count) {
      cudaMemcpyAsync(&h, c->d_slab_live_count, sizeof(h), cudaMemcpyDeviceToHost, mut->stream);
      cudaStreamSynchronize(mut->stream);
      *value = (double)h / ((double)c->nao * c->nao);
    } else {
      *value = 1.0;
    }
  }
  else return MQ_EINVAL;
  return MQ_OK;
}

}  // extern "C"
