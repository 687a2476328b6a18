// batch.cu -- many independent closed-shell RHF problems solved together.
//
// The reference solves one molecule per run (src/scf/scf.f90:61-216 with
// dens, RHFI2G and DSYGV per iteration).  Here a batch of molecules of uneven
// size shares every launch:
//   - one pair table for all molecules (class-major, then molecule), so the
//     integral kernels run one launch per shell-pair class / class combination
//     over all molecules (int1e.cu, eri.cu; each work item finds its molecule
//     by its pair's tag or a binary search over quartet-count prefixes);
//   - one pair-slab Fock launch over the tiles (i, j-run, molecule) of all
//     molecules (fock.cu);
//   - per-molecule kernels, one CTA per molecule, for everything dense:
//     S^-1/2, F = H + G and the energy, DIIS (commutator errors, B matrix,
//     the small linear solve, extrapolation), and the density step
//     (X F X, Jacobi in shared memory, aufbau occupation, D, convergence).
// Molecules converge independently: a converged molecule's flag turns its
// tiles and CTAs into no-ops while the others iterate.  One iteration is a
// fixed sequence of launches with all state on the device, so it is captured
// once in a CUDA graph and replayed; the host only polls the count of active
// molecules every few iterations.
//
// Semantics per molecule are those of scf_device: iteration k uses D_k, stops
// when k > 0 and max|D_{k+1} - D_k| (or the RMS) is below the threshold,
// reports E_k and keeps D_k.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "internal.h"
#include "jacobi.cuh"

namespace mq {

constexpr int BT = 256;  // threads of the per-molecule kernels
constexpr int BATCH_MAX_N = 116;  // 2 n^2 doubles of shared memory per CTA

__device__ __forceinline__ double bsum(double v, double *red) { return jac_block_sum(v, red); }

__device__ __forceinline__ double bmax(double v, double *red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t = fmax(t, red[w]);
  return t;
}

// C = A B for n x n column-major matrices (any of them shared or global)
__device__ __forceinline__ void cta_matmul(int n, const double *A, const double *B, double *C) {
  const size_t n2 = (size_t)n * n;
  for (size_t idx = threadIdx.x; idx < n2; idx += blockDim.x) {
    const int i = (int)(idx % n), j = (int)(idx / n);
    double s = 0.0;
    for (int k = 0; k < n; ++k) s += A[i + (size_t)n * k] * B[k + (size_t)n * j];
    C[idx] = s;
  }
}

// X = S^-1/2 = U s^-1/2 U^T per molecule; status bit 1 if S is not positive definite
__global__ void __launch_bounds__(BT) batch_orth_kernel(const MolDesc *__restrict__ mols,
                                                        const double *__restrict__ S, double *__restrict__ X,
                                                        int *__restrict__ status) {
  extern __shared__ double sm[];
  __shared__ double red[BT / 32];
  __shared__ int flag;
  const MolDesc md = mols[blockIdx.x];
  const int n = md.n;
  const size_t n2 = (size_t)n * n;
  double *A = sm, *V = sm + n2, *cs = V + n2;
  for (size_t idx = threadIdx.x; idx < n2; idx += blockDim.x) A[idx] = S[md.mat + idx];
  __syncthreads();
  const bool ok = jacobi_block(n, A, V, cs, red, &flag, 60, 1e-14);
  // s^-1/2 on the diagonal of A
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double s = A[i + (size_t)n * i];
    if (!(s > 0.0)) atomicOr(status + blockIdx.x, 1);
    cs[i] = s > 0.0 ? rsqrt(s) : 0.0;
  }
  __syncthreads();
  if (threadIdx.x == 0 && !ok) atomicOr(status + blockIdx.x, 2);
  for (size_t idx = threadIdx.x; idx < n2; idx += blockDim.x) {
    const int k = (int)(idx % n), l = (int)(idx / n);
    double x = 0.0;
    for (int i = 0; i < n; ++i) x += V[k + (size_t)n * i] * cs[i] * V[l + (size_t)n * i];
    X[md.mat + idx] = x;
  }
}

// F = H + G and E_k = 1/2 sum D (F + H) + E_nuc (getEnr, scf.f90:1122-1152;
// RHFiter's energy :775-781) for the active molecules
__global__ void __launch_bounds__(BT) batch_energy_kernel(const MolDesc *__restrict__ mols,
                                                          const int *__restrict__ active,
                                                          const double *__restrict__ H, const double *__restrict__ G,
                                                          const double *__restrict__ D, const double *__restrict__ enuc,
                                                          double *__restrict__ F, double *__restrict__ Ek) {
  __shared__ double red[BT / 32];
  const int m = blockIdx.x;
  if (!active[m]) return;
  const MolDesc md = mols[m];
  const size_t n2 = (size_t)md.n * md.n;
  double e = 0.0;
  for (size_t idx = threadIdx.x; idx < n2; idx += blockDim.x) {
    const size_t o = md.mat + idx;
    const double f = H[o] + G[o];
    F[o] = f;
    e += D[o] * (f + H[o]);
  }
  e = bsum(e, red);
  if (threadIdx.x == 0) Ek[m] = 0.5 * e + enuc[m];
}

// DIIS for the active molecules: e = F D S - S D F stored with F in ring slot
// head, a new row of B, the bordered system of the slots in use (scaled by the
// largest diagonal, partial pivoting, one thread), Fx = sum c_j F_j.
constexpr int DIIS_MAX = 16;
__global__ void __launch_bounds__(BT) batch_diis_kernel(const MolDesc *__restrict__ mols,
                                                        const int *__restrict__ active, const double *__restrict__ F,
                                                        const double *__restrict__ D, const double *__restrict__ S,
                                                        double *__restrict__ Fh, double *__restrict__ Eh,
                                                        double *__restrict__ Bm, int2 *__restrict__ state, int ndiis,
                                                        size_t mat_total, double *__restrict__ Fx) {
  extern __shared__ double sm[];
  __shared__ double red[BT / 32];
  __shared__ double cvec[DIIS_MAX];
  __shared__ double sys[(DIIS_MAX + 1) * (DIIS_MAX + 2)];
  const int m = blockIdx.x;
  if (!active[m]) return;
  const MolDesc md = mols[m];
  const int n = md.n;
  const size_t n2 = (size_t)n * n;
  double *T = sm, *U = sm + n2;
  const int2 st = state[m];
  const int h = st.x, nh = min(st.y + 1, ndiis);
  cta_matmul(n, F + md.mat, D + md.mat, T);
  __syncthreads();
  cta_matmul(n, T, S + md.mat, U);
  __syncthreads();
  double *Fs = Fh + mat_total * h + md.mat, *Es = Eh + mat_total * h + md.mat;
  for (size_t idx = threadIdx.x; idx < n2; idx += blockDim.x) {
    const size_t t = (idx % n) * n + idx / n;
    Fs[idx] = F[md.mat + idx];
    Es[idx] = U[idx] - U[t];
  }
  __syncthreads();
  double *B = Bm + (size_t)m * ndiis * ndiis;
  for (int j = 0; j < nh; ++j) {
    const double *Ej = Eh + mat_total * j + md.mat;
    double d = 0.0;
    for (size_t idx = threadIdx.x; idx < n2; idx += blockDim.x) d += Es[idx] * Ej[idx];
    d = bsum(d, red);
    if (threadIdx.x == 0) B[h * ndiis + j] = B[j * ndiis + h] = d;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    bool ok = nh >= 2;
    const int N = nh + 1, W = N + 1;  // augmented rows [A | b]
    if (ok) {
      double scale = 0.0;
      for (int i = 0; i < nh; ++i) scale = fmax(scale, fabs(B[i * ndiis + i]));
      ok = scale > 0.0;
      for (int i = 0; i < N && ok; ++i)
        for (int j = 0; j < W; ++j) {
          double v;
          if (j == N) v = (i == nh) ? -1.0 : 0.0;
          else if (i < nh && j < nh) v = B[i * ndiis + j] / scale;
          else if (i == nh && j == nh) v = 0.0;
          else v = -1.0;
          sys[i * W + j] = v;
        }
      for (int k = 0; k < N && ok; ++k) {
        int piv = k;
        for (int i = k + 1; i < N; ++i)
          if (fabs(sys[i * W + k]) > fabs(sys[piv * W + k])) piv = i;
        if (fabs(sys[piv * W + k]) < 1e-300) {
          ok = false;
          break;
        }
        if (piv != k)
          for (int j = 0; j < W; ++j) {
            const double t = sys[k * W + j];
            sys[k * W + j] = sys[piv * W + j];
            sys[piv * W + j] = t;
          }
        for (int i = k + 1; i < N; ++i) {
          const double f = sys[i * W + k] / sys[k * W + k];
          for (int j = k; j < W; ++j) sys[i * W + j] -= f * sys[k * W + j];
        }
      }
      if (ok)
        for (int i = N - 1; i >= 0; --i) {
          double s = sys[i * W + N];
          for (int j = i + 1; j < N; ++j) s -= sys[i * W + j] * sys[j * W + N];
          sys[i * W + N] = s / sys[i * W + i];
        }
    }
    for (int j = 0; j < ndiis && j < DIIS_MAX; ++j) cvec[j] = ok ? (j < nh ? sys[j * W + N] : 0.0) : (j == h);
    state[m] = make_int2((h + 1) % ndiis, nh);
  }
  __syncthreads();
  for (size_t idx = threadIdx.x; idx < n2; idx += blockDim.x) {
    double v = 0.0;
    for (int j = 0; j < nh; ++j) v += cvec[j] * Fh[mat_total * j + md.mat + idx];
    Fx[md.mat + idx] = v;
  }
}

// Density step per molecule: F' = X Fx X, Jacobi, eigenvalues ascending (eps),
// C_occ = X V_occ, D_new = 2 C_occ C_occ^T (dens.f90:115-124), then
//   guess mode: D <- D_new;
//   iteration mode: it += 1; converged when it > 0 and the max (or RMS) of
//   D_new - D is below thr (checkConv, scf.f90:1227-1258): the molecule
//   leaves the active set, keeps D_k and reports E_k; otherwise D <- D_new,
//   and a molecule at max_iter leaves unconverged.
__global__ void __launch_bounds__(BT) batch_density_kernel(
    int guess, const MolDesc *__restrict__ mols, int *__restrict__ active, const double *__restrict__ X,
    const double *__restrict__ Fx, double *__restrict__ D, double *__restrict__ Dn, double *__restrict__ eps,
    int *__restrict__ iters, int *__restrict__ conv, const double *__restrict__ Ek, double *__restrict__ Efin,
    double thr, int conv_rms, int max_iter, int *__restrict__ status) {
  extern __shared__ double sm[];
  __shared__ double red[BT / 32];
  __shared__ int flag, decision;
  const int m = blockIdx.x;
  if (!guess && !active[m]) return;
  const MolDesc md = mols[m];
  const int n = md.n, nocc = md.nocc;
  const size_t n2 = (size_t)n * n;
  double *A = sm, *V = sm + n2, *cs = V + n2;
  int *perm = (int *)(cs + n + 2);
  const double *Xm = X + md.mat;
  cta_matmul(n, Fx + md.mat, Xm, V);  // T = Fx X
  __syncthreads();
  cta_matmul(n, Xm, V, A);  // X T (X symmetric)
  __syncthreads();
  const bool ok = jacobi_block(n, A, V, cs, red, &flag, 60, 1e-14);
  if (threadIdx.x == 0 && !ok) atomicOr(status + m, 2);
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const int r = jacobi_rank(n, A, i);
    perm[r] = i;
    eps[md.vec + r] = A[i + (size_t)n * i];
  }
  __syncthreads();
  // C_occ (n x nocc) into A
  for (size_t idx = threadIdx.x; idx < (size_t)n * nocc; idx += blockDim.x) {
    const int k = (int)(idx % n), r = (int)(idx / n);
    const double *v = V + (size_t)n * perm[r];
    double s = 0.0;
    for (int l = 0; l < n; ++l) s += Xm[k + (size_t)n * l] * v[l];
    A[idx] = s;
  }
  __syncthreads();
  double dmax = 0.0, dss = 0.0;
  for (size_t idx = threadIdx.x; idx < n2; idx += blockDim.x) {
    const int k = (int)(idx % n), l = (int)(idx / n);
    double s = 0.0;
    for (int r = 0; r < nocc; ++r) s += A[k + (size_t)n * r] * A[l + (size_t)n * r];
    s *= 2.0;
    const double d = s - D[md.mat + idx];
    dmax = fmax(dmax, fabs(d));
    dss += d * d;
    Dn[md.mat + idx] = s;
  }
  dmax = bmax(dmax, red);
  dss = bsum(dss, red);
  if (threadIdx.x == 0) {
    int keep_new = 1;
    if (!guess) {
      const int it = iters[m];
      const double diff = conv_rms ? sqrt(dss / (double)n2) : dmax;
      const bool cv = it > 0 && diff < thr;
      iters[m] = it + 1;
      if (cv || it + 1 >= max_iter) {
        active[m] = 0;
        conv[m] = cv ? 1 : 0;
        Efin[m] = Ek[m];
        keep_new = cv ? 0 : 1;
      }
    }
    decision = keep_new;
  }
  __syncthreads();
  if (decision)
    for (size_t idx = threadIdx.x; idx < n2; idx += blockDim.x) D[md.mat + idx] = Dn[md.mat + idx];
}

// D <- the caller's guess for molecules whose block does not start with NaN
// and that passes the guess checks (else the core guess stays): electron
// count |tr(D S) - 2 nocc| < 0.5 and idempotency ||D S D / 2 - D||_F / ||D||_F
// < 0.25 (the checks the learned guess must pass), in FP64, T = D S in
// shared memory (n^2 doubles).  used[m] = 1 when the guess was taken.
__global__ void batch_guess_kernel(const MolDesc *__restrict__ mols, const double *__restrict__ Dg,
                                   const double *__restrict__ S, double *__restrict__ D, int *__restrict__ used) {
  extern __shared__ double T[];
  __shared__ double red[32];
  const MolDesc md = mols[blockIdx.x];
  const int n = md.n;
  const size_t n2 = (size_t)n * n;
  if (isnan(Dg[md.mat])) {
    if (threadIdx.x == 0) used[blockIdx.x] = 0;
    return;
  }
  const double *G = Dg + md.mat, *Sm = S + md.mat;
  for (size_t idx = threadIdx.x; idx < n2; idx += blockDim.x) {  // T = G S (column-major)
    const int i = (int)(idx % n), j = (int)(idx / n);
    double v = 0.0;
    for (int k = 0; k < n; ++k) v = fma(G[i + (size_t)n * k], Sm[k + (size_t)n * j], v);
    T[idx] = v;
  }
  __syncthreads();
  double tr = 0.0, e2 = 0.0, g2 = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) tr += T[i + (size_t)n * i];
  for (size_t idx = threadIdx.x; idx < n2; idx += blockDim.x) {  // E = T G / 2 - G
    const int i = (int)(idx % n), j = (int)(idx / n);
    double v = 0.0;
    for (int k = 0; k < n; ++k) v = fma(T[i + (size_t)n * k], G[k + (size_t)n * j], v);
    const double e = 0.5 * v - G[idx];
    e2 = fma(e, e, e2);
    g2 = fma(G[idx], G[idx], g2);
  }
  tr = bsum(tr, red);
  e2 = bsum(e2, red);
  g2 = bsum(g2, red);
  __shared__ int ok;
  if (threadIdx.x == 0) {
    ok = isfinite(tr) && fabs(tr - 2.0 * md.nocc) < 0.5 && sqrt(e2) < 0.25 * fmax(sqrt(g2), 1e-30);
    used[blockIdx.x] = ok;
  }
  __syncthreads();
  if (!ok) return;
  for (size_t idx = threadIdx.x; idx < n2; idx += blockDim.x) D[md.mat + idx] = G[idx];
}

__global__ void batch_count_kernel(const int *__restrict__ active, int nmol, int *__restrict__ out) {
  __shared__ int s;
  if (threadIdx.x == 0) s = 0;
  __syncthreads();
  int k = 0;
  for (int m = threadIdx.x; m < nmol; m += blockDim.x) k += active[m] != 0;
  atomicAdd(&s, k);
  __syncthreads();
  if (threadIdx.x == 0) *out = s;
}

// -------------------------------------------------------------------- host

static double nuc_rep(const std::vector<double> &nuc) {
  const size_t na = nuc.size() / 4;
  double E = 0.0;
  for (size_t a = 0; a < na; ++a)
    for (size_t b = 0; b < a; ++b) {
      double r2 = 0.0;
      for (int k = 0; k < 3; ++k) r2 += (nuc[4 * a + k] - nuc[4 * b + k]) * (nuc[4 * a + k] - nuc[4 * b + k]);
      E += nuc[4 * a + 3] * nuc[4 * b + 3] / std::sqrt(r2);
    }
  return E;
}

static void free_batch_pairs(mq_ctx *c) {
  for (void *p : c->batch_allocs) cudaFree(p);
  c->batch_allocs.clear();
}

int batch_clear(mq_ctx *c) {
  c->bmols.clear();
  free_batch_pairs(c);
  return MQ_OK;
}

int batch_add(mq_ctx *c, int nnuc, const int *Z, const double *xyz, const double *bas, const double *set,
              const int *basinfo, const int *setinfo, int nocc) {
  mq_ctx tmp;  // host-side shell construction only: no device state is touched
  tmp.mode = MQ_MODE_TIGHT;
  if (build_shells(&tmp, nnuc, Z, xyz, bas, set, basinfo, setinfo) != MQ_OK)
    return set_err(c, MQ_EINVAL, "batch molecule: " + tmp.err);
  if (tmp.nao > BATCH_MAX_N) return set_err(c, MQ_EINVAL, "batch molecule larger than 116 basis functions");
  if (nocc < 0 || nocc > tmp.nao) return set_err(c, MQ_EINVAL, "batch molecule: bad occupation");
  BatchMol bm;
  bm.n = tmp.nao;
  bm.nocc = nocc;
  bm.nnuc = nnuc;
  pairs_host(tmp.shells, tmp.xyz, bm.pairs);
  bm.nuc.resize(4 * (size_t)nnuc);
  for (int a = 0; a < nnuc; ++a) {
    for (int k = 0; k < 3; ++k) bm.nuc[4 * a + k] = tmp.xyz[3 * a + k];
    bm.nuc[4 * a + 3] = Z[a];
  }
  bm.enuc = nuc_rep(bm.nuc);
  c->bmols.push_back(std::move(bm));
  return MQ_OK;
}

template <class T>
static T *upload_vec(mq_ctx *c, const char *name, const std::vector<T> &v) {
  T *d = (T *)buf(c, name, std::max<size_t>(1, v.size()) * sizeof(T));
  if (!d) return nullptr;
  if (!v.empty() && cudaMemcpyAsync(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, c->stream) != cudaSuccess) {
    set_err(c, MQ_ECUDA, "batch upload");
    return nullptr;
  }
  return d;
}

int batch_scf(mq_ctx *c, const mq_batch_opts *o, double *energy, int *iters, int *converged, double *D_out,
              double *eps_out) {
  const int M = (int)c->bmols.size();
  if (M == 0) return set_err(c, MQ_ESTATE, "empty batch");
  if (M > 65535) return set_err(c, MQ_EINVAL, "batch larger than 65535 molecules");
  const int max_iter = o->max_iter > 0 ? o->max_iter : 500;
  const double thr = o->conv > 0 ? o->conv : 1e-7;
  const int ndiis = std::min(std::max(o->diis, 0), DIIS_MAX);
  const int poll = o->check_every > 0 ? o->check_every : 4;
  auto &mols = c->bmols;
  // ---- packed layout
  std::vector<MolDesc> md(M);
  size_t xx = 0, mat = 0, vec = 0, q = 0;
  int nuc_off = 0, nmax = 0;
  for (int m = 0; m < M; ++m) {
    const size_t n = mols[m].n;
    md[m] = MolDesc{};
    md[m].n = (int)n;
    md[m].nocc = mols[m].nocc;
    md[m].nnuc = mols[m].nnuc;
    md[m].nuc_off = nuc_off;
    md[m].xx = (long long)xx;
    md[m].mat = (long long)mat;
    md[m].vec = (long long)vec;
    md[m].q = (long long)q;
    xx += n * n * n * n;
    mat += n * n;
    vec += n;
    q += n * n * n;
    nuc_off += mols[m].nnuc;
    nmax = std::max(nmax, (int)n);
  }
  // ---- batch pair table (class-major, then molecule)
  HostPairs bh;
  std::vector<int> pstart(3 * (size_t)M), pcount(3 * (size_t)M);
  for (int cl = 0; cl < 3; ++cl) {
    bh.class_off[cl] = (int)bh.shA.size();
    for (int m = 0; m < M; ++m) {
      pstart[3 * m + cl] = (int)bh.shA.size();
      append_pairs_class(bh, mols[m].pairs, cl, m);
      pcount[3 * m + cl] = (int)bh.shA.size() - pstart[3 * m + cl];
    }
  }
  bh.class_off[3] = (int)bh.shA.size();
  if (bh.off.empty()) bh.off.push_back(0);
  // quartet-count prefixes per class combination
  std::vector<long long> mqo[6];
  long long total[6];
  for (int cP = 0; cP < 3; ++cP)
    for (int cQ = 0; cQ <= cP; ++cQ) {
      const int k = cP * (cP + 1) / 2 + cQ;
      mqo[k].assign(M + 1, 0);
      for (int m = 0; m < M; ++m) {
        const long long nP = pcount[3 * m + cP], nQ = pcount[3 * m + cQ];
        mqo[k][m + 1] = mqo[k][m] + (cP == cQ ? nP * (nP + 1) / 2 : nP * nQ);
      }
      total[k] = mqo[k][M];
    }
  // Fock tiles (i, j-run of 2, molecule) and per-molecule row tables
  const int JC = 2;
  std::vector<int4> tl;
  std::vector<int> rf;
  for (int m = 0; m < M; ++m) {
    md[m].row_first = (int)rf.size();
    pair_tiles_host(md[m].n, JC, m, tl, rf);
  }
  std::vector<double> nuc, en(M);
  for (int m = 0; m < M; ++m) {
    nuc.insert(nuc.end(), mols[m].nuc.begin(), mols[m].nuc.end());
    en[m] = mols[m].enuc;
  }
  // ---- device data
  cudaSetDevice(c->device);
  if (!c->d_boys_tight) {
    std::vector<double> tab;
    tight_boys_device_table(tab);
    MQ_CUDA(c, cudaMalloc((void **)&c->d_boys_tight, tab.size() * sizeof(double)));
    MQ_CUDA(c, cudaMemcpy(c->d_boys_tight, tab.data(), tab.size() * sizeof(double), cudaMemcpyHostToDevice));
  }
  free_batch_pairs(c);
  PairTable bpt;
  MQ_TRY(upload_pairs(c, bh, &c->batch_allocs, bpt));
  MolDesc *d_md = upload_vec(c, "batch_mols", md);
  double *d_nuc = upload_vec(c, "batch_nuc", nuc);
  double *d_en = upload_vec(c, "batch_enuc", en);
  int *d_pstart = upload_vec(c, "batch_pstart", pstart);
  int *d_pcount = upload_vec(c, "batch_pcount", pcount);
  int4 *d_tiles = upload_vec(c, "batch_tiles", tl);
  int *d_rf = upload_vec(c, "batch_rowfirst", rf);
  const long long *d_mqo[6];
  for (int k = 0; k < 6; ++k) {
    const std::string name = "batch_mqoff" + std::to_string(k);
    d_mqo[k] = upload_vec(c, name.c_str(), mqo[k]);
    if (!d_mqo[k]) return MQ_ENOMEM;
  }
  if (!d_md || !d_nuc || !d_en || !d_pstart || !d_pcount || !d_tiles || !d_rf) return MQ_ENOMEM;
  const int nd = std::max(ndiis, 1);
  double *d_XX = (double *)buf(c, "batch_XX", xx * sizeof(double) + 64);
  // matrices: S H X D Dn F G Fx J K | DIIS F ring | DIIS error ring
  double *d_mats = (double *)buf(c, "batch_mats", mat * sizeof(double) * (10 + 2 * (size_t)nd));
  double *d_vecs = (double *)buf(c, "batch_vecs", (vec + 2 * (size_t)M) * sizeof(double));
  double *d_B = (double *)buf(c, "batch_B", (size_t)M * nd * nd * sizeof(double));
  int *d_ints = (int *)buf(c, "batch_ints", (size_t)M * 8 * sizeof(int) + 64);
  float2 *d_DJ = (float2 *)buf(c, "batch_dsplit", mat * sizeof(float2));
  double *d_Kp = (double *)buf(c, "batch_kslices", tl.size() * (size_t)nmax * sizeof(double));
  double *d_Q = (double *)buf(c, "batch_Q", std::max<size_t>(q, 1) * sizeof(double));
  if (!d_XX || !d_mats || !d_vecs || !d_B || !d_ints || !d_DJ || !d_Kp || !d_Q) return MQ_ENOMEM;
  double *dS = d_mats, *dH = dS + mat, *dX = dH + mat, *dD = dX + mat, *dDn = dD + mat, *dF = dDn + mat,
         *dG = dF + mat, *dFx = dG + mat, *dJ = dFx + mat, *dK = dJ + mat, *dFh = dK + mat,
         *dEh = dFh + mat * (size_t)nd;
  double *d_eps = d_vecs, *d_Ek = d_vecs + vec, *d_Ef = d_Ek + M;
  int *d_active = d_ints, *d_it = d_ints + M, *d_conv = d_ints + 2 * M, *d_status = d_ints + 3 * M;
  int2 *d_state = (int2 *)(d_ints + 4 * M);
  int *d_count = d_ints + 6 * M;
  MQ_CUDA(c, cudaMemsetAsync(d_ints, 0, (size_t)M * 8 * sizeof(int), c->stream));
  MQ_CUDA(c, cudaMemsetAsync(d_B, 0, (size_t)M * nd * nd * sizeof(double), c->stream));
  {
    std::vector<int> ones(M, 1);
    MQ_CUDA(c, cudaMemcpyAsync(d_active, ones.data(), M * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    MQ_CUDA(c, cudaStreamSynchronize(c->stream));
  }
  // ---- integrals
  double *saved_boys = c->d_boys;
  c->d_boys = c->d_boys_tight;
  int rc = int1e_batch_device(c, bpt, d_nuc, d_md, mat, dS, dH);
  if (rc == MQ_OK) rc = eri_batch_device(c, bpt, d_md, M, d_pstart, d_pcount, d_mqo, total, d_XX, xx);
  c->d_boys = saved_boys;
  MQ_TRY(rc);
  // ---- S^-1/2 and the core-Hamiltonian guess
  const size_t smem = (2 * (size_t)nmax * nmax + nmax + 2) * sizeof(double) + nmax * sizeof(int) + 16;
  const size_t smem_diis = 2 * (size_t)nmax * nmax * sizeof(double);
  MQ_CUDA(c, cudaFuncSetAttribute(batch_orth_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  MQ_CUDA(c, cudaFuncSetAttribute(batch_density_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  MQ_CUDA(c, cudaFuncSetAttribute(batch_diis_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_diis));
  batch_orth_kernel<<<M, BT, smem, c->stream>>>(d_md, dS, dX, d_status);
  batch_density_kernel<<<M, BT, smem, c->stream>>>(1, d_md, d_active, dX, dH, dD, dDn, d_eps, d_it, d_conv, d_Ek,
                                                   d_Ef, thr, o->conv_rms, max_iter, d_status);
  c->stats.launches += 2;
  c->stats.guesses_taken = 0;
  if (o->D_in) {
    double *dg = (double *)buf(c, "batch_guess", mat * sizeof(double));
    int *d_used = (int *)buf(c, "batch_guess_used", (size_t)M * sizeof(int));
    if (!dg || !d_used) return MQ_ENOMEM;
    MQ_CUDA(c, cudaMemcpyAsync(dg, o->D_in, mat * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    const size_t sm_g = (size_t)nmax * nmax * sizeof(double);
    MQ_CUDA(c, cudaFuncSetAttribute(batch_guess_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_g));
    batch_guess_kernel<<<M, BT, sm_g, c->stream>>>(d_md, dg, dS, dD, d_used);
    c->stats.launches += 1;
    std::vector<int> used(M);
    MQ_CUDA(c, cudaMemcpyAsync(used.data(), d_used, (size_t)M * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    MQ_CUDA(c, cudaStreamSynchronize(c->stream));
    for (int v : used) c->stats.guesses_taken += v;
  }
  MQ_CUDA(c, cudaGetLastError());
  // ---- one SCF iteration for all active molecules
  PairLaunch L{};
  L.XX = d_XX;
  L.arith = c->fock_df32 ? FOCK_ARITH_DF32 : FOCK_ARITH_F64;  // FP64: the densities themselves; double-float: split copies
  L.DJ = L.arith ? (const void *)d_DJ : (const void *)dD;
  L.DKa = L.DJ;
  L.tiles = d_tiles;
  L.row_first = d_rf;
  L.mols = d_md;
  L.active = d_active;
  L.ntiles = (int)tl.size();
  L.nmol = M;
  L.nmax = nmax;
  L.J = dJ;
  L.Kpa = d_Kp;
  L.Qa = d_Q;
  L.Ka = dK;
  auto iteration = [&]() -> int {
    if (L.arith) MQ_TRY(split_density(c, dD, nullptr, mat, d_DJ, d_DJ, nullptr, 0));
    MQ_TRY(pair_digest(c, JC, false, L, dG, nullptr, false));
    batch_energy_kernel<<<M, BT, 0, c->stream>>>(d_md, d_active, dH, dG, dD, d_en, dF, d_Ek);
    const double *Fuse = dF;
    if (ndiis > 0) {
      batch_diis_kernel<<<M, BT, smem_diis, c->stream>>>(d_md, d_active, dF, dD, dS, dFh, dEh, d_B, d_state, ndiis,
                                                         mat, dFx);
      Fuse = dFx;
    }
    batch_density_kernel<<<M, BT, smem, c->stream>>>(0, d_md, d_active, dX, Fuse, dD, dDn, d_eps, d_it, d_conv,
                                                     d_Ek, d_Ef, thr, o->conv_rms, max_iter, d_status);
    MQ_CUDA(c, cudaGetLastError());
    return MQ_OK;
  };
  const int per_iter = 4 + (ndiis > 0 ? 1 : 0) + 3;  // split, digest (3), energy, diis, density
  StageTimer t_all;
  t_all.start(c->stream);
  MQ_TRY(iteration());  // eager: sets kernel attributes outside any capture
  c->stats.launches += per_iter;
  int done_iters = 1;
  cudaGraphExec_t exec = nullptr;
  if (o->graph) {
    cudaGraph_t graph = nullptr;
    MQ_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    const int rc2 = iteration();
    cudaError_t e = cudaStreamEndCapture(c->stream, &graph);
    if (rc2 != MQ_OK) return rc2;
    MQ_CUDA(c, e);
    e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    MQ_CUDA(c, e);
  }
  int graph_launches = 0;
  while (done_iters < max_iter) {
    if (done_iters % poll == 0) {
      batch_count_kernel<<<1, 256, 0, c->stream>>>(d_active, M, d_count);
      int h = 0;
      MQ_CUDA(c, cudaMemcpyAsync(&h, d_count, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
      MQ_CUDA(c, cudaStreamSynchronize(c->stream));
      if (h == 0) break;
    }
    if (exec) {
      MQ_CUDA(c, cudaGraphLaunch(exec, c->stream));
      ++graph_launches;
    } else {
      MQ_TRY(iteration());
    }
    c->stats.launches += per_iter;
    ++done_iters;
  }
  t_all.stop(c->stream);
  MQ_CUDA(c, cudaStreamSynchronize(c->stream));
  if (exec) cudaGraphExecDestroy(exec);
  t_all.collect();
  c->stats.ms_scf = t_all.total;
  c->stats.scf_iters = done_iters;
  c->stats.graph_launches = graph_launches;
  // ---- outputs
  std::vector<int> st(M), it(M), cv(M);
  MQ_CUDA(c, cudaMemcpy(energy, d_Ef, M * sizeof(double), cudaMemcpyDeviceToHost));
  MQ_CUDA(c, cudaMemcpy(it.data(), d_it, M * sizeof(int), cudaMemcpyDeviceToHost));
  MQ_CUDA(c, cudaMemcpy(cv.data(), d_conv, M * sizeof(int), cudaMemcpyDeviceToHost));
  MQ_CUDA(c, cudaMemcpy(st.data(), d_status, M * sizeof(int), cudaMemcpyDeviceToHost));
  if (iters) std::memcpy(iters, it.data(), M * sizeof(int));
  if (converged) std::memcpy(converged, cv.data(), M * sizeof(int));
  if (D_out) MQ_CUDA(c, cudaMemcpy(D_out, dD, mat * sizeof(double), cudaMemcpyDeviceToHost));
  if (eps_out) MQ_CUDA(c, cudaMemcpy(eps_out, d_eps, vec * sizeof(double), cudaMemcpyDeviceToHost));
  for (int m = 0; m < M; ++m)
    if (st[m] & 1) return set_err(c, MQ_EINVAL, "batch molecule " + std::to_string(m) + ": overlap not positive definite");
  return MQ_OK;
}

}  // namespace mq
