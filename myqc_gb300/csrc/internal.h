// internal.h -- shared declarations of libmyqc (not part of the C ABI).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <map>
#include <string>
#include <vector>

#include "../../include/myqc.h"

namespace mq {

constexpr int KMAX = 6;            // primitives per contracted shell (mybasis "max sets")
constexpr int FTAB_NT = 121;       // Ftab rows: T = 0.0 .. 12.0 step 0.1
constexpr int FTAB_NM = 23;        // Ftab columns: m = 0 .. 22
constexpr int TIGHT_NT = 361;      // own table rows: T = 0.0 .. 36.0 step 0.1
constexpr int TIGHT_NM = 13;       // m = 0 .. 12 (order <= 4 plus 8 Taylor terms)
constexpr double PI_REF = (double)3.1415926535897931f;  // the reference's pi
constexpr double PI_TRUE = 3.14159265358979323846;

// A contracted shell: s (1 function), or sp (4 functions: s, px, py, pz that
// share exponents).  A p-only shell is an sp shell whose s coefficients are 0.
struct HostShell {
  int atom;
  int type;      // 0: s, 1: sp
  int qlmax;     // lmax of the reference's primitive sets (Boys order, parity)
  int ao0;       // AO index of the first function
  int has_s, has_p;
  int nprim;
  double alpha[KMAX];
  double cs[KMAX];  // s coefficient x gtoD(0, alpha)
  double cp[KMAX];  // p coefficient x gtoD(1, alpha)
};

// Device view of the shell-pair / primitive-pair tables (structure of arrays).
struct PairTable {
  int npairs;            // shell pairs in class order
  int class_off[4];      // pair index ranges per class: [0]=ss, [1]=(sp,s), [2]=(sp,sp), [3]=end
  int *shA, *shB;        // shells of each pair (type(A) >= type(B))
  int *pp_off;           // primitive-pair offset, npairs+1
  int *aoA, *aoB;        // first AO of A and B (within the pair's molecule)
  int *mol;              // molecule of each pair (0 for a single system)
  double *schwarz;       // sqrt(max |(ab|ab)|) per pair
  // primitive pairs
  int npp;
  double *p, *inv2p, *beta, *Px, *Py, *Pz, *PAx, *PAy, *PAz, *PBx, *PBy, *PBz, *K, *c4;  // c4: 4 per pp
  // single-precision copy, 4 float4 per primitive pair:
  // p 1/2p K Px | Py Pz PAx PAy | PAz PBx PBy PBz | c4
  float4 *pf;
};

// Host copy of a pair table (same fields as PairTable), built per molecule
// and concatenated for batches.
struct HostPairs {
  int class_off[4] = {0, 0, 0, 0};
  std::vector<int> shA, shB, off, aoA, aoB, mol;
  std::vector<double> p, inv2p, beta, Px, Py, Pz, PAx, PAy, PAz, PBx, PBy, PBz, K, c4;
};

// One molecule added to a batch: host pair table, nuclei (x, y, z, Z) and
// closed-shell occupation.
struct BatchMol {
  int n = 0, nocc = 0, nnuc = 0;
  double enuc = 0.0;
  HostPairs pairs;
  std::vector<double> nuc;
};

struct DeviceBuf {
  void *ptr = nullptr;
  size_t bytes = 0;
};

// Device time (CUDA events on the context's stream) of the last call of each
// stage; the SCF accumulates over its iterations.
// device tile table of the pair-slab Fock kernel for one tile length
struct FockTiles {
  int n = 0, ntiles = 0;
  char *d = nullptr;  // int4 tiles[ntiles], int row_first[n + 1], MolDesc, in a named context buffer
  size_t rf_off = 0, mol_off = 0;
};

// One molecule of a (possibly one-molecule) batch as device kernels see it:
// its order and occupation, its nuclei in the packed nuclear table, and the
// offsets (in elements) of its XX (n^4), n x n matrices, n-vectors, Q (n^3)
// and Fock row table in the packed batch arrays.
struct MolDesc {
  int n, nocc, nnuc, nuc_off;
  long long xx, mat, vec, q;
  int row_first, pad;
};

// Quartet store: every contracted shell quartet that survives the Schwarz
// screen, its integral block written once (qstore.cu).  The pairs of each
// class are ranked by Schwarz bound, descending; for a class combination
// (bra class cP >= ket class cQ) the surviving ket ranks of bra rank r are
// then a prefix s < len_r ("staircase": len_r = m_r, or min(m_r, r + 1) when
// cP == cQ, with m_r = #{s : bound_P(r) bound_Q(s) >= threshold}).
struct QCombo {
  int cP = 0, cQ = 0, tri = 0, nout = 0;  // classes, same class, integrals per quartet
  int nP = 0, nQ = 0;                     // ranks in the bra and ket class
  long long total = 0;                    // quartets
  long long base = 0;                     // offset (doubles) of the combination's blocks in the store
  long long *off = nullptr;               // device: nP + 1 quartet offsets by bra rank
  int *len = nullptr;                     // device: nP staircase lengths
  int *rcol = nullptr;                    // device: per ket rank s, R_s = #{r : m_r > s}
};
struct QStore {
  int valid = 0;        // the store holds the current system's integrals
  int tables_valid = 0; // ranking, staircase and digestion tables of the current system and thr
  double thr = 0.0;     // Schwarz threshold it was built with
  int ncls[3] = {0, 0, 0}, cls_off[3] = {0, 0, 0};
  int *perm = nullptr;  // device: class offset + rank -> pair index
  QCombo combo[6];      // index cP (cP + 1) / 2 + cQ
  double *X = nullptr;  // device: the integral blocks
  size_t X_elems = 0;
  // digestion tables (device), built with the store
  int nthr = 0, nsp_pad = 0;  // row-pass threads: sp-shell AOs, padded to 32 (nsp_pad), then s AOs, padded
  int *thr_shell = nullptr;   // row-pass thread -> shell (-1: idle)
  int *thr_ao = nullptr;      // row-pass thread -> its AO column
  int4 *rinfo = nullptr;      // by class offset + rank: pair, A | B << 16, i0 | j0 << 16
  int *lst_off = nullptr;     // [(3 classes x 2 roles) x (nshell + 1)] offsets into lst
  int4 *lst = nullptr;        // pairs of class cQ whose role-th shell is s, by ascending rank:
                              // (rank, pair, C | D << 16, k0 | l0 << 16)
  int *ksh_off = nullptr;     // [nshell + 1] offsets into ksh
  int2 *ksh = nullptr;        // (pair, row offset of the shell in the pair's partial K rows)
  int *shell_ao0 = nullptr;   // [nshell] first AO of each shell
  int *ao_shell = nullptr;    // [n] shell of each AO
  double *shell_qmax = nullptr;  // [nshell] the largest Schwarz bound of a pair containing the shell
  int4 *pinfo = nullptr;      // [S1 * nshell + S2]: pair, class, rank, bit 0: stored as (S2, S1), bit 1: S1 = S2
  int *partners = nullptr;    // [S * nshell + k]: the shells D by the bound of the pair (D, S), descending
  double quartets = 0;        // quartets stored
  double unique = 0;          // canonical unique integrals stored (the digestion's 6 FMAs each)
};

struct Stats {
  double ms_eri = 0, ms_fock = 0, ms_diag = 0, ms_ao2mo = 0, ms_mp2 = 0, ms_scf = 0;
  double ms_ao2mo_first = 0;  // the transform's first quarter (from the quartet store), last transform
  double fock_calls = 0, diag_calls = 0, scf_iters = 0, purify_steps = 0, fock_jc = 0, tune_fock_ms = 0;
  double purify_persistent = 0, purify_stepwise = 0;  // purifications of the last SCF by form
  double guesses_taken = 0;  // batch: caller guesses that passed the checks (last batched SCF)
  double launches = 0, lib_launches = 0, quartets = 0, prim_quartets = 0;
  double ms_fock_kernel = 0, fock_kernel_launches = 0;  // the digestion kernel alone, last SCF or mq_fock
  double graph_launches = 0;  // CUDA-graph replays of the last batch SCF
  double eig_cluster = 0;     // CTAs of the last FP32 cluster eigensolve (0: none)
  double ms_eig_final = 0;    // the last SCF's final eigensolve (purification mode)
  // last cold eigensolve: FP32 cluster sweeps and off-norm ratio reached, its
  // phases' times, FP64 Jacobi sweeps
  double eig_f32_sweeps = 0, eig_f32_off = 0, ms_eig_f32 = 0, ms_eig_refine = 0, ms_eig_jacobi = 0;
  double eig_jacobi_sweeps = 0;
  double fock_inc_builds = 0;  // FP32 incremental builds of the last SCF
  double fock_screened_builds = 0;  // screened FP64 increments from the quartet store, last SCF
  double fock_full_builds = 0;      // stored full builds of the last SCF, and their time (ms)
  double ms_fock_full = 0;
  double eig_early = 0;        // 1: the last SCF's final eigensolve started from its early eigensolve
};

// Event pair on the context's stream that adds its elapsed time to a counter
// at the next synchronisation point.
struct StageTimer {
  cudaEvent_t a = nullptr, b = nullptr;
  double total = 0;
  bool pending = false;
  void start(cudaStream_t s) {
    if (!a) {
      cudaEventCreate(&a);
      cudaEventCreate(&b);
    }
    cudaEventRecord(a, s);
  }
  void stop(cudaStream_t s) {
    cudaEventRecord(b, s);
    pending = true;
  }
  void collect_sync() {  // wait for the end event first
    if (pending) cudaEventSynchronize(b);
    collect();
  }
  void collect() {  // call after the stream has been synchronised
    if (!pending) return;
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    total += ms;
    pending = false;
  }
  ~StageTimer() {
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
  }
};

}  // namespace mq

namespace mq {
// The integral autotuner's choice for one launch signature (eri_store.cu):
// launch order binned by surviving primitive quartets or not, CTA size,
// persistent work queue or one warp per work unit, and the time the
// candidate took when it was measured
struct EriTune {
  int binned = 1;
  int block = 128;
  int persistent = 0;  // warps take work units from a queue in a grid of resident CTAs
  float ms = 0.f;
};
}  // namespace mq

struct mq_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;  // the context's stream (highest priority)
  // side stream (lowest priority) for work that overlaps the main stream: the
  // slicing of XX for the split transform during the SCF's final eigensolve
  // (mq_set_ao2mo_prefetch).  ev_side marks the end of the last side work;
  // anything that rewrites XX or the slice buffers waits for it (join_side).
  cudaStream_t side = nullptr;
  cudaEvent_t ev_main = nullptr, ev_side = nullptr;
  int side_pending = 0;
  // aux stream (highest priority) for the learned guess's network forward
  // pass, so that it does not queue behind the integral pass on the main
  // stream; ev_params marks the last write of the network's parameters
  cudaStream_t aux = nullptr;
  cudaEvent_t ev_params = nullptr;
  cudaEvent_t ev_early = nullptr;  // the SCF's early eigensolve on the aux stream
  int ao2mo_prefetch = 0;  // planes (2, 3) to slice XX into ahead of the transform; 0: off
  int xx_sliced = 0;       // the slice buffers hold XX cut into this many planes (0: not)
  std::string err;
  // system
  int have_system = 0;
  int mode = MQ_MODE_REFERENCE;
  int nnuc = 0, nao = 0, nshell = 0;
  double schwarz_thr = 0.0;
  std::vector<int> Z;
  std::vector<double> xyz;  // nnuc x 3, row-major (atom, xyz)
  std::vector<mq::HostShell> shells;
  std::vector<int> pair_class_count;
  // device data
  double *d_boys = nullptr;  // Ftab (parity) or own table (tight)
  float *d_boys_f32 = nullptr;  // tight table in single precision (mixed-precision integrals)
  double eri_f32_tau = 0.0;     // quartets with a Schwarz bound below this are computed in FP32 (0: off)
  double *d_nuc = nullptr;   // nnuc x 4: x, y, z, Z
  mq::PairTable pt{};
  std::vector<void *> pair_allocs;
  void *pin = nullptr;  // pinned staging buffer of the pair-table uploads
  size_t pin_bytes = 0;
  int boys_loaded = -1;  // mode whose Boys table d_boys holds (-1: none; reference tables are always reloaded)
  int nuc_cap = 0;       // nuclei d_nuc has room for
  double *d_XX = nullptr;    // n^4 full integral array (kept allocated across systems of the same order)
  int xx_valid = 0;          // d_XX holds the current system's integrals (mq_eri_store / mq_eri_upload)
  // batch of independent closed-shell molecules (mq_batch_*)
  std::vector<mq::BatchMol> bmols;
  std::vector<void *> batch_allocs;  // batch pair table
  double *d_boys_tight = nullptr;    // the tight Boys table, for batches
  void *mlp = nullptr;               // the learned guess's network (mlp.cu)
  mq::StageTimer t_fock_kernel;
  mq::StageTimer t_eri;                       // the last integral pass, collected when asked for
  mq::StageTimer t_eri_kernel;                // its integral kernels alone (quartet store)
  // live[i + n j] = 0 when every integral of slab XX(:,:,i,j) was screened out
  // (Schwarz bound of the slab's shell pair times the largest bound below the
  // threshold): the slab is zero and the digestion skips it.  Valid for the
  // integrals of the last mq_eri_store with a threshold; null otherwise.
  unsigned char *d_slab_live = nullptr;
  int slab_live_valid = 0;
  int schwarz_valid = 0;  // pt.schwarz holds the bounds of the current system
  unsigned long long *d_slab_live_count = nullptr;  // live slabs (i, j), both orders counted
  // integral storage of mq_eri_store: 0 the full n^4 array (the reference's
  // XX layout), 1 the quartet store (Schwarz threshold > 0, RHF digestion;
  // the n^4 array is filled from it when a consumer needs it)
  int eri_storage = 0;
  // this process's share of a single molecule's quartets (mq_set_partition):
  // the quartet-store rows whose bra pair index is part mod nparts
  int part = 0, nparts = 1;
  mq::QStore qs;
  // integral autotuner (eri_store.cu): 1 tune launches of a new signature on
  // first use, 0 the defaults; choices per (epilogue, class combination,
  // size class) and the measured candidates, in the order tuned
  int eri_tune_mode = 1;
  // the basis library text as tokenised lines, and the row of its STO-3G key
  // (mq_basis_library; basis_lib.cu)
  std::vector<std::vector<std::string>> basis_rows;
  int basis_key = -1;
  // the learned guess's feature and output standardisation (mq_guess_model; guess.cu)
  std::vector<double> guess_mu_x, guess_sd_x, guess_mu_y, guess_sd_y;
  std::map<unsigned long long, mq::EriTune> eri_tune;
  std::vector<std::pair<unsigned long long, std::vector<mq::EriTune>>> eri_tune_log;
  std::vector<int> hp_shA, hp_shB, hp_aoA, hp_aoB;  // host copy of the pair table's shells and AO offsets
  int hp_class_off[4] = {0, 0, 0, 0};
  unsigned long long *d_eri_counters = nullptr;  // its quartet counters (device)  // the digestion kernel alone, collected at the caller's sync points
  mq::FockTiles fock_tiles[9];  // pair-slab tile tables, indexed by slabs per tile
  int fock_jc[2][3] = {{0, 0, 0}, {0, 0, 0}}, fock_jc_n[2][3] = {{0, 0, 0}, {0, 0, 0}};  // tile length [uhf][arith]
  int fock_df32 = 0;  // digestion arithmetic: 0 FP64, 1 double-float (mq_set_fock_precision)
  // mq_scf with stored integrals: once max|D_k - D_{k-1}| < fock_inc_tau, G_k =
  // G_{k-1} + G[D_k - D_{k-1}] digested in FP32 (0: every build full; mq_set_fock_incremental)
  double fock_inc_tau = 0.0;
  // mq_scf from the quartet store (RHF): after the first build, G_k = G_{k-1} +
  // G[D_k - D_{k-1}] in FP64 over the quartets with Q_P Q_Q max|dD| >= this
  // (0: full builds; mq_set_fock_screened_increments)
  double fock_inc_screen = 0.0;
  size_t XX_elems = 0;
  double *d_iajb = nullptr;  // last (ia|jb) block
  size_t iajb_elems = 0;
  int iajb_dims[4] = {0, 0, 0, 0};
  int iajb_precision = 0;  // MQ_PREC_* of the transform that produced d_iajb
  // named device work buffers: each grows on demand and is reused across calls
  std::map<std::string, mq::DeviceBuf> bufs;
  mq::Stats stats;
};

namespace mq {
// error helpers
int set_err(mq_ctx *c, int code, const std::string &msg);
int cuda_check(mq_ctx *c, cudaError_t e, const char *what);
// device buffer `name` of at least `bytes` (contents undefined after growth);
// nullptr on failure with the error set
void *buf(mq_ctx *c, const char *name, size_t bytes);
// With MYQC_SYNC_CHECK=1 in the environment: synchronise the stream and report
// the first failing stage by `label` (a diagnostic; off by default).
int sync_check(mq_ctx *c, const char *label);

// batched kernels (int1e.cu, eri.cu, fock.cu)
int int1e_batch_device(mq_ctx *c, const PairTable &t, const double *d_nuc, const MolDesc *d_mols, size_t mat_total,
                       double *d_S, double *d_H);
int eri_batch_device(mq_ctx *c, const PairTable &t, const MolDesc *d_mols, int nmol, const int *d_pstart,
                     const int *d_pcount, const long long *const d_mq_off[6], const long long total[6], double *d_XX,
                     size_t xx_total);
void pair_tiles_host(int n, int JC, int mol, std::vector<int4> &tl, std::vector<int> &rf);
// Everything one pair-slab Fock launch needs; `nmax` is the largest order among
// the molecules (thread count, shared memory, K-slice stride).
struct PairLaunch {
  const double *XX;
  const void *DJ, *DKa, *DKb;  // float2 (df32) or double arrays
  const int4 *tiles;
  const int *row_first;
  const MolDesc *mols;
  const int *active;
  int ntiles, nmol, nmax;
  int tri;   // DJ carries lower-triangle weights: J sums over l <= k only
  const unsigned char *live;  // slab (i,j) may be nonzero (n x n, single system); null: every slab
  int arith;  // FOCK_ARITH_*: FP64 arrays, float pairs (double-float), or floats (FP32 increments)
  const double *Gbase;  // single system: G = Gbase + J - f K (null: G = J - f K)
  double *J, *Kpa, *Kpb, *Qa, *Qb, *Ka, *Kb;
};
// density operands of the digestion in the context's arithmetic (fock.cu)
int fock_densities(mq_ctx *c, int n, const double *d_Da, const double *d_Db, const void **DJ, const void **DKa,
                   const void **DKb);
enum { FOCK_ARITH_F64 = 0, FOCK_ARITH_DF32 = 1, FOCK_ARITH_F32 = 2 };
int pair_digest(mq_ctx *c, int JC, bool uhf, const PairLaunch &L, double *d_Ga, double *d_Gb, bool timed);
// G = Gprev + G[D - Dprev] for the stored integrals, digested in FP32 (the
// incremental builds of mq_scf); RHF when the beta arguments are null
int fock_stored_increment(mq_ctx *c, const double *d_Da, const double *d_Db, const double *d_Dpa,
                          const double *d_Dpb, const double *d_Gpa, const double *d_Gpb, double *d_Ga, double *d_Gb);
// densities as hi/lo float pairs: DJ from Da (+ Db), DKa from Da, DKb from Db;
// tri_n > 0: DJ with lower-triangle weights for a system of order tri_n
int split_density(mq_ctx *c, const double *Da, const double *Db, size_t n2, float2 *DJ, float2 *DKa, float2 *DKb,
                  int tri_n);
// mlp.cu
int mlp_init(mq_ctx *c, int nin, int width, int nout);
int mlp_param_count(mq_ctx *c);
int mlp_set_params(mq_ctx *c, const float *h);
int mlp_get_params(mq_ctx *c, float *h);
int mlp_forward(mq_ctx *c, int rows, const float *X, float *Y);
int mlp_grad(mq_ctx *c, int rows, const float *X, const float *T, const float *Wl, float *grads, double *loss);
int mlp_set_data(mq_ctx *c, long long n, const float *X, const float *T, const float *Wl);
int mlp_train_epoch(mq_ctx *c, const int *perm, int batch, float lr, double *loss);
void mlp_free(mq_ctx *c);
// batch.cu
int batch_clear(mq_ctx *c);
int batch_add(mq_ctx *c, int nnuc, const int *Z, const double *xyz, const double *bas, const double *set,
              const int *basinfo, const int *setinfo, int nocc);
int batch_scf(mq_ctx *c, const mq_batch_opts *o, double *energy, int *iters, int *converged, double *D_out,
              double *eps_out);

// basis.cu
int build_shells(mq_ctx *c, int nnuc, const int *Z, const double *xyz, const double *bas, const double *set,
                 const int *basinfo, const int *setinfo);
int build_pairs(mq_ctx *c);
void pairs_host(const std::vector<HostShell> &shells, const std::vector<double> &xyz, HostPairs &h);
void append_pairs_class(HostPairs &dst, const HostPairs &src, int cl, int mol);
int upload_pairs(mq_ctx *c, const HostPairs &h, std::vector<void *> *allocs, PairTable &t);
void free_pairs(mq_ctx *c);
void tight_boys_table(std::vector<double> &tab);  // TIGHT_NT x TIGHT_NM, row-major [T][m]
constexpr int BOYS_SCALED_M = 5;                  // orders with their own Taylor-coefficient table
void tight_boys_device_table(std::vector<double> &tab);  // the table, its grid, the scaled tables

// eri.cu
int eri_full_device(mq_ctx *c, double *d_XX);
// integral blocks of every combination of the quartet store (tables built)
int eri_store_quartets(mq_ctx *c);
// mlp.cu: the network's forward pass on device features (the learned guess)
int mlp_forward_device(mq_ctx *c, int rows, const float *dX, float **dY);
int mlp_dims(mq_ctx *c, int dims[4]);
std::string eri_tune_report(const mq_ctx *c);  // the autotuner's choices and timings, one line per signature
// qstore.cu: rank the pairs, build the staircase and digestion tables, compute
// the integral blocks; RHF G from the store; the n^4 array filled from it
int qstore_build(mq_ctx *c);
// G = d_Gprev + G[d_D] (d_Gprev null: G[d_D]); kscreen > 0 skips the shell
// quartets with Schwarz bounds Q_P Q_Q < kscreen (screened increments)
int qstore_fock_rhf(mq_ctx *c, const double *d_D, double *d_G, const double *d_Gprev = nullptr,
                    double kscreen = 0.0);
int qstore_expand(mq_ctx *c, double *d_XX);
// direct RHF G (no integrals kept between builds): the store's integral blocks
// recomputed, then digested like a stored build (atomic-free, deterministic)
int fock_direct_store_rhf(mq_ctx *c, const double *d_D, double *d_G);
// the full n^4 array of the current system: computed (full storage) or filled
// from the quartet store
int ensure_xx_full(mq_ctx *c);
int ensure_xx_alloc(mq_ctx *c);  // the n^4 device array of the current order (capi.cu)
int eri_schwarz(mq_ctx *c);
int ensure_schwarz(mq_ctx *c);  // eri_schwarz unless the current system's bounds are there
int fock_direct_device(mq_ctx *c, const double *d_Da, const double *d_Db, double *d_J, double *d_Ka, double *d_Kb);
// G = sym(J) - f sym(K) from the direct kernel's half-sums (f = 1/2 RHF, 1 UHF)
int direct_combine(mq_ctx *c, const double *J, const double *Ka, const double *Kb, double *Ga, double *Gb);

// int1e.cu
int int1e_device(mq_ctx *c, double *d_S, double *d_H);
int int1p_device(mq_ctx *c, double *d_Px);  // dipole integrals, 3 n x n (x, y, z)

// fock.cu
int fock_stored_device(mq_ctx *c, const double *d_Da, const double *d_Db, double *d_Ga, double *d_Gb);

// linalg.cu
constexpr int JAC_SMEM_MAX = 110;  // largest order whose A and V (2 n^2 doubles) fit in shared memory
int syev_batched_device(mq_ctx *c, int n, int batch, double *d_A, double *d_w, double *d_V);
// one matrix of order n > JAC_SMEM_MAX on all SMs; d_V0 (optional) are start
// vectors and d_A must then already be V0^T A V0
int syev_large_device(mq_ctx *c, int n, double *d_A, const double *d_V0, double *d_w, double *d_V,
                      bool async = false);
// after an async syev_large_device/cold solve has finished: its status (0 ok,
// MQ_ETIMEOUT, MQ_ENOCONV), read from the solver's workspace on c->stream
int syev_large_status(mq_ctx *c);
// one matrix of order n > JAC_SMEM_MAX without start vectors: FP32 Jacobi on a
// thread-block cluster, FP64 refinement, then syev_large_device (eigen.cu)
// async: queue everything on c->stream and return without reading anything
// back (no host synchronisation); syev_large_status then gives the outcome
int syev_large_cold(mq_ctx *c, int n, double *d_A, double *d_w, double *d_V, bool async = false);
// from start vectors d_V of a nearby matrix: FP64 refinement by GEMMs (first-order
// rotations of the separated pairs), then the FP64 Jacobi cleanup (eigen.cu)
int syev_large_warm(mq_ctx *c, int n, double *d_A, double *d_w, double *d_V);
// start vectors d_V of a matrix of order JAC_SMEM_MAX < n <= 512 for a later
// syev_large_warm: FP32 cluster Jacobi and the FP64 first-order refinement,
// queued on c->stream with no grid-wide barrier and nothing read back (eigen.cu)
int syev_large_start(mq_ctx *c, int n, const double *d_A, double *d_V);
// small FP64 products on all SMs (dgemm.cu); gemm() takes them when they fit
bool dgemm_small_fits(int m, int n, int k);
int dgemm_small(mq_ctx *c, char ta, char tb, int m, int n, int k, double alpha, const double *A, int lda,
                const double *B, int ldb, double beta, double *C, int ldc);
// any FP64 product, batched over blockIdx.z with strides sA, sB, sC (dgemm.cu)
int dgemm_batched(mq_ctx *c, char ta, char tb, int m, int n, int k, double alpha, const double *A, int lda,
                  long long sA, const double *B, int ldb, long long sB, double beta, double *C, int ldc,
                  long long sC, int batch);
int gemm(mq_ctx *c, char ta, char tb, int m, int n, int k, double alpha, const double *A, int lda, const double *B,
         int ldb, double beta, double *C, int ldc);
int gemm_strided_batched(mq_ctx *c, char ta, char tb, int m, int n, int k, double alpha, const double *A, int lda,
                         long long sA, const double *B, int ldb, long long sB, double beta, double *C, int ldc,
                         long long sC, int batch);
int density_device(mq_ctx *c, int n, int nocc, const double *d_C, double factor, double *d_D);
int syrk_lower(mq_ctx *c, int n, int k, double alpha, const double *A, int lda, double beta, double *C, int ldc);
// spectral projector onto the nocc lowest eigenvectors of the symmetric d_Fp
// by trace-correcting purification (d_T, d_W: n x n scratch; d_err: >= 120
// doubles); MQ_ENOCONV when the frontier levels are degenerate
int purify_projector(mq_ctx *c, int n, int nocc, const double *d_Fp, double *d_P, double *d_T, double *d_W,
                     double *d_err, int *steps);
// X = S^-1/2 by the coupled Newton-Schulz iteration (w: 5 n^2 doubles of
// scratch, d_err: >= 101 doubles); MQ_ENOCONV when it does not settle
int inv_sqrt_ns(mq_ctx *c, int n, const double *d_S, double *d_X, double *w, double *d_err, int *steps);

// ao2mo.cu
int ao2mo_device(mq_ctx *c, const double *d_Ci, int no1, const double *d_Ca, int nv1, const double *d_Cj, int no2,
                 const double *d_Cb, int nv2, int precision, double *d_out);
int mp2_rhf_device(mq_ctx *c, const double *d_iajb, const double *d_eig, int nocc, int nvir, double *e_out);
// sums[0] = sum_{ijab} x^2/D, sums[1] = sum_{i<j,a<b} (x_iajb - x_ibja)^2/D (same_spin only);
// d_e1/d_e2: orbital energies of the (i,a) and (j,b) spins, occupied first
int mp2_pair_sums(mq_ctx *c, const double *d_Om, int no1, int nv1, int no2, int nv2, const double *d_e1,
                  const double *d_e2, int same_spin, double *sums);
// ao2mo_split.cu: split-BF16 tensor-core transform (tcgen05) with 2 or 3 operand planes
int ao2mo_split_device(mq_ctx *c, const double *d_Ci, int no1, const double *d_Ca, int nv1, const double *d_Cj,
                       int no2, const double *d_Cb, int nv2, double *d_out, int planes);
// XX cut into c->ao2mo_prefetch planes on the side stream, after the work queued
// so far on the main stream; the next split transform of the same XX uses it
int ao2mo_preslice_xx(mq_ctx *c);
// the aux stream (highest priority) and the event of its SCF hand-overs, created on first use
int ensure_aux(mq_ctx *c);
// the main stream waits for the side stream's last work (no-op when none is pending)
int join_side(mq_ctx *c);

// scf.cu
int scf_device(mq_ctx *c, const double *S, const double *H, const mq_scf_opts *o, double *C, double *eps, double *D,
               double *energy, int *iters, double *history);
}  // namespace mq

#define MQ_CUDA(c, call)                                   \
  do {                                                     \
    cudaError_t _e = (call);                               \
    if (_e != cudaSuccess) return mq::cuda_check(c, _e, #call); \
  } while (0)

#define MQ_TRY(call)         \
  do {                       \
    int _rc = (call);        \
    if (_rc != MQ_OK) return _rc; \
  } while (0)
