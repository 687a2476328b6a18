/*
 * myqc.h -- C ABI of libmyqc, the GB300 (sm_103a) engine behind the myQC
 * drop-in executables int2e, scf, ao2mo and mp2.
 *
 * Every entry point is extern "C", takes plain pointers and sizes, and
 * returns an int status (MQ_OK == 0).  Host arrays follow the reference's
 * Fortran conventions: column-major, 0-based in Fortran terms, owned by the
 * caller and read or written only during the call.  Device memory and the
 * CUDA stream belong to the opaque context.  A context is single-threaded
 * (one caller thread at a time), like the reference's programs.
 *
 * Each declaration names the reference routine it replaces (file:line in
 * jhthorpe/myQC).  A Fortran host binds them through iso_c_binding with the
 * interface module include/myqc_gpu.f90.
 */
#ifndef MYQC_H
#define MYQC_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define MQ_OK 0
#define MQ_EINVAL 1     /* bad argument, unsupported basis, size limits */
#define MQ_ENOMEM 2     /* device allocation failed */
#define MQ_ECUDA 3      /* CUDA runtime / launch error */
#define MQ_ETIMEOUT 4   /* a bounded device wait gave up */
#define MQ_ENOCONV 5    /* SCF or eigensolver did not converge */
#define MQ_ESTATE 6     /* call order violated (e.g. no system set) */

/* Boys-function / pi mode passed to mq_set_system */
#define MQ_MODE_REFERENCE 0 /* reference parity: Ftab Taylor table, the
                               reference's float-valued pi and its regimes */
#define MQ_MODE_TIGHT 1     /* accurate FP64 Boys (~1e-15) and true pi */

typedef struct mq_ctx mq_ctx;

/* Create / destroy a context on CUDA device `device`.  The reference has one
 * process per stage; a context plays that role (src/myQC/myQC.f90:29-105). */
int mq_init(mq_ctx **ctx, int device);
int mq_free(mq_ctx *ctx);

/* Copy the last error message (NUL-terminated, truncated to len). */
int mq_last_error(const mq_ctx *ctx, char *buf, int len);

/* Library version string, e.g. "myqc-gb300 0.1 sm_103a". */
const char *mq_version(void);

/* FP64 fused multiply-add rate of the context's GPU in TFLOP/s, measured by a
 * short kernel of independent FP64 fma chains.  No counterpart in the
 * reference: the denominator of the FP64-bound kernels' roofline. */
int mq_probe_fp64(mq_ctx *ctx, double *tflops);

/* Define the molecule and basis.  Replaces getenv (src/myQC/env.f90:16-74)
 * plus buildBasis (src/myQC/basis.f90:23-226) plus the Ftab read
 * (src/integrals/int2e.f90:160-163):
 *   Z[nnuc]           nuclear charges (atoms(0:nnuc-1))
 *   xyz[nnuc*3]       bohr, Fortran xyz(0:nnuc-1,0:2), column-major
 *   bas, set, basinfo, setinfo   the flat arrays buildBasis returns
 *   ftab[121*23]      Ft(0:120,0:22) column-major; required in
 *                     MQ_MODE_REFERENCE, may be NULL in MQ_MODE_TIGHT
 * Contracted s and p functions only (the reference rejects d:
 * basis.f90:170-174).  Uploads shells, primitive pairs and the Boys table. */
int mq_set_system(mq_ctx *ctx, int nnuc, const int *Z, const double *xyz, const double *bas, const double *set,
                  const int *basinfo, const int *setinfo, const double *ftab, int mode);

/* Number of AOs (basinfo(1)) of the current system. */
int mq_norb(const mq_ctx *ctx, int *norb);

/* Contracted-quartet Schwarz threshold for the integral kernels
 * (0 = off, the reference's behaviour; 1e-12 for direct SCF at scale). */
int mq_set_schwarz(mq_ctx *ctx, double threshold);

/* Mixed-precision integral pass (MQ_MODE_TIGHT only; 0 = off, every quartet
 * in FP64): contracted quartets whose Schwarz bound is below tau are computed
 * in FP32, the rest in FP64 (dynamic precision as in Luehr, Ufimtsev and
 * Martinez, J. Chem. Theory Comput. 7, 949 (2011)); an integral's FP32 error
 * stays a small multiple of tau * 1e-6.  Applies to mq_eri_store/mq_eri_full. */
int mq_set_eri_mixed(mq_ctx *ctx, double tau);

/* One-electron integrals S and H = T + V, n x n column-major host arrays.
 * Replaces proc1e (src/integrals/int1e.f90:132-280). */
int mq_int1e(mq_ctx *ctx, double *S, double *H);

/* Dipole integrals Px(c, u, v) = <u| r_c |v> about the origin (bohr), c = x, y, z,
 * written as three n x n column-major matrices one after the other (the order of
 * the reference's Pxuv file); replaces proc1p (src/integrals/int1p.f90:150-300).
 * The dipole moment of cphf_dipole_rhf (src/props/cphf.f90:80-131) is then
 * mu_c = -sum_uv D(u,v) Px(c,v,u) + sum_A Z_A R_A,c on the host. */
int mq_int1p(mq_ctx *ctx, double *Px);

/* Full two-electron integral array XX(i,j,g,h) at i+n*(j+n*(g+n*h)), all 8
 * permutations filled, into a host buffer of n^4 doubles.  Replaces proc2e +
 * fillsym (src/integrals/int2e.f90:78-351,540-613).  Also leaves the array
 * resident on the device for mq_fock / mq_ao2mo_iajb. */
int mq_eri_full(mq_ctx *ctx, double *XX);

/* As mq_eri_full but keeps the integrals on the device only (no host copy),
 * in the storage mq_set_eri_storage selected. */
int mq_eri_store(mq_ctx *ctx);

/* Device storage of mq_eri_store (no counterpart in the reference, which
 * writes the full XX file, src/integrals/int2e.f90:540-613):
 *   MQ_STORE_FULL (default): the n^4 array XX(i,j,g,h), every permutation;
 *   MQ_STORE_QUARTETS: each contracted shell quartet that passes the Schwarz
 *     screen (threshold > 0 required at mq_eri_store) stored once as one
 *     block; the RHF Fock build digests it directly (six FP64 multiply-adds
 *     per unique integral), and consumers of the full array (UHF builds, the
 *     four-index transform, mq_eri_full) get it filled from the store on
 *     first use. */
/* This process's share of one molecule's Fock builds when several processes
 * (one GPU each) split it: the quartet store and the direct RHF build keep
 * only the shell quartets whose bra shell pair index is part mod nparts, so
 * mq_fock / mq_fock_direct return that share's part of G; the sum over the
 * parts (one all-reduce of n x n doubles) is the full G.  No counterpart in
 * the reference (one process, src/I2G/RHFI2G.f90:80-90).  (0, 1): no split. */
int mq_set_partition(mq_ctx *ctx, int part, int nparts);

#define MQ_STORE_FULL 0
#define MQ_STORE_QUARTETS 1
int mq_set_eri_storage(mq_ctx *ctx, int storage);

/* The integral autotuner (no counterpart in the reference, whose set-quartet
 * loop has no launch shape, src/integrals/int2e.f90:192-241): mode 1
 * (default) times the candidate launch shapes of each integral launch of a
 * new size class once -- launch order binned by surviving primitive quartets
 * or not, 64/128/256 threads per CTA -- and keeps the fastest for the
 * context's later passes; mode 0 uses the defaults (binned, 128). */
int mq_set_eri_tuning(mq_ctx *ctx, int mode);

/* The autotuner's choices so far as text, one line per launch signature (the
 * candidates with their times, the chosen one marked '*'); truncated to len. */
int mq_eri_tuning_report(const mq_ctx *ctx, char *buf, int len);

/* Upload an existing XX (n^4 doubles, the int2e file payload) to the device,
 * e.g. when a drop-in scf reads the reference's XX file. */
int mq_eri_upload(mq_ctx *ctx, const double *XX);

/* Fock two-electron part from the device-resident XX.
 * RHF (Db == NULL, Gb == NULL): G = sum_kl D_kl[(ij|kl) - 1/4(ik|jl) - 1/4(il|jk)]
 *   replaces RHFI2G (src/I2G/RHFI2G.f90:80-90);
 * UHF: Ga = J[Da+Db] - K[Da], Gb = J[Da+Db] - K[Db]
 *   replaces UHFI2G (src/I2G/UHFI2G.f90:80-93).
 * All matrices n x n column-major host arrays. */
int mq_fock(mq_ctx *ctx, const double *Da, const double *Db, double *Ga, double *Gb);

/* Arithmetic of the stored-integral Fock digestion (mq_fock, mq_scf, batches).
 * MQ_FOCK_FP64 (default): FP64 products and sums, the reference's arithmetic.
 * MQ_FOCK_DF32: each integral split into a float pair, products and row sums
 * in double-float on the FP32 pipes (~2^-48 relative per product, below 1e-12
 * relative on G), sums over slabs in FP64; no reference counterpart. */
#define MQ_FOCK_FP64 0
#define MQ_FOCK_DF32 1
int mq_set_fock_precision(mq_ctx *ctx, int precision);

/* Incremental Fock builds in mq_scf with stored integrals; no reference
 * counterpart.  tau > 0: once the density of an iteration differs from the
 * previous one by less than tau (max |D_k - D_(k-1)|), the build is
 * G_k = G_(k-1) + G[D_k - D_(k-1)] with the increment digested in FP32 on the
 * FP32 pipes; larger changes get full builds in the mq_set_fock_precision
 * arithmetic.  The increment's error scales with its size: on (H2O)8 the
 * converged energy stays within 1e-9 Eh of full builds for tau up to 1e-2.
 * tau = 0 (default): full builds only.  MQ_EINVAL outside [0, 1e-2]. */
int mq_set_fock_incremental(mq_ctx *ctx, double tau);

/* Screened FP64 increments in mq_scf from the quartet store (RHF; no
 * reference counterpart: the reference rebuilds G from all of XX every
 * iteration, src/I2G/RHFI2G.f90:80-90).  tau > 0: after the SCF's first build,
 * each build is G_k = G_(k-1) + G[D_k - D_(k-1)] in FP64, digesting only the
 * shell quartets whose Schwarz bounds satisfy Q_P Q_Q max|D_k - D_(k-1)| >=
 * tau -- the integral screen's own criterion applied to the density change,
 * so late iterations, whose density moves little, digest a small part of the
 * store.  tau = 0 (default): full builds.  MQ_EINVAL outside [0, 1e-6]. */
int mq_set_fock_screened_increments(mq_ctx *ctx, double tau);

/* Overlap for the split-precision transform; no reference counterpart.
 * planes = 2 or 3 (MQ_PREC_SPLIT_BF16 / MQ_PREC_SPLIT_BF16X3): an mq_scf that
 * ends with an eigensolve of the purified Fock matrix (opts.purify) cuts the
 * stored XX into that many BF16 planes on a low-priority side stream while
 * the eigensolve runs, and the next split mq_ao2mo_iajb / mq_mp2_* of the same
 * XX starts from those slices.  Results are identical with and without it.
 * 0 (default): off. */
int mq_set_ao2mo_prefetch(mq_ctx *ctx, int planes);

/* Allocation-free RHF Fock build.  No counterpart in the reference: it exists
 * for callers that cannot allocate device memory themselves (device arrays
 * owned by an OpenACC / OpenMP-offload runtime or a preallocated pool, code
 * that must not call cudaMalloc while it runs).  All pointers are device
 * pointers the caller owns: d_XX (n^4 doubles, the XX layout), d_D (n x n
 * total density), d_G (n x n output, G = J - K/2 as mq_fock computes it).
 * No context is needed and nothing is allocated or freed: the kernels'
 * scratch is a fixed 16 MiB array inside the library, held by every GPU that
 * loads it until the process exits.  It holds G's J part and the K partial
 * sums (FP64 arithmetic), which with n <= 1024 always fit (2 n^2 <= 2097152
 * doubles); larger n returns MQ_EINVAL.  The work is queued on
 * `stream` (NULL: the default stream) and the call returns without waiting;
 * G is ready once that stream reaches this point.  All calls share the one
 * scratch array, so calls that overlap on the GPU (other streams, other host
 * threads) race; serialise them.  The first call on each device looks up the
 * array's device address (cudaGetSymbolAddress, with that device current);
 * make that first call before any stream capture.  msg (may be NULL) receives
 * a message on failure. */
int mq_fock_rhf_noalloc(int n, const double *d_XX, const double *d_D, double *d_G, void *stream, char *msg,
                        int msglen);

/* Direct Fock build: integrals recomputed and digested in one kernel, no
 * stored XX (the (H2O)64-scale path).  Same meaning as mq_fock. */
int mq_fock_direct(mq_ctx *ctx, const double *Da, const double *Db, double *Ga, double *Gb);

/* SCF options (zero-initialise, then set what you need). */
typedef struct mq_scf_opts {
  int uhf;          /* 0 RHF, 1 UHF (options(3), src/parser/parser.f90:25) */
  int nalpha;       /* nelcA */
  int nbeta;        /* nelcB */
  int max_iter;     /* 0 -> 500 RHF / 300 UHF (src/scf/scf.f90:172,337) */
  double conv;      /* density threshold; 0 -> 1e-7 (options(8)=7) */
  int conv_rms;     /* 0: max|D_new-D_old| (the reference, scf.f90:1227-1258);
                       1: RMS of D_new-D_old */
  int diis;         /* 0: plain Roothaan like the reference; >0: DIIS subspace */
  int direct;       /* 0: digest the device-resident XX; 1: direct Fock build */
  int guess;        /* 0: core Hamiltonian (scf.f90:410-512); 1: use C_in;
                       2: use D_in (density guess, e.g. the learned guess) */
  const double *C_in;   /* guess orbitals, n x n (x2 for UHF) */
  const double *D_in;   /* guess density, n x n (x2 for UHF: alpha, beta) */
  int purify;       /* 0: new density from the eigenvectors each iteration (the
                       reference's DSYGV step); 1: from the spectral projector
                       by trace-correcting purification (GEMMs only), one
                       eigensolve at the end for C and eps; an iteration whose
                       frontier levels are degenerate falls back to the
                       eigensolver.  Same fixed point either way. */
} mq_scf_opts;

/* Converged SCF.  Replaces the scf executable's iteration loop
 * (src/scf/scf.f90:61-404, RHFiter :720-904, UHFiter :909-1117) including the
 * dens and RHFI2G/UHFI2G child processes it spawns each iteration.
 *   S, H     n x n host arrays (Suv, Huv)
 *   C        out, n x n (RHF) or 2 x n x n (UHF alpha then beta), C^T S C = 1
 *   eps      out, n (RHF) or 2n (UHF), ascending
 *   D        out (may be NULL), the last input density(ies) n x n (x2)
 *   energy   out, total SCF energy of the last iteration's input density,
 *            as the reference prints it (scf.f90:900)
 *   iters    out, iterations taken
 *   history  out (may be NULL), 2*max_iter doubles: (E_k, maxdiff_k) */
int mq_scf(mq_ctx *ctx, const double *S, const double *H, const mq_scf_opts *opts, double *C, double *eps,
           double *D, double *energy, int *iters, double *history);

/* Precision of the four-index transform */
#define MQ_PREC_FP64 0      /* plain FP64 GEMMs */
#define MQ_PREC_SPLIT_BF16 1   /* hi+lo BF16 operands on tcgen05 tensor cores,
                                  3 MMAs per K step, FP32 accumulation
                                  (~16-bit operands) */
#define MQ_PREC_SPLIT_BF16X3 2 /* hi+mid+lo BF16 operands, 6 MMAs per K step,
                                  FP32 accumulation (~24-bit operands) */

/* (ia|jb) block, Om(i,a,j,b) with i fastest (ao2mo.f90:465-602 and the
 * idx1..idx4_trans quarter transforms :1306-1439).  Ci: n x no1, Ca: n x nv1,
 * Cj: n x no2, Cb: n x nv2 column-major (leading dimension n).  out is a host
 * buffer of no1*nv1*no2*nv2 doubles, or NULL to keep it on the device for
 * mq_mp2_energy. */
int mq_ao2mo_iajb(mq_ctx *ctx, const double *Ci, int no1, const double *Ca, int nv1, const double *Cj, int no2,
                  const double *Cb, int nv2, int precision, double *out);

/* RHF MP2 from the device-resident (ia|jb) of the last mq_ao2mo_iajb call:
 * e_out[0] = E(AA) = sum_{i<j,a<b}[(ia|jb)-(ib|ja)]^2/D,
 * e_out[1] = E(AB) = sum_{ijab}(ia|jb)^2/D, e_out[2] = E(MBPT2) = 2*E(AA)+E(AB)
 * (src/mp2/mp2.f90:79-144).  eig: n orbital energies. */
int mq_mp2_rhf(mq_ctx *ctx, const double *eig, int nocc, int nvir, double *e_out);

/* UHF MP2 (src/mp2/mp2.f90:154-232 with ao2mo.f90:614-904): CA, CB n x n,
 * eA, eB n.  e_out = {E(AA), E(BB), E(AB), E(MBPT2)}. */
int mq_mp2_uhf(mq_ctx *ctx, const double *CA, const double *CB, const double *eA, const double *eB, int noA,
               int noB, int precision, double *e_out);

/* MP2 pair sums of a given (ia|jb) block (host array, i fastest, as
 * mq_ao2mo_iajb returns it), e.g. the records of the ijab_* files that
 * src/mp2/mp2.f90:79-232 reads: e1 = energies of the first pair's occupied
 * then virtual orbitals (no1 + nv1), e2 likewise.  e_out[0] =
 * sum_{ijab} (ia|jb)^2 / D; e_out[1] = sum_{i<j, a<b} [(ia|jb) - (ib|ja)]^2 / D
 * when same_spin (else 0), D = e_i + e_j - e_a - e_b.  No system is needed. */
int mq_mp2_pairs(mq_ctx *ctx, const double *iajb, int no1, int nv1, int no2, int nv2, const double *e1,
                 const double *e2, int same_spin, double *e_out);

/* Batched symmetric eigensolver (FP64 Jacobi): `batch` matrices of order n,
 * A (n*n each, column-major, overwritten) -> eigenvalues w (ascending, n each)
 * and eigenvectors V (n*n each).  Replaces DSYEV/DSYGV's eigen step
 * (src/scf/scf.f90:692,848). */
int mq_syev_batched(mq_ctx *ctx, int n, int batch, double *A, double *w, double *V);

/* C = alpha op(A) op(B) + beta C on the device, host arrays column-major
 * (BLAS DGEMM semantics; transa/transb 'N' or 'T'), e.g. the DGEMM products of
 * the reference's SCF (src/scf/scf.f90:1306-1307).  Orders up to ~1000 run
 * on the library's own FP64 kernel spread over all SMs. */
int mq_dgemm(mq_ctx *ctx, char transa, char transb, int m, int n, int k, double alpha, const double *A, int lda,
             const double *B, int ldb, double beta, double *C, int ldc);

/* Generalized problem F C = S C eps (DSYGV itype 1, 'V', 'L',
 * src/scf/scf.f90:478,848) for one n x n pair of host matrices. */
int mq_sygv(mq_ctx *ctx, int n, const double *F, const double *S, double *w, double *C);

/* ---- Batches of independent closed-shell molecules (no reference
 * counterpart: the reference runs one molecule per invocation of scf,
 * src/scf/scf.f90:61-216).  Molecules of uneven size (at most 116 basis
 * functions each) are added one by one with the arrays buildBasis returns,
 * then solved together: integrals, Fock builds and the dense per-molecule
 * steps of every molecule share each launch, and one SCF iteration is a CUDA
 * graph replayed until every molecule has converged.  Integrals use
 * MQ_MODE_TIGHT.  Per molecule the iteration and convergence rule are those of
 * mq_scf (RHF).  Packed arrays hold molecule m's n_m x n_m block (column-major)
 * after those of molecules 0..m-1; vectors likewise. */
typedef struct mq_batch_opts {
  int max_iter;        /* 0 -> 500 */
  double conv;         /* density threshold; 0 -> 1e-7 */
  int conv_rms;        /* 0: max|dD|; 1: RMS */
  int diis;            /* 0: plain Roothaan; >0: DIIS subspace (<= 16) */
  int graph;           /* 1: replay one captured iteration as a CUDA graph */
  int check_every;     /* poll the count of unconverged molecules every k iterations (0 -> 4) */
  const double *D_in;  /* packed guess densities, or NULL for the core-Hamiltonian guess;
                          a block whose first element is NaN takes the core guess */
} mq_batch_opts;

/* The learned initial density (no reference counterpart; the reference starts
 * from the core Hamiltonian, src/scf/scf.f90:410-512).  mq_guess_model loads the
 * network (nin = 64 descriptors, width, nout = 25 block entries; params as
 * mq_mlp_set_params takes them) and its standardisation: mu_x, sd_x (64 each)
 * and mu_y, sd_y (5 block types x 25).  mq_guess_predict forms, on the GPU, the
 * pair descriptors of nmol molecules (nnuc[m] atoms each, concatenated: Z, and
 * xyz in bohr as xyz(0:N-1, 0:2) column-major over all N atoms), runs the
 * network and assembles each
 * molecule's predicted density (n x n, concatenated in order) into D.  A
 * batched SCF given these densities checks each one (electron count, idempotency)
 * and keeps the core guess where a check fails. */
int mq_guess_model(mq_ctx *ctx, int nin, int width, int nout, const float *params, const double *mu_x,
                   const double *sd_x, const double *mu_y, const double *sd_y);
int mq_guess_predict(mq_ctx *ctx, int nmol, const int *nnuc, const int *Z, const double *xyz, double *D);

/* The basis library (the text of a mybasis file) kept by the context for the
 * calls below; its STO-3G section is used, as the reference's buildBasis
 * reads it (src/myQC/basis.f90:81). */
int mq_basis_library(mq_ctx *ctx, const char *text);

/* buildBasis (src/myQC/basis.f90:23-226) in the library: the flat bas, set,
 * basinfo and setinfo arrays of the atoms Z[nnuc] from the library above.
 * sizes[4]: on entry the capacities of the four arrays, on return the sizes
 * needed; the arrays are written only when all four fit (null arrays: sizes
 * only). */
int mq_basis_build(mq_ctx *ctx, int nnuc, const int *Z, double *bas, double *set, int *basinfo, int *setinfo,
                   int sizes[4]);

/* mq_batch_add with the molecule's basis built by the library (mq_basis_library
 * first): nuclei Z and coordinates xyz (bohr, xyz(0:nnuc-1, 0:2) column-major
 * as mq_batch_add takes them), nocc doubly occupied orbitals. */
int mq_batch_add_atoms(mq_ctx *ctx, int nnuc, const int *Z, const double *xyz, int nocc);

/* Empty the context's batch. */
int mq_batch_clear(mq_ctx *ctx);

/* Append one closed-shell molecule with nocc doubly occupied orbitals. */
int mq_batch_add(mq_ctx *ctx, int nnuc, const int *Z, const double *xyz, const double *bas, const double *set,
                 const int *basinfo, const int *setinfo, int nocc);

/* Number of molecules, and (norb may be NULL) each one's basis size. */
int mq_batch_info(const mq_ctx *ctx, int *nmol, int *norb);

/* Solve every molecule of the batch.  energy, iters, converged: one entry per
 * molecule (E of the last iteration's input density; iterations taken;
 * 1 if converged).  D (may be NULL): packed last input densities; eps (may be
 * NULL): packed orbital energies of the last diagonalisation. */
int mq_batch_scf(mq_ctx *ctx, const mq_batch_opts *opts, double *energy, int *iters, int *converged, double *D,
                 double *eps);

/* ---- The learned density guess's network (no reference counterpart).  A
 * 3-layer MLP nin -> width -> width -> nout with SiLU activations, BF16
 * weights and activations and FP32 accumulation on the tensor cores, trained
 * by Adam on the device.  One network per context.  Parameters are packed as
 * FP32: W1 [width][nin], b1, W2 [width][width], b2, W3 [nout][width], b3.
 * Rows of X (nin floats), T and W (nout floats) are samples. */
int mq_mlp_init(mq_ctx *ctx, int nin, int width, int nout); /* width, nout <= 256; nin % 8 == 0 */
int mq_mlp_param_count(mq_ctx *ctx, int *n);
int mq_mlp_set_params(mq_ctx *ctx, const float *params);   /* also resets the Adam moments */
int mq_mlp_get_params(mq_ctx *ctx, float *params);
int mq_mlp_forward(mq_ctx *ctx, int rows, const float *X, float *Y);
/* Loss sum W (Y - T)^2 / sum W over the rows and its gradient (packed like the parameters). */
int mq_mlp_grad(mq_ctx *ctx, int rows, const float *X, const float *T, const float *W, float *grads, double *loss);
/* Training set kept on the device, then one epoch of Adam minibatches in the order perm (a
 * permutation of 0..n-1); batch a multiple of 128; mean minibatch loss to *loss. */
int mq_mlp_set_data(mq_ctx *ctx, long long n, const float *X, const float *T, const float *W);
int mq_mlp_train_epoch(mq_ctx *ctx, const int *perm, int batch, float lr, double *loss);

/* Profiling counters.  Device milliseconds (CUDA events on the context's
 * stream) of the last call of each stage: "eri", "ao2mo", "mp2", "scf" (whole
 * SCF), "fock" and "diag" (summed over the last SCF's iterations; "diag" is
 * the density step, eigensolver or purification), "fock_kernel" (the stored
 * digestion kernel alone) with "fock_kernel_launches"; "fock_calls",
 * "scf_iters", "diag_calls" (eigensolves), "purify_steps"; "fock_jc" (tile
 * length the autotuner picked) and "tune_fock_ms" (its best time per build);
 * cumulative launch counts "launches" (this library's kernels) and
 * "lib_launches" (cuBLAS calls); "quartets" and "prim_quartets" of the last
 * integral pass.  MQ_EINVAL on an unknown key. */
int mq_stat(const mq_ctx *ctx, const char *key, double *value);

#ifdef __cplusplus
}
#endif
#endif /* MYQC_H */
