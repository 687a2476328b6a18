! myqc_gpu.f90 -- iso_c_binding interface module of libmyqc for the
! reference's Fortran programs: one BIND(C) interface per function of
! include/myqc.h, with the status codes and option structures.  Compile it
! with the host program and link libmyqc.so; a nonzero status maps to the
! reference's failure path (touch error, then STOP).
MODULE myqc_gpu
  USE iso_c_binding
  IMPLICIT NONE
  INTEGER(c_int), PARAMETER :: MQ_OK = 0, MQ_MODE_REFERENCE = 0, MQ_MODE_TIGHT = 1
  INTEGER(c_int), PARAMETER :: MQ_STORE_FULL = 0, MQ_STORE_QUARTETS = 1
  INTEGER(c_int), PARAMETER :: MQ_PREC_FP64 = 0, MQ_PREC_SPLIT_BF16 = 1, MQ_PREC_SPLIT_BF16X3 = 2

  TYPE, BIND(C) :: mq_scf_opts
    INTEGER(c_int) :: uhf, nalpha, nbeta, max_iter
    REAL(c_double) :: conv
    INTEGER(c_int) :: conv_rms, diis, direct, guess
    TYPE(c_ptr)    :: C_in, D_in
    INTEGER(c_int) :: purify
  END TYPE

  TYPE, BIND(C) :: mq_batch_opts
    INTEGER(c_int) :: max_iter
    REAL(c_double) :: conv
    INTEGER(c_int) :: conv_rms, diis, graph, check_every
    TYPE(c_ptr)    :: D_in
  END TYPE

  INTERFACE
    INTEGER(c_int) FUNCTION mq_init(ctx, device) BIND(C)
      IMPORT; TYPE(c_ptr) :: ctx; INTEGER(c_int), VALUE :: device
    END FUNCTION
    INTEGER(c_int) FUNCTION mq_free(ctx) BIND(C)
      IMPORT; TYPE(c_ptr), VALUE :: ctx
    END FUNCTION
    INTEGER(c_int) FUNCTION mq_last_error(ctx, buf, len) BIND(C)
      IMPORT; TYPE(c_ptr), VALUE :: ctx; CHARACTER(c_char) :: buf(*); INTEGER(c_int), VALUE :: len
    END FUNCTION
    INTEGER(c_int) FUNCTION mq_set_system(ctx, nnuc, Z, xyz, bas, set, basinfo, setinfo, ftab, mode) BIND(C)
      IMPORT; TYPE(c_ptr), VALUE :: ctx; INTEGER(c_int), VALUE :: nnuc, mode
      INTEGER(c_int) :: Z(*), basinfo(*), setinfo(*)
      REAL(c_double) :: xyz(*), bas(*), set(*), ftab(*)
    END FUNCTION
    INTEGER(c_int) FUNCTION mq_norb(ctx, norb) BIND(C)
      IMPORT; TYPE(c_ptr), VALUE :: ctx; INTEGER(c_int) :: norb
    END FUNCTION
    INTEGER(c_int) FUNCTION mq_set_schwarz(ctx, thr) BIND(C)
      IMPORT; TYPE(c_ptr), VALUE :: ctx; REAL(c_double), VALUE :: thr
    END FUNCTION
    INTEGER(c_int) FUNCTION mq_set_fock_precision(ctx, precision) BIND(C)
      IMPORT; TYPE(c_ptr), VALUE :: ctx; INTEGER(c_int), VALUE :: precision
    END FUNCTION
    INTEGER(c_int) FUNCTION mq_set_fock_incremental(ctx, tau) BIND(C)
      IMPORT; TYPE(c_ptr), VALUE :: ctx; REAL(c_double), VALUE :: tau
    END FUNCTION
    INTEGER(c_int) FUNCTION mq_set_ao2mo_prefetch(ctx, planes) BIND(C)
      IMPORT; TYPE(c_ptr), VALUE :: ctx; INTEGER(c_int), VALUE :: planes
    END FUNCTION
    INTEGER(c_int) FUNCTION mq_set_eri_mixed(ctx, tau) BIND(C)
      IMPORT; TYPE(c_ptr), VALUE :: ctx; REAL(c_double), VALUE :: tau
    END FUNCTION
    INTEGER(c_int) FUNCTION mq_probe_fp64(ctx, tflops) BIND(C)
      IMPORT; TYPE(c_ptr), VALUE :: ctx; REAL(c_double) :: tflops
    END FUNCTION
    INTEGER(c_int) FUNCTION mq_set_partition(ctx, part, nparts) BIND(C)
      IMPORT; TYPE(c_ptr), VALUE :: ctx; INTEGER(c_int), VALUE :: part, nparts
    END FUNCTION
    INTEGER(c_int) FUNCTION mq_set_eri_storage(ctx, storage) BIND(C)
      IMPORT; TYPE(c_ptr), VALUE :: ctx; INTEGER(c_int), VALUE :: storage   ! MQ_STORE_FULL / MQ_STORE_QUARTETS
    END FUNCTION
    INTEGER(c_int) FUNCTION mq_set_fock_screened_increments(ctx, tau) BIND(C)
      IMPORT; TYPE(c_ptr), VALUE :: ctx; REAL(c_double), VALUE :: tau
    END FUNCTION
    INTEGER(c_int) FUNCTION mq_guess_model(ctx, nin, width, nout, params, mu_x, sd_x, mu_y, sd_y) BIND(C)
      IMPORT; TYPE(c_ptr), VALUE :: ctx; INTEGER(c_int), VALUE :: nin, width, nout; REAL(c_float) :: params(*)
      REAL(c_double) :: mu_x(*), sd_x(*), mu_y(*), sd_y(*)
    END FUNCTION
    INTEGER(c_int) FUNCTION mq_guess_predict(ctx, nmol, nnuc, Z, xyz, D) BIND(C)
      IMPORT; TYPE(c_ptr), VALUE :: ctx; INTEGER(c_int), VALUE :: nmol; INTEGER(c_int) :: nnuc(*), Z(*)
      REAL(c_double) :: xyz(*), D(*)
    END FUNCTION
    INTEGER(c_int) FUNCTION mq_basis_library(ctx, text) BIND(C)
      IMPORT; TYPE(c_ptr), VALUE :: ctx; CHARACTER(KIND=c_char) :: text(*)   ! NUL-terminated mybasis text
    END FUNCTION
    INTEGER(c_int) FUNCTION mq_basis_build(ctx, nnuc, Z, bas, set, basinfo, setinfo, sizes) BIND(C)
      IMPORT; TYPE(c_ptr), VALUE :: ctx; INTEGER(c_int), VALUE :: nnuc; INTEGER(c_int) :: Z(*)
      REAL(c_double) :: bas(*), set(*); INTEGER(c_int) :: basinfo(*), setinfo(*), sizes(4)
    END FUNCTION
    INTEGER(c_int) FUNCTION mq_batch_add_atoms(ctx, nnuc, Z, xyz, nocc) BIND(C)
      IMPORT; TYPE(c_ptr), VALUE :: ctx; INTEGER(c_int), VALUE :: nnuc, nocc; INTEGER(c_int) :: Z(*)
      REAL(c_double) :: xyz(*)
    END FUNCTION
    INTEGER(c_int) FUNCTION mq_set_eri_tuning(ctx, mode) BIND(C)
      IMPORT; TYPE(c_ptr), VALUE :: ctx; INTEGER(c_int), VALUE :: mode
    END FUNCTION
    INTEGER(c_int) FUNCTION mq_eri_tuning_report(ctx, buf, len) BIND(C)
      IMPORT; TYPE(c_ptr), VALUE :: ctx; CHARACTER(KIND=c_char) :: buf(*); INTEGER(c_int), VALUE :: len
    END FUNCTION
    INTEGER(c_int) FUNCTION mq_int1e(ctx, S, H) BIND(C)
      IMPORT; TYPE(c_ptr), VALUE :: ctx; REAL(c_double) :: S(*), H(*)
    END FUNCTION
    INTEGER(c_int) FUNCTION mq_int1p(ctx, Px) BIND(C)
      IMPORT; TYPE(c_ptr), VALUE :: ctx; REAL(c_double) :: Px(*)   ! x, y, z n x n matrices in turn
    END FUNCTION
    INTEGER(c_int) FUNCTION mq_eri_full(ctx, XX) BIND(C)
      IMPORT; TYPE(c_ptr), VALUE :: ctx; REAL(c_double) :: XX(*)
    END FUNCTION
    INTEGER(c_int) FUNCTION mq_eri_store(ctx) BIND(C)
      IMPORT; TYPE(c_ptr), VALUE :: ctx
    END FUNCTION
    INTEGER(c_int) FUNCTION mq_eri_upload(ctx, XX) BIND(C)
      IMPORT; TYPE(c_ptr), VALUE :: ctx; REAL(c_double) :: XX(*)
    END FUNCTION
    INTEGER(c_int) FUNCTION mq_fock(ctx, Da, Db, Ga, Gb) BIND(C)
      IMPORT; TYPE(c_ptr), VALUE :: ctx, Db, Gb   ! c_null_ptr for RHF
      REAL(c_double) :: Da(*), Ga(*)
    END FUNCTION
    INTEGER(c_int) FUNCTION mq_fock_direct(ctx, Da, Db, Ga, Gb) BIND(C)
      IMPORT; TYPE(c_ptr), VALUE :: ctx, Db, Gb
      REAL(c_double) :: Da(*), Ga(*)
    END FUNCTION
    INTEGER(c_int) FUNCTION mq_scf(ctx, S, H, opts, C, eps, D, energy, iters, history) BIND(C)
      IMPORT; TYPE(c_ptr), VALUE :: ctx, D, history
      REAL(c_double) :: S(*), H(*), C(*), eps(*), energy
      TYPE(mq_scf_opts) :: opts; INTEGER(c_int) :: iters
    END FUNCTION
    INTEGER(c_int) FUNCTION mq_ao2mo_iajb(ctx, Ci, no1, Ca, nv1, Cj, no2, Cb, nv2, precision, out) BIND(C)
      IMPORT; TYPE(c_ptr), VALUE :: ctx, out       ! c_null_ptr: keep (ia|jb) on the device
      REAL(c_double) :: Ci(*), Ca(*), Cj(*), Cb(*)
      INTEGER(c_int), VALUE :: no1, nv1, no2, nv2, precision
    END FUNCTION
    INTEGER(c_int) FUNCTION mq_mp2_rhf(ctx, eig, nocc, nvir, e_out) BIND(C)
      IMPORT; TYPE(c_ptr), VALUE :: ctx; REAL(c_double) :: eig(*), e_out(3)
      INTEGER(c_int), VALUE :: nocc, nvir
    END FUNCTION
    INTEGER(c_int) FUNCTION mq_mp2_uhf(ctx, CA, CB, eA, eB, noA, noB, precision, e_out) BIND(C)
      IMPORT; TYPE(c_ptr), VALUE :: ctx; REAL(c_double) :: CA(*), CB(*), eA(*), eB(*), e_out(4)
      INTEGER(c_int), VALUE :: noA, noB, precision
    END FUNCTION
    INTEGER(c_int) FUNCTION mq_syev_batched(ctx, n, batch, A, w, V) BIND(C)
      IMPORT; TYPE(c_ptr), VALUE :: ctx; INTEGER(c_int), VALUE :: n, batch
      REAL(c_double) :: A(*), w(*), V(*)
    END FUNCTION
    INTEGER(c_int) FUNCTION mq_sygv(ctx, n, F, S, w, C) BIND(C)
      IMPORT; TYPE(c_ptr), VALUE :: ctx; INTEGER(c_int), VALUE :: n
      REAL(c_double) :: F(*), S(*), w(*), C(*)
    END FUNCTION
    INTEGER(c_int) FUNCTION mq_stat(ctx, key, value) BIND(C)
      IMPORT; TYPE(c_ptr), VALUE :: ctx; CHARACTER(c_char) :: key(*); REAL(c_double) :: value
    END FUNCTION
    TYPE(c_ptr) FUNCTION mq_version() BIND(C)
      IMPORT
    END FUNCTION
    INTEGER(c_int) FUNCTION mq_mp2_pairs(ctx, iajb, no1, nv1, no2, nv2, e1, e2, same_spin, e_out) BIND(C)
      IMPORT; TYPE(c_ptr), VALUE :: ctx; INTEGER(c_int), VALUE :: no1, nv1, no2, nv2, same_spin
      REAL(c_double) :: iajb(*), e1(*), e2(*), e_out(2)
    END FUNCTION
    INTEGER(c_int) FUNCTION mq_dgemm(ctx, transa, transb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc) BIND(C)
      IMPORT; TYPE(c_ptr), VALUE :: ctx; CHARACTER(c_char), VALUE :: transa, transb
      INTEGER(c_int), VALUE :: m, n, k, lda, ldb, ldc; REAL(c_double), VALUE :: alpha, beta
      REAL(c_double) :: A(*), B(*), C(*)
    END FUNCTION
    INTEGER(c_int) FUNCTION mq_batch_clear(ctx) BIND(C)
      IMPORT; TYPE(c_ptr), VALUE :: ctx
    END FUNCTION
    INTEGER(c_int) FUNCTION mq_batch_add(ctx, nnuc, Z, xyz, bas, set, basinfo, setinfo, nocc) BIND(C)
      IMPORT; TYPE(c_ptr), VALUE :: ctx; INTEGER(c_int), VALUE :: nnuc, nocc
      INTEGER(c_int) :: Z(*), basinfo(*), setinfo(*)
      REAL(c_double) :: xyz(*), bas(*), set(*)
    END FUNCTION
    INTEGER(c_int) FUNCTION mq_batch_info(ctx, nmol, norb) BIND(C)
      IMPORT; TYPE(c_ptr), VALUE :: ctx; INTEGER(c_int) :: nmol, norb(*)
    END FUNCTION
    INTEGER(c_int) FUNCTION mq_batch_scf(ctx, opts, energy, iters, converged, D, eps) BIND(C)
      IMPORT; TYPE(c_ptr), VALUE :: ctx; TYPE(mq_batch_opts) :: opts
      REAL(c_double) :: energy(*), D(*), eps(*); INTEGER(c_int) :: iters(*), converged(*)
    END FUNCTION
    INTEGER(c_int) FUNCTION mq_mlp_init(ctx, nin, width, nout) BIND(C)
      IMPORT; TYPE(c_ptr), VALUE :: ctx; INTEGER(c_int), VALUE :: nin, width, nout
    END FUNCTION
    INTEGER(c_int) FUNCTION mq_mlp_param_count(ctx, n) BIND(C)
      IMPORT; TYPE(c_ptr), VALUE :: ctx; INTEGER(c_int) :: n
    END FUNCTION
    INTEGER(c_int) FUNCTION mq_mlp_set_params(ctx, params) BIND(C)
      IMPORT; TYPE(c_ptr), VALUE :: ctx; REAL(c_float) :: params(*)
    END FUNCTION
    INTEGER(c_int) FUNCTION mq_mlp_get_params(ctx, params) BIND(C)
      IMPORT; TYPE(c_ptr), VALUE :: ctx; REAL(c_float) :: params(*)
    END FUNCTION
    INTEGER(c_int) FUNCTION mq_mlp_forward(ctx, rows, X, Y) BIND(C)
      IMPORT; TYPE(c_ptr), VALUE :: ctx; INTEGER(c_int), VALUE :: rows; REAL(c_float) :: X(*), Y(*)
    END FUNCTION
    INTEGER(c_int) FUNCTION mq_mlp_grad(ctx, rows, X, T, W, grads, loss) BIND(C)
      IMPORT; TYPE(c_ptr), VALUE :: ctx; INTEGER(c_int), VALUE :: rows
      REAL(c_float) :: X(*), T(*), W(*), grads(*); REAL(c_double) :: loss
    END FUNCTION
    INTEGER(c_int) FUNCTION mq_mlp_set_data(ctx, n, X, T, W) BIND(C)
      IMPORT; TYPE(c_ptr), VALUE :: ctx; INTEGER(c_long_long), VALUE :: n
      REAL(c_float) :: X(*), T(*), W(*)
    END FUNCTION
    INTEGER(c_int) FUNCTION mq_mlp_train_epoch(ctx, perm, batch, lr, loss) BIND(C)
      IMPORT; TYPE(c_ptr), VALUE :: ctx; INTEGER(c_int) :: perm(*); INTEGER(c_int), VALUE :: batch
      REAL(c_float), VALUE :: lr; REAL(c_double) :: loss
    END FUNCTION
    INTEGER(c_int) FUNCTION mq_fock_rhf_noalloc(n, d_XX, d_D, d_G, stream, msg, msglen) BIND(C)
      IMPORT; INTEGER(c_int), VALUE :: n, msglen
      TYPE(c_ptr), VALUE :: d_XX, d_D, d_G, stream
      CHARACTER(c_char) :: msg(*)
    END FUNCTION
  END INTERFACE
END MODULE
