"""Python host over the C ABI: one ``Context`` per GPU, mirroring the stages of
the reference's executables (int1e, int2e, scf with dens + RHFI2G/UHFI2G,
ao2mo, mp2) as method calls on device-resident data."""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import MODE_REFERENCE, MODE_TIGHT, PREC_FP64, PREC_SPLIT_BF16, MyQCError, f64, ptr
from .formats import BasisArrays, System


@dataclass
class SCFResult:
    energy: float
    eig: np.ndarray      # (n,) RHF or (2, n) UHF
    C: np.ndarray        # (n, n) RHF or (2, n, n) UHF, column-major orbitals
    D: np.ndarray        # last input density (total for RHF; alpha, beta for UHF)
    iterations: int
    history: np.ndarray  # (iterations, 2): energy, max|dD|


class Context:
    def __init__(self, device: int = 0):
        self.L = _lib.lib()
        h = ctypes.c_void_p()
        rc = self.L.mq_init(ctypes.byref(h), device)
        if rc != 0:
            raise MyQCError(rc, "mq_init failed (no CUDA device?)")
        self.h = h
        self.n = 0

    def close(self):
        if getattr(self, "h", None):
            self.L.mq_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc: int):
        if rc != 0:
            buf = ctypes.create_string_buffer(512)
            self.L.mq_last_error(self.h, buf, 512)
            raise MyQCError(rc, buf.value.decode())

    # ---------------------------------------------------------------- setup
    def set_system(self, sysm: System, basis: BasisArrays, ftab: np.ndarray | None = None,
                   mode: int = MODE_REFERENCE):
        Z = np.ascontiguousarray(sysm.atoms, dtype=np.int32)
        xyz = f64(np.asarray(sysm.xyz).reshape(-1, 3))  # Fortran xyz(0:nnuc-1,0:2)
        self._keep = (Z, xyz, np.ascontiguousarray(basis.bas, dtype=np.float64),
                      np.ascontiguousarray(basis.set, dtype=np.float64),
                      np.ascontiguousarray(basis.basinfo, dtype=np.int32),
                      np.ascontiguousarray(basis.setinfo, dtype=np.int32),
                      None if ftab is None else np.ascontiguousarray(ftab, dtype=np.float64))
        k = self._keep
        self._check(self.L.mq_set_system(self.h, len(Z), ptr(k[0]), ptr(k[1]), ptr(k[2]), ptr(k[3]), ptr(k[4]),
                                         ptr(k[5]), ptr(k[6]), mode))
        n = ctypes.c_int()
        self._check(self.L.mq_norb(self.h, ctypes.byref(n)))
        self.n = n.value
        self.sys = sysm

    # ---------------------------------------------------------------- batches
    def batch_clear(self):
        self._check(self.L.mq_batch_clear(self.h))

    def batch_add(self, sysm: System, basis: BasisArrays):
        """Append one closed-shell molecule (nelcA doubly occupied orbitals)."""
        if sysm.nelcA != sysm.nelcB:
            raise ValueError("batches hold closed-shell molecules")
        Z = np.ascontiguousarray(sysm.atoms, dtype=np.int32)
        xyz = f64(np.asarray(sysm.xyz).reshape(-1, 3))
        k = (Z, xyz, np.ascontiguousarray(basis.bas, dtype=np.float64),
             np.ascontiguousarray(basis.set, dtype=np.float64), np.ascontiguousarray(basis.basinfo, dtype=np.int32),
             np.ascontiguousarray(basis.setinfo, dtype=np.int32))
        self._check(self.L.mq_batch_add(self.h, len(Z), ptr(k[0]), ptr(k[1]), ptr(k[2]), ptr(k[3]), ptr(k[4]),
                                        ptr(k[5]), sysm.nelcA))

    def guess_model(self, dims, params, mu_x, sd_x, mu_y, sd_y):
        """Load the learned guess's network (dims nin, width, width, nout) and its
        feature / output standardisation."""
        P = np.ascontiguousarray(params, dtype=np.float32)
        arrs = [f64(np.asarray(a).ravel()) for a in (mu_x, sd_x, mu_y, sd_y)]
        self._check(self.L.mq_guess_model(self.h, int(dims[0]), int(dims[1]), int(dims[3]), ptr(P),
                                          *[ptr(a) for a in arrs]))
        self.mlp_dims = (int(dims[0]), int(dims[1]), int(dims[2]), int(dims[3]))

    def guess_predict(self, systems) -> list:
        """Predicted densities of the systems (one GPU pass for all of them)."""
        nnuc = np.array([len(s.atoms) for s in systems], dtype=np.int32)
        Z = np.ascontiguousarray(np.concatenate([np.asarray(s.atoms) for s in systems]), dtype=np.int32)
        xyz = f64(np.concatenate([np.asarray(s.xyz, dtype=float).reshape(-1, 3) for s in systems]))
        sizes = [int(sum(1 if z <= 2 else 5 for z in s.atoms)) for s in systems]
        D = np.zeros(sum(n * n for n in sizes))
        self._check(self.L.mq_guess_predict(self.h, len(systems), ptr(nnuc), ptr(Z), ptr(xyz), ptr(D)))
        out, o = [], 0
        for n in sizes:
            out.append(D[o: o + n * n].reshape(n, n, order="F"))
            o += n * n
        return out

    def basis_library(self, text: str):
        """Keep the mybasis text in the library (its STO-3G section) for
        basis_build and batch_add_atoms."""
        self._check(self.L.mq_basis_library(self.h, text.encode()))

    def basis_build(self, atoms) -> BasisArrays:
        """buildBasis in the library: the bas / set / basinfo / setinfo arrays of the atoms."""
        Z = np.ascontiguousarray(atoms, dtype=np.int32)
        sizes = np.zeros(4, dtype=np.int32)
        self._check(self.L.mq_basis_build(self.h, len(Z), ptr(Z), None, None, None, None, ptr(sizes)))
        bas, st = np.zeros(int(sizes[0])), np.zeros(int(sizes[1]))
        bi, si = np.zeros(int(sizes[2]), dtype=np.int32), np.zeros(int(sizes[3]), dtype=np.int32)
        self._check(self.L.mq_basis_build(self.h, len(Z), ptr(Z), ptr(bas), ptr(st), ptr(bi), ptr(si), ptr(sizes)))
        return BasisArrays(bas=bas, set=st, basinfo=bi, setinfo=si)

    def batch_add_atoms(self, sysm: System):
        """batch_add with the basis built by the library (basis_library first)."""
        if sysm.nelcA != sysm.nelcB:
            raise ValueError("batches hold closed-shell molecules")
        Z = np.ascontiguousarray(sysm.atoms, dtype=np.int32)
        xyz = f64(np.asarray(sysm.xyz).reshape(-1, 3))
        self._check(self.L.mq_batch_add_atoms(self.h, len(Z), ptr(Z), ptr(xyz), sysm.nelcA))

    def batch_sizes(self) -> np.ndarray:
        nm = ctypes.c_int()
        self._check(self.L.mq_batch_info(self.h, ctypes.byref(nm), None))
        out = np.zeros(nm.value, dtype=np.int32)
        self._check(self.L.mq_batch_info(self.h, ctypes.byref(nm), ptr(out)))
        return out

    def batch_scf(self, conv: float = 1e-7, conv_rms: bool = False, diis: int = 0, max_iter: int = 0,
                  graph: bool = True, check_every: int = 4, D_guess=None):
        """Solve the batch.  D_guess: list of n x n arrays (None entries take the
        core guess).  Returns dict with energy, iterations, converged, D, eps
        (lists of per-molecule arrays)."""
        sizes = self.batch_sizes()
        M = len(sizes)
        mat = np.concatenate([[0], np.cumsum(sizes.astype(np.int64) ** 2)])
        vec = np.concatenate([[0], np.cumsum(sizes.astype(np.int64))])
        o = _lib.BatchOpts()
        o.max_iter, o.conv, o.conv_rms, o.diis = max_iter, conv, int(conv_rms), diis
        o.graph, o.check_every = int(graph), check_every
        keep = None
        if D_guess is not None:
            keep = np.empty(int(mat[-1]))
            for m in range(M):
                g = D_guess[m]
                if g is None:
                    keep[mat[m]] = np.nan
                else:
                    keep[mat[m]:mat[m + 1]] = np.asarray(g, dtype=np.float64).reshape(-1, order="F")
            o.D_in = keep.ctypes.data
        E = np.zeros(M)
        it = np.zeros(M, dtype=np.int32)
        cv = np.zeros(M, dtype=np.int32)
        D = np.zeros(int(mat[-1]))
        eps = np.zeros(int(vec[-1]))
        self._check(self.L.mq_batch_scf(self.h, ctypes.byref(o), ptr(E), ptr(it), ptr(cv), ptr(D), ptr(eps)))
        Ds = [D[mat[m]:mat[m + 1]].reshape(sizes[m], sizes[m], order="F") for m in range(M)]
        es = [eps[vec[m]:vec[m + 1]].copy() for m in range(M)]
        return {"energy": E, "iterations": it, "converged": cv.astype(bool), "D": Ds, "eps": es}

    # ---------------------------------------------------------------- learned-guess network
    def mlp_init(self, nin: int, width: int, nout: int):
        self._check(self.L.mq_mlp_init(self.h, nin, width, nout))
        self.mlp_dims = (nin, width, width, nout)

    def mlp_param_count(self) -> int:
        n = ctypes.c_int()
        self._check(self.L.mq_mlp_param_count(self.h, ctypes.byref(n)))
        return n.value

    def mlp_set_params(self, params):
        p = np.ascontiguousarray(params, dtype=np.float32)
        self._check(self.L.mq_mlp_set_params(self.h, ptr(p)))

    def mlp_get_params(self) -> np.ndarray:
        p = np.zeros(self.mlp_param_count(), dtype=np.float32)
        self._check(self.L.mq_mlp_get_params(self.h, ptr(p)))
        return p

    def mlp_forward(self, X) -> np.ndarray:
        X = np.ascontiguousarray(X, dtype=np.float32)
        Y = np.zeros((X.shape[0], self.mlp_dims[3]), dtype=np.float32)
        self._check(self.L.mq_mlp_forward(self.h, X.shape[0], ptr(X), ptr(Y)))
        return Y

    def mlp_grad(self, X, T, W):
        X, T, W = (np.ascontiguousarray(a, dtype=np.float32) for a in (X, T, W))
        g = np.zeros(self.mlp_param_count(), dtype=np.float32)
        loss = ctypes.c_double()
        self._check(self.L.mq_mlp_grad(self.h, X.shape[0], ptr(X), ptr(T), ptr(W), ptr(g), ctypes.byref(loss)))
        return loss.value, g

    def mlp_set_data(self, X, T, W):
        X, T, W = (np.ascontiguousarray(a, dtype=np.float32) for a in (X, T, W))
        self._check(self.L.mq_mlp_set_data(self.h, X.shape[0], ptr(X), ptr(T), ptr(W)))
        self._mlp_n = X.shape[0]

    def mlp_train_epoch(self, batch: int, lr: float, seed: int) -> float:
        perm = np.random.default_rng(seed).permutation(self._mlp_n).astype(np.int32)
        loss = ctypes.c_double()
        self._check(self.L.mq_mlp_train_epoch(self.h, ptr(perm), batch, ctypes.c_float(lr), ctypes.byref(loss)))
        return loss.value

    def set_fock_precision(self, precision: int):
        """_lib.FOCK_FP64 (default) or _lib.FOCK_DF32 (double-float digestion)."""
        self._check(self.L.mq_set_fock_precision(self.h, precision))

    def set_fock_incremental(self, tau: float):
        """FP32 incremental Fock builds in scf() once max|D_k - D_(k-1)| < tau
        (0: off; tau in [0, 1e-2], else MyQCError)."""
        self._check(self.L.mq_set_fock_incremental(self.h, float(tau)))

    def set_ao2mo_prefetch(self, planes: int):
        """Slice XX for the split transform (2 or 3 planes) during the purified SCF's final eigensolve (0: off)."""
        self._check(self.L.mq_set_ao2mo_prefetch(self.h, int(planes)))

    def set_schwarz(self, thr: float):
        self._check(self.L.mq_set_schwarz(self.h, thr))

    def set_eri_storage(self, storage: int):
        """_lib.STORE_FULL (the n^4 array, default) or _lib.STORE_QUARTETS (each
        screened shell quartet once; needs a Schwarz threshold > 0)."""
        self._check(self.L.mq_set_eri_storage(self.h, int(storage)))

    def set_fock_screened_increments(self, tau: float):
        """tau > 0: after the first build of an RHF SCF from the quartet store,
        each build adds G[D_k - D_(k-1)] in FP64 over the shell quartets with
        Q_P Q_Q max|dD| >= tau; 0 (default): full builds."""
        self._check(self.L.mq_set_fock_screened_increments(self.h, float(tau)))

    def set_eri_tuning(self, mode: int):
        """1 (default): the integral autotuner times the candidate launch shapes
        of each new launch signature once and keeps the fastest; 0: defaults."""
        self._check(self.L.mq_set_eri_tuning(self.h, int(mode)))

    def eri_tuning_report(self) -> str:
        """The autotuner's choices and candidate timings, one line per signature."""
        buf = ctypes.create_string_buffer(1 << 16)
        self._check(self.L.mq_eri_tuning_report(self.h, buf, 1 << 16))
        return buf.value.decode()

    def set_partition(self, part: int, nparts: int):
        """Keep only this process's share (part of nparts) of the molecule's
        shell quartets in RHF Fock builds from the quartet store or direct;
        the parts' G matrices sum to the full G."""
        self._check(self.L.mq_set_partition(self.h, int(part), int(nparts)))

    def set_eri_mixed(self, tau: float):
        """Quartets with a Schwarz bound below tau in FP32 (tight mode; 0: all FP64)."""
        self._check(self.L.mq_set_eri_mixed(self.h, float(tau)))

    # ---------------------------------------------------------------- integrals
    def int1e(self):
        n = self.n
        S = np.zeros((n, n), order="F")
        H = np.zeros((n, n), order="F")
        self._check(self.L.mq_int1e(self.h, ptr(S), ptr(H)))
        return S, H

    def int1p(self) -> np.ndarray:
        """Dipole integrals (3, n, n): <u| x |v>, <u| y |v>, <u| z |v> about the origin."""
        n = self.n
        P = np.zeros(3 * n * n)
        self._check(self.L.mq_int1p(self.h, ptr(P)))
        return np.stack([P[c * n * n:(c + 1) * n * n].reshape(n, n, order="F") for c in range(3)])

    def eri_full(self) -> np.ndarray:
        n = self.n
        XX = np.zeros((n, n, n, n), order="F")
        self._check(self.L.mq_eri_full(self.h, ptr(XX)))
        return XX

    def eri_store(self):
        self._check(self.L.mq_eri_store(self.h))

    def eri_upload(self, XX: np.ndarray):
        X = f64(XX)
        self._check(self.L.mq_eri_upload(self.h, ptr(X)))

    def fock(self, Da, Db=None, direct: bool = False):
        n = self.n
        Da_, Db_ = f64(Da), (None if Db is None else f64(Db))
        Ga = np.zeros((n, n), order="F")
        Gb = None if Db is None else np.zeros((n, n), order="F")
        fn = self.L.mq_fock_direct if direct else self.L.mq_fock
        self._check(fn(self.h, ptr(Da_), ptr(Db_), ptr(Ga), ptr(Gb)))
        return Ga if Db is None else (Ga, Gb)

    # ---------------------------------------------------------------- SCF
    def scf(self, S, H, nalpha: int, nbeta: int, uhf: bool = False, conv: float = 1e-7, conv_rms: bool = False,
            diis: int = 0, direct: bool = False, max_iter: int = 0, D_guess=None, C_guess=None,
            raise_on_noconv: bool = True, purify: bool = False) -> SCFResult:
        n, ns = self.n, 2 if uhf else 1
        o = _lib.ScfOpts()
        o.uhf, o.nalpha, o.nbeta, o.max_iter = int(uhf), nalpha, nbeta, max_iter
        o.conv, o.conv_rms, o.diis, o.direct, o.purify = conv, int(conv_rms), diis, int(direct), int(purify)
        keep = []
        if D_guess is not None:
            Dg = f64(np.asarray(D_guess).reshape(ns, n, n).transpose(1, 2, 0))  # (n, n, ns) F-order = ns blocks
            keep.append(Dg)
            o.guess, o.D_in = 2, Dg.ctypes.data
        elif C_guess is not None:
            Cg = f64(np.asarray(C_guess).reshape(ns, n, n).transpose(1, 2, 0))
            keep.append(Cg)
            o.guess, o.C_in = 1, Cg.ctypes.data
        S_, H_ = f64(S), f64(H)
        C = np.zeros((n, n, ns), order="F")
        eps = np.zeros((n, ns), order="F")
        D = np.zeros((n, n, ns), order="F")
        E = ctypes.c_double()
        it = ctypes.c_int()
        cap = max_iter if max_iter > 0 else (300 if uhf else 500)
        hist = np.zeros(2 * cap)
        rc = self.L.mq_scf(self.h, ptr(S_), ptr(H_), ctypes.byref(o), ptr(C), ptr(eps), ptr(D), ctypes.byref(E),
                           ctypes.byref(it), ptr(hist))
        if not (rc == _lib.MQ_ENOCONV and not raise_on_noconv):
            self._check(rc)
        k = it.value
        if uhf:
            return SCFResult(E.value, eps.T.copy(), np.moveaxis(C, 2, 0).copy(), np.moveaxis(D, 2, 0).copy(), k,
                             hist[: 2 * k].reshape(k, 2))
        return SCFResult(E.value, eps[:, 0].copy(), C[:, :, 0].copy(order="F"), D[:, :, 0].copy(order="F"), k,
                         hist[: 2 * k].reshape(k, 2))

    # ---------------------------------------------------------------- post-HF
    def ao2mo_iajb(self, Ci, Ca, Cj, Cb, precision: int = PREC_FP64, copy_out: bool = True):
        Ci, Ca, Cj, Cb = f64(Ci), f64(Ca), f64(Cj), f64(Cb)
        dims = (Ci.shape[1], Ca.shape[1], Cj.shape[1], Cb.shape[1])
        out = np.zeros(dims, order="F") if copy_out else None
        self._check(self.L.mq_ao2mo_iajb(self.h, ptr(Ci), dims[0], ptr(Ca), dims[1], ptr(Cj), dims[2], ptr(Cb),
                                         dims[3], precision, ptr(out)))
        return out

    def mp2_rhf(self, eig, nocc: int, precision: int = PREC_FP64, C=None) -> dict:
        if C is not None:
            self.ao2mo_iajb(C[:, :nocc], C[:, nocc:], C[:, :nocc], C[:, nocc:], precision, copy_out=False)
        e = np.zeros(3)
        eg = np.ascontiguousarray(eig, dtype=np.float64)
        self._check(self.L.mq_mp2_rhf(self.h, ptr(eg), nocc, self.n - nocc, ptr(e)))
        return {"E_AA": e[0], "E_AB": e[1], "E_MP2": e[2]}

    def mp2_uhf(self, CA, CB, eA, eB, noA: int, noB: int, precision: int = PREC_FP64) -> dict:
        e = np.zeros(4)
        CA_, CB_ = f64(CA), f64(CB)
        eA_, eB_ = np.ascontiguousarray(eA, dtype=np.float64), np.ascontiguousarray(eB, dtype=np.float64)
        self._check(self.L.mq_mp2_uhf(self.h, ptr(CA_), ptr(CB_), ptr(eA_), ptr(eB_), noA, noB, precision, ptr(e)))
        return {"E_AA": e[0], "E_BB": e[1], "E_AB": e[2], "E_MP2": e[3]}

    # ---------------------------------------------------------------- linear algebra
    def dgemm(self, A: np.ndarray, B: np.ndarray, transa: str = "N", transb: str = "N", alpha: float = 1.0,
              beta: float = 0.0, C: np.ndarray = None):
        """alpha op(A) op(B) + beta C through mq_dgemm (FP64 on the device)."""
        A_, B_ = f64(A), f64(B)
        m = A_.shape[1] if transa == "T" else A_.shape[0]
        k = A_.shape[0] if transa == "T" else A_.shape[1]
        n = B_.shape[0] if transb == "T" else B_.shape[1]
        C_ = np.zeros((m, n), order="F") if C is None else np.asfortranarray(np.array(C, dtype=np.float64))
        self._check(self.L.mq_dgemm(self.h, transa.encode(), transb.encode(), m, n, k, alpha, ptr(A_), A_.shape[0],
                                    ptr(B_), B_.shape[0], beta, ptr(C_), m))
        return C_

    def syev_batched(self, A: np.ndarray):
        A = np.asarray(A, dtype=np.float64)
        batch, n = A.shape[0], A.shape[1]
        Ab = np.ascontiguousarray(np.stack([np.asfortranarray(a).reshape(-1, order="F") for a in A]))
        w = np.zeros((batch, n))
        V = np.zeros((batch, n * n))
        self._check(self.L.mq_syev_batched(self.h, n, batch, ptr(Ab), ptr(w), ptr(V)))
        return w, np.stack([v.reshape(n, n, order="F") for v in V])

    def sygv(self, F, S):
        n = F.shape[0]
        F_, S_ = f64(F), f64(S)
        w = np.zeros(n)
        C = np.zeros((n, n), order="F")
        self._check(self.L.mq_sygv(self.h, n, ptr(F_), ptr(S_), ptr(w), ptr(C)))
        return w, C

    def probe_fp64(self) -> float:
        """FP64 fma rate of this GPU in TFLOP/s (a short measuring kernel)."""
        v = ctypes.c_double()
        self._check(self.L.mq_probe_fp64(self.h, ctypes.byref(v)))
        return v.value

    def stat(self, key: str) -> float:
        v = ctypes.c_double()
        self._check(self.L.mq_stat(self.h, key.encode(), ctypes.byref(v)))
        return v.value


def run_job(sysm: System, basis: BasisArrays, ftab=None, mode: int = MODE_REFERENCE, conv: float | None = None,
            diis: int = 0, precision: int = PREC_FP64, ctx: Context | None = None, mp2: bool | None = None):
    """parse -> int1e -> int2e -> scf [-> ao2mo -> mp2] on the GPU (the myQC.f90 stage order)."""
    own = ctx is None
    ctx = ctx or Context()
    try:
        ctx.set_system(sysm, basis, ftab, mode)
        S, H = ctx.int1e()
        ctx.eri_store()
        lim = conv if conv is not None else 10.0 ** (-min(sysm.options[8], 12))
        res = ctx.scf(S, H, sysm.nelcA, sysm.nelcB, uhf=sysm.uhf, conv=lim, diis=diis)
        out = {"S": S, "H": H, "scf": res}
        do_mp2 = (sysm.options[1] == 1) if mp2 is None else mp2
        if do_mp2:
            if sysm.uhf:
                out["mp2"] = ctx.mp2_uhf(res.C[0], res.C[1], res.eig[0], res.eig[1], sysm.nelcA, sysm.nelcB,
                                         precision)
            else:
                out["mp2"] = ctx.mp2_rhf(res.eig, sysm.nelcA, precision, C=res.C)
        return out
    finally:
        if own:
            ctx.close()
