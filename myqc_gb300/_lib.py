"""ctypes binding of libmyqc (include/myqc.h).

The library is the product: there is no CPU fallback.  Loading fails loudly
when ``myqc_gb300/lib/libmyqc.so`` has not been built (``python -m
myqc_gb300.build``) or no CUDA device is present.
"""
from __future__ import annotations

import ctypes
import os
import re

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libmyqc.so")
HEADER = os.path.join(HERE, "..", "include", "myqc.h")

MQ_OK, MQ_EINVAL, MQ_ENOMEM, MQ_ECUDA, MQ_ETIMEOUT, MQ_ENOCONV, MQ_ESTATE = range(7)
MODE_REFERENCE, MODE_TIGHT = 0, 1
PREC_FP64, PREC_SPLIT_BF16, PREC_SPLIT_BF16X3 = 0, 1, 2
FOCK_FP64, FOCK_DF32 = 0, 1
STORE_FULL, STORE_QUARTETS = 0, 1
_NAMES = {0: "MQ_OK", 1: "MQ_EINVAL", 2: "MQ_ENOMEM", 3: "MQ_ECUDA", 4: "MQ_ETIMEOUT", 5: "MQ_ENOCONV",
          6: "MQ_ESTATE"}


class MyQCError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{_NAMES.get(code, code)}: {msg}")
        self.code = code


class ScfOpts(ctypes.Structure):
    _fields_ = [("uhf", ctypes.c_int), ("nalpha", ctypes.c_int), ("nbeta", ctypes.c_int),
                ("max_iter", ctypes.c_int), ("conv", ctypes.c_double), ("conv_rms", ctypes.c_int),
                ("diis", ctypes.c_int), ("direct", ctypes.c_int), ("guess", ctypes.c_int),
                ("C_in", ctypes.c_void_p), ("D_in", ctypes.c_void_p), ("purify", ctypes.c_int)]


class BatchOpts(ctypes.Structure):
    _fields_ = [("max_iter", ctypes.c_int), ("conv", ctypes.c_double), ("conv_rms", ctypes.c_int),
                ("diis", ctypes.c_int), ("graph", ctypes.c_int), ("check_every", ctypes.c_int),
                ("D_in", ctypes.c_void_p)]


def header_symbols() -> list[str]:
    """Names of every function the public header declares."""
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(mq_\w+)\s*\(", txt, re.M)))


_lib = None


def lib(path: str | None = None):
    """Load libmyqc.so (once) and declare argument types."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise OSError(f"libmyqc.so not built at {p}; run `python -m myqc_gb300.build`")
    L = ctypes.CDLL(p)
    vp, ip, dp, c_int, c_double = ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.c_void_p, ctypes.c_int, \
        ctypes.c_double
    L.mq_version.restype = ctypes.c_char_p
    L.mq_init.argtypes = [ctypes.POINTER(vp), c_int]
    L.mq_free.argtypes = [vp]
    L.mq_last_error.argtypes = [vp, ctypes.c_char_p, c_int]
    L.mq_set_system.argtypes = [vp, c_int, vp, vp, vp, vp, vp, vp, vp, c_int]
    L.mq_norb.argtypes = [vp, ip]
    L.mq_set_schwarz.argtypes = [vp, c_double]
    L.mq_set_eri_mixed.argtypes = [vp, c_double]
    L.mq_set_eri_storage.argtypes = [vp, c_int]
    L.mq_set_eri_tuning.argtypes = [vp, c_int]
    L.mq_basis_library.argtypes = [vp, ctypes.c_char_p]
    L.mq_guess_model.argtypes = [vp, c_int, c_int, c_int, vp, vp, vp, vp, vp]
    L.mq_guess_predict.argtypes = [vp, c_int, vp, vp, vp, vp]
    L.mq_basis_build.argtypes = [vp, c_int, vp, vp, vp, vp, vp, vp]
    L.mq_batch_add_atoms.argtypes = [vp, c_int, vp, vp, c_int]
    L.mq_set_fock_screened_increments.argtypes = [vp, ctypes.c_double]
    L.mq_eri_tuning_report.argtypes = [vp, ctypes.c_char_p, c_int]
    L.mq_set_partition.argtypes = [vp, c_int, c_int]
    L.mq_probe_fp64.argtypes = [vp, ctypes.POINTER(ctypes.c_double)]
    L.mq_int1e.argtypes = [vp, dp, dp]
    L.mq_int1p.argtypes = [vp, vp]
    L.mq_eri_full.argtypes = [vp, dp]
    L.mq_eri_store.argtypes = [vp]
    L.mq_eri_upload.argtypes = [vp, dp]
    L.mq_fock.argtypes = [vp, dp, dp, dp, dp]
    L.mq_fock_direct.argtypes = [vp, dp, dp, dp, dp]
    L.mq_fock_rhf_noalloc.argtypes = [c_int, vp, vp, vp, vp, ctypes.c_char_p, c_int]
    L.mq_scf.argtypes = [vp, dp, dp, ctypes.POINTER(ScfOpts), dp, dp, dp, ctypes.POINTER(c_double), ip, dp]
    L.mq_ao2mo_iajb.argtypes = [vp, dp, c_int, dp, c_int, dp, c_int, dp, c_int, c_int, dp]
    L.mq_mp2_rhf.argtypes = [vp, dp, c_int, c_int, dp]
    L.mq_mp2_uhf.argtypes = [vp, dp, dp, dp, dp, c_int, c_int, c_int, dp]
    L.mq_mp2_pairs.argtypes = [vp, dp, c_int, c_int, c_int, c_int, dp, dp, c_int, dp]
    L.mq_syev_batched.argtypes = [vp, c_int, c_int, dp, dp, dp]
    L.mq_dgemm.argtypes = [vp, ctypes.c_char, ctypes.c_char, c_int, c_int, c_int, ctypes.c_double, dp, c_int, dp, c_int,
                           ctypes.c_double, dp, c_int]
    L.mq_sygv.argtypes = [vp, c_int, dp, dp, dp, dp]
    L.mq_stat.argtypes = [vp, ctypes.c_char_p, ctypes.POINTER(c_double)]
    L.mq_mlp_init.argtypes = [vp, c_int, c_int, c_int]
    L.mq_mlp_param_count.argtypes = [vp, ip]
    L.mq_mlp_set_params.argtypes = [vp, vp]
    L.mq_mlp_get_params.argtypes = [vp, vp]
    L.mq_mlp_forward.argtypes = [vp, c_int, vp, vp]
    L.mq_mlp_grad.argtypes = [vp, c_int, vp, vp, vp, vp, ctypes.POINTER(c_double)]
    L.mq_mlp_set_data.argtypes = [vp, ctypes.c_longlong, vp, vp, vp]
    L.mq_mlp_train_epoch.argtypes = [vp, vp, c_int, ctypes.c_float, ctypes.POINTER(c_double)]
    L.mq_set_fock_precision.argtypes = [vp, c_int]
    L.mq_set_fock_incremental.argtypes = [vp, c_double]
    L.mq_set_ao2mo_prefetch.argtypes = [vp, c_int]
    L.mq_batch_clear.argtypes = [vp]
    L.mq_batch_add.argtypes = [vp, c_int, vp, vp, vp, vp, vp, vp, c_int]
    L.mq_batch_info.argtypes = [vp, ip, vp]
    L.mq_batch_scf.argtypes = [vp, ctypes.POINTER(BatchOpts), dp, vp, vp, dp, dp]
    _lib = L
    return L


def ptr(a: np.ndarray | None):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


def f64(a) -> np.ndarray:
    """Fortran-ordered contiguous float64 copy/view."""
    return np.asfortranarray(np.asarray(a, dtype=np.float64))
