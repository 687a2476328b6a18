"""myqc_gb300 -- GB300-native engine for myQC's Hartree-Fock/MP2 hot path.

The compute lives in libmyqc.so (hand-written sm_103a CUDA behind the C ABI of
include/myqc.h); this package is its Python host: file formats, a ctypes
Context, and the synthetic workloads used by the benchmark."""
from ._lib import (FOCK_DF32, FOCK_FP64, MODE_REFERENCE, MODE_TIGHT, PREC_FP64, PREC_SPLIT_BF16,  # noqa: F401
                   PREC_SPLIT_BF16X3, STORE_FULL, STORE_QUARTETS, MyQCError)
from .formats import BasisArrays, System, parse_mybasis_text, parse_zmat_text  # noqa: F401

__version__ = "0.1.0"


def Context(device: int = 0):
    from .session import Context as _C
    return _C(device)
