"""Smallest split-transform case (CO2) with per-stage stream checks.

    MYQC_SYNC_CHECK=1 python tests/diag_split_case.py [bf16|bf16x3]

Prints the failing stage, if any.  A diagnostic, not collected by pytest."""
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import numpy as np  # noqa: E402

from myqc_gb300 import MODE_TIGHT, PREC_FP64, PREC_SPLIT_BF16, PREC_SPLIT_BF16X3, formats  # noqa: E402
from myqc_gb300.session import Context  # noqa: E402

g = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
prec = PREC_SPLIT_BF16X3 if len(sys.argv) > 1 and sys.argv[1] == "bf16x3" else PREC_SPLIT_BF16
s = formats.parse_zmat_text(open(os.path.join(g, "zmat", "CO2.ZMAT")).read())
b = formats.parse_mybasis_text(open(os.path.join(g, "mybasis")).read(), s.atoms)
ctx = Context(0)
ctx.set_system(s, b, None, MODE_TIGHT)
S, H = ctx.int1e()
ctx.eri_store()
r = ctx.scf(S, H, s.nelcA, s.nelcB, conv=1e-10, diis=8)
no = s.nelcA
blocks = (r.C[:, :no], r.C[:, no:], r.C[:, :no], r.C[:, no:])
ref = ctx.ao2mo_iajb(*blocks, PREC_FP64)
got = ctx.ao2mo_iajb(*blocks, prec)
print("max |split - fp64| / max|fp64| =", np.max(np.abs(got - ref)) / np.max(np.abs(ref)))
