"""Split-BF16 tensor-core transform (tcgen05) against the FP64 path.

Operand rows are cut into 2 or 3 exact 8-bit BF16 slices under one power-of-two
scale per row; the slice products accumulate exactly, so the only error is the
unbiased rounding of the slicing (2^-16 or 2^-24 of each row's largest
element).  The MP2 energy sees that error at second order: hi+lo slices leave
~1e-5 Eh, hi+mid+lo slices stay well below the 1 uEh target.  Each mode is
checked to its own bound, on the transform (relative to the largest |(ia|jb)|)
and on E(MBPT2)."""
import numpy as np
import pytest

from conftest import golden
from myqc_gb300 import MODE_TIGHT, PREC_FP64, PREC_SPLIT_BF16, PREC_SPLIT_BF16X3, formats, molecules

pytestmark = pytest.mark.gpu

MODES = [(PREC_SPLIT_BF16, 1e-2, 5e-5), (PREC_SPLIT_BF16X3, 1e-4, 1e-6)]


def _systems():
    out = []
    for name in ("CO2", "HF", "NO"):
        out.append((name, formats.parse_zmat_text(open(golden("zmat", name + ".ZMAT")).read())))
    for nm in (2, 4):
        out.append((f"(H2O){nm}", molecules.water_cluster_system(nm, (27.0 * nm) ** (1 / 3) + 1.0, 7)))
    return out


@pytest.mark.parametrize("prec,tol_rel,tol_mp2", MODES)
@pytest.mark.parametrize("idx", range(5))
def test_split_transform_matches_fp64(ctx, basis_text, idx, prec, tol_rel, tol_mp2):
    name, sysm = _systems()[idx]
    basis = formats.parse_mybasis_text(basis_text, sysm.atoms)
    ctx.set_system(sysm, basis, None, MODE_TIGHT)
    S, H = ctx.int1e()
    ctx.eri_store()
    res = ctx.scf(S, H, sysm.nelcA, sysm.nelcB, uhf=sysm.uhf, conv=1e-10, diis=8)
    C = res.C[0] if sysm.uhf else res.C
    no = sysm.nelcA
    blocks = (C[:, :no], C[:, no:], C[:, :no], C[:, no:])
    ref = ctx.ao2mo_iajb(*blocks, PREC_FP64)
    got = ctx.ao2mo_iajb(*blocks, prec)
    assert np.max(np.abs(got - ref)) < tol_rel * np.max(np.abs(ref))
    if sysm.uhf:
        e64 = ctx.mp2_uhf(res.C[0], res.C[1], res.eig[0], res.eig[1], sysm.nelcA, sysm.nelcB, PREC_FP64)
        e16 = ctx.mp2_uhf(res.C[0], res.C[1], res.eig[0], res.eig[1], sysm.nelcA, sysm.nelcB, prec)
    else:
        e64 = ctx.mp2_rhf(res.eig, no, PREC_FP64, C=C)
        e16 = ctx.mp2_rhf(res.eig, no, prec, C=C)
    assert abs(e16["E_MP2"] - e64["E_MP2"]) < tol_mp2, (name, e16, e64)


def test_split_rectangular_blocks(ctx, basis_text):
    """Unequal occupied / virtual blocks and odd sizes (K padding, partial tiles)."""
    sysm = formats.parse_zmat_text(open(golden("zmat", "CO.ZMAT")).read())
    basis = formats.parse_mybasis_text(basis_text, sysm.atoms)
    ctx.set_system(sysm, basis, None, MODE_TIGHT)
    ctx.eri_store()
    n = ctx.n
    rng = np.random.default_rng(5)
    Ci, Ca, Cj, Cb = (rng.standard_normal((n, k)) * 0.3 for k in (3, 7, 5, 2))
    ref = ctx.ao2mo_iajb(Ci, Ca, Cj, Cb, PREC_FP64)
    for prec, tol, _ in MODES:
        got = ctx.ao2mo_iajb(Ci, Ca, Cj, Cb, prec)
        assert np.max(np.abs(got - ref)) < tol * np.max(np.abs(ref))
