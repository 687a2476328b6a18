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


def test_prefetched_slices_identical(ctx, basis_text):
    """XX sliced on the side stream during the purified SCF's final eigensolve
    (mq_set_ao2mo_prefetch) gives the same (ia|jb) and E(MBPT2), bit for bit,
    as slicing it inside the transform; a second solve of another system with
    the prefetch on still matches (the slices follow XX)."""
    from myqc_gb300 import FOCK_FP64
    for k, seed in ((4, 3), (6, 4)):
        sysm = molecules.water_cluster_system(k, (27.0 * k) ** (1 / 3) + 1.0, seed)
        basis = formats.parse_mybasis_text(basis_text, sysm.atoms)
        ctx.set_fock_precision(FOCK_FP64)
        ctx.set_system(sysm, basis, None, MODE_TIGHT)
        S, H = ctx.int1e()
        kw = dict(conv=1e-10, conv_rms=True, diis=8, purify=True)
        ctx.eri_store()
        ctx.set_ao2mo_prefetch(0)
        r0 = ctx.scf(S, H, sysm.nelcA, sysm.nelcB, **kw)
        e0 = ctx.mp2_rhf(r0.eig, sysm.nelcA, PREC_SPLIT_BF16X3, C=r0.C)
        try:
            ctx.set_ao2mo_prefetch(3)
            r1 = ctx.scf(S, H, sysm.nelcA, sysm.nelcB, **kw)
            e1 = ctx.mp2_rhf(r1.eig, sysm.nelcA, PREC_SPLIT_BF16X3, C=r1.C)
        finally:
            ctx.set_ao2mo_prefetch(0)
        assert r1.energy == r0.energy
        assert np.array_equal(r1.C, r0.C)
        assert e1["E_MP2"] == e0["E_MP2"], (k, e1, e0)
