"""The allocation-free Fock entry point against the regular one.

mq_fock_rhf_noalloc is for callers that cannot allocate device memory: it runs
on device buffers the caller owns and keeps its scratch in a fixed array inside
the library.  Here torch owns the device buffers (standing in for such a
caller's runtime); the result must match mq_fock (host arrays, context-owned
scratch) to the Fock tolerance of the parity tests, on two calls in a row --
the second with a different density, so stale scratch from the first call
would show.  This file sorts last so that a run stopping at the first failure
has run every other test first; it also passes alone in a fresh process."""
import ctypes

import numpy as np
import pytest

from myqc_gb300 import MODE_TIGHT, _lib, formats, molecules

pytestmark = pytest.mark.gpu


def test_fock_noalloc_matches_fock(ctx, basis_text):
    torch = pytest.importorskip("torch")
    sysm = molecules.water_cluster_system(4, 5.0, 11)
    basis = formats.parse_mybasis_text(basis_text, sysm.atoms)
    ctx.set_system(sysm, basis, None, MODE_TIGHT)
    XX = ctx.eri_full()
    n = ctx.n
    L = _lib.lib()
    dev = torch.device("cuda", 0)
    d_xx = torch.from_numpy(np.ascontiguousarray(XX.reshape(-1, order="F"))).to(dev)
    d_g = torch.empty(n * n, dtype=torch.float64, device=dev)
    rng = np.random.default_rng(2)
    for call in range(2):
        D = rng.standard_normal((n, n))
        D = D + D.T
        d_d = torch.from_numpy(np.ascontiguousarray(D.reshape(-1, order="F"))).to(dev)
        d_g.fill_(float("nan"))
        msg = ctypes.create_string_buffer(256)
        stream = torch.cuda.current_stream(dev).cuda_stream
        rc = L.mq_fock_rhf_noalloc(n, ctypes.c_void_p(d_xx.data_ptr()), ctypes.c_void_p(d_d.data_ptr()),
                                   ctypes.c_void_p(d_g.data_ptr()), ctypes.c_void_p(stream), msg, 256)
        assert rc == 0, msg.value
        torch.cuda.synchronize(dev)
        G = d_g.cpu().numpy().reshape(n, n, order="F")
        ref = ctx.fock(D)
        assert np.max(np.abs(G - ref)) < 1e-11 * max(1.0, np.max(np.abs(ref))), call


def test_fock_noalloc_rejects_oversize():
    msg = ctypes.create_string_buffer(256)
    one = ctypes.c_void_p(16)  # never dereferenced: the size check comes first
    rc = _lib.lib().mq_fock_rhf_noalloc(1100, one, one, one, None, msg, 256)
    assert rc == _lib.MQ_EINVAL and msg.value
