"""adp_power_noalloc: PowDis on caller-owned device arrays with no handle and
no allocation, for callers that cannot call cudaMalloc (their device memory
belongs to another allocator, or cudaMalloc's implicit synchronisation is
not acceptable on their path).  Its output must match adp_power's on the
same flux, within the power tolerance of the parity tests, on two calls in
a row.  This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PTOL = 1e-6


def _solve(seed, ng):
    from adpres_gb300 import deck, synth
    from adpres_gb300.core import Core
    dk = deck.parse(synth.small_core(seed=seed, ng=ng, adf=True))
    c = Core.from_deck(dk)
    c.outer()
    p_ref = c.power()
    f0, _, _, _ = c.state()
    c.close()
    vdel = dk.xdel[dk.ix - 1] * dk.ydel[dk.iy - 1] * dk.zdel[dk.iz - 1]
    sigf = dk.xsigf[dk.mat - 1]                       # (nnod, ng)
    return dk, f0, sigf, vdel, p_ref


def test_power_noalloc_matches_adp_power_twice():
    torch = pytest.importorskip("torch")
    from adpres_gb300 import _lib
    L = _lib.load()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for seed, ng in ((1, 2), (2, 3)):                  # two calls in a row, different cores
        dk, f0, sigf, vdel, p_ref = _solve(seed, ng)
        d_f0 = torch.tensor(np.asfortranarray(f0).reshape(-1, order="F"), dtype=torch.float64, device="cuda")
        d_sf = torch.tensor(np.asfortranarray(sigf).reshape(-1, order="F"), dtype=torch.float64, device="cuda")
        d_v = torch.tensor(vdel, dtype=torch.float64, device="cuda")
        d_p = torch.full((dk.nnod,), -1.0, dtype=torch.float64, device="cuda")
        st = L.adp_power_noalloc(dk.nnod, dk.ng, ctypes.c_void_p(d_f0.data_ptr()), ctypes.c_void_p(d_sf.data_ptr()),
                                 ctypes.c_void_p(d_v.data_ptr()), ctypes.c_void_p(d_p.data_ptr()), stream)
        assert st == _lib.ADP_OK, _lib.last_error(None)
        p = d_p.cpu().numpy()
        np.testing.assert_allclose(p, p_ref, rtol=PTOL, atol=0)
        assert abs(p.sum() - 1.0) < 1e-12


def test_power_noalloc_rejects_sizes_and_zero_power():
    torch = pytest.importorskip("torch")
    from adpres_gb300 import _lib
    L = _lib.load()
    nul = ctypes.c_void_p(0)
    assert L.adp_power_noalloc(0, 2, nul, nul, nul, nul, nul) == _lib.ADP_ERR_INPUT
    assert L.adp_power_noalloc(10, 9, nul, nul, nul, nul, nul) == _lib.ADP_ERR_INPUT
    assert "maximum" in _lib.last_error(None)
    assert L.adp_power_noalloc(2 ** 30, 4, nul, nul, nul, nul, nul) == _lib.ADP_ERR_INPUT
    assert "maximum" in _lib.last_error(None)
    z = torch.zeros(8, dtype=torch.float64, device="cuda")
    v = torch.ones(4, dtype=torch.float64, device="cuda")
    out = torch.zeros(4, dtype=torch.float64, device="cuda")
    st = L.adp_power_noalloc(4, 2, ctypes.c_void_p(z.data_ptr()), ctypes.c_void_p(z.data_ptr()),
                             ctypes.c_void_p(v.data_ptr()), ctypes.c_void_p(out.data_ptr()), nul)
    assert st == _lib.ADP_ERR_ZEROPOWER
    # on that error p holds the unnormalised per-node powers (all zero here)
    assert np.all(out.cpu().numpy() == 0.0)
    # the status word is cleared per call: a valid call afterwards succeeds
    f = torch.ones(8, dtype=torch.float64, device="cuda")
    st = L.adp_power_noalloc(4, 2, ctypes.c_void_p(f.data_ptr()), ctypes.c_void_p(f.data_ptr()),
                             ctypes.c_void_p(v.data_ptr()), ctypes.c_void_p(out.data_ptr()), nul)
    assert st == _lib.ADP_OK
    np.testing.assert_allclose(out.cpu().numpy(), np.full(4, 0.25))


def test_power_noalloc_many_blocks_matches_adp_power():
    """A core of more than 262,144 nodes (the 68x68x80 four-group core,
    369,920 nodes): more blocks than the scratch holds partial sums for, so
    the launch is capped at that many blocks and each block sums several
    rows per thread.  A seeded positive flux, through adp_power on a handle
    and through the allocation-free call twice."""
    torch = pytest.importorskip("torch")
    from adpres_gb300 import _lib, deck, synth
    from adpres_gb300.core import Core
    dk = deck.parse(synth.core_4g(0))
    assert dk.nnod > 1024 * 256
    c = Core.from_deck(dk)
    rng = np.random.default_rng(5)
    f0 = rng.uniform(0.1, 2.0, (dk.nnod, dk.ng))
    c.set_state(f0=f0, fs0=np.ones(dk.nnod), keff=1.0)
    p_ref = c.power()
    c.close()
    L = _lib.load()
    vdel = dk.xdel[dk.ix - 1] * dk.ydel[dk.iy - 1] * dk.zdel[dk.iz - 1]
    sigf = dk.xsigf[dk.mat - 1]
    d_f0 = torch.tensor(np.asfortranarray(f0).reshape(-1, order="F"), dtype=torch.float64, device="cuda")
    d_sf = torch.tensor(np.asfortranarray(sigf).reshape(-1, order="F"), dtype=torch.float64, device="cuda")
    d_v = torch.tensor(vdel, dtype=torch.float64, device="cuda")
    for _ in range(2):
        d_p = torch.full((dk.nnod,), -1.0, dtype=torch.float64, device="cuda")
        st = L.adp_power_noalloc(dk.nnod, dk.ng, ctypes.c_void_p(d_f0.data_ptr()), ctypes.c_void_p(d_sf.data_ptr()),
                                 ctypes.c_void_p(d_v.data_ptr()), ctypes.c_void_p(d_p.data_ptr()), ctypes.c_void_p(0))
        assert st == _lib.ADP_OK, _lib.last_error(None)
        np.testing.assert_allclose(d_p.cpu().numpy(), p_ref, rtol=PTOL, atol=0)
