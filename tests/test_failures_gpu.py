"""Every status code of the C ABI's failure paths, on the GPU, from inputs
made on the host (tests/failure_cases.py); none faults or hangs the GPU.

* ADP_ERR_PIVOT and ADP_ERR_DIVERGED: the same inputs make the oracle stop
  with the same codes (tests/test_failures_oracle.py); the message names a
  node of the material with the tiny ADFs / the size of the change.
* ADP_ERR_BREAKDOWN (a zero flux and fission source: BiCGSTAB's (rs, r) is
  0) and ADP_ERR_NAN (a NaN cross section): the reference produces k = NaN
  there without stopping.
* ADP_ERR_TIMEOUT: with adp_test_missing_block the launches count one block
  more than they launch, so every barrier wait runs out after the wait
  limit (5 ms here); the same handle then solves normally.
"""
import numpy as np
import pytest

import oracle
from adpres_gb300 import deck
from adpres_gb300._lib import (ADP_ERR_BREAKDOWN, ADP_ERR_DIVERGED, ADP_ERR_NAN, ADP_ERR_PIVOT, ADP_ERR_TIMEOUT,
                               AdpError)
from failure_cases import DN_BIG, TEXT, TINY_ADF_MAT, nan_siga, tiny_adf

pytestmark = pytest.mark.gpu


def _core(**over):
    from adpres_gb300.core import Core
    dk = deck.parse(TEXT)
    return dk, Core.from_deck(dk, **over)


def _node_tables(dk):
    m = dk.mat - 1
    return dk.xsigtr[m], dk.xsiga[m], dk.xnuf[m], dk.xsigf[m], dk.xsigs[m]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_pivot(precision):
    dk, c = _core(precision=precision)
    tr, sa, nf, sf, ss = _node_tables(dk)
    c.xs_updt_nodes(tr, sa, nf, sf, dk.chi, dk.mat, ss, tiny_adf(dk.dc, dk.mat))
    with pytest.raises(AdpError) as e:
        c.outer()
    assert e.value.status == ADP_ERR_PIVOT
    msg = str(e.value)
    assert "diagonal elements close to zero" in msg
    i, j, k = (int(v) for v in msg.split("I = ")[1].replace("J = ", "").replace("K = ", "").split(","))
    # the node of a failing face system, as LU_solve reports it: the face's
    # n node, of the tiny-ADF material or its neighbour across the face
    nodes = np.nonzero((abs(dk.ix - i) + abs(dk.iy - j) + abs(dk.iz - k)) <= 1)[0]
    assert np.any((dk.ix[nodes] == i) & (dk.iy[nodes] == j) & (dk.iz[nodes] == k))
    assert np.any(dk.mat[nodes] == TINY_ADF_MAT)


def test_diverged():
    dk, c0 = _core()
    c0.outer()
    f0, fs0, k0, dn = c0.state()
    # a nodal update after every outer, from the converged flux with every
    # coupling coefficient at 2e3
    _, c = _core(nupd=1)
    c.set_state(f0=f0, fs0=fs0, keff=k0, dn=np.full_like(dn, DN_BIG))
    with pytest.raises(AdpError) as e:
        c.outer()
    assert e.value.status == ADP_ERR_DIVERGED
    assert "seems not stable" in str(e.value)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_breakdown_on_zero_start(precision):
    dk, c = _core(precision=precision)
    c.outer()
    f0, fs0, k0, dn = c.state()
    c.set_state(f0=np.zeros_like(f0), fs0=np.zeros_like(fs0), keff=k0, dn=dn)
    with pytest.raises(AdpError) as e:
        c.outer()
    assert e.value.status == ADP_ERR_BREAKDOWN
    # the handle recovers from a fresh start
    c.reset()
    assert c.outer().converged


def test_nan_cross_section():
    dk, c = _core()
    tr, sa, nf, sf, ss = _node_tables(dk)
    c.xs_updt_nodes(tr, nan_siga(sa), nf, sf, dk.chi, dk.mat, ss, dk.dc)
    with pytest.raises(AdpError) as e:
        c.outer()
    assert e.value.status == ADP_ERR_NAN


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_timeout_then_normal_solve(precision):
    dk, c = _core(precision=precision)
    c.set_wait_limit(0.005)
    c.test_missing_block(True)
    with pytest.raises(AdpError) as e:
        c.outer()
    assert e.value.status == ADP_ERR_TIMEOUT
    assert "ran out of time" in str(e.value)
    c.test_missing_block(False)
    c.set_wait_limit(0.0)
    c.reset()
    rep = c.outer()
    o = oracle.Oracle(text=TEXT)
    o.run()
    assert rep.converged and abs(rep.keff - o.getd("Ke")) <= 1e-6 * o.getd("Ke")
