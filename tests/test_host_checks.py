"""Host-side argument checks of the Python mirror (no device call): arrays
handed to the C library must hold exactly the values it reads."""
import types

import numpy as np
import pytest

from adpres_gb300._lib import ADP_ERR_INPUT, AdpError
from adpres_gb300.core import Core


def _fake(nnod=10, ng=2):
    return types.SimpleNamespace(nnod=nnod, ng=ng)


def _tables(rows, ng):
    return [np.ones((rows, ng)) for _ in range(4)]


def test_xs_args_accepts_the_reference_shapes():
    f = _fake()
    nmat, args, m, s, d = Core._xs_args(f, "mat", _tables(3, 2), np.ones((3, 2)), np.ones(10, int),
                                        np.ones((3, 2, 2)), np.ones((10, 2, 6)))
    assert nmat == 3 and len(args) == 5 and m.dtype == np.int32 and s.size == 12 and d.size == 120
    nmat, args, m, s, d = Core._xs_args(f, "node", _tables(10, 2), np.ones((3, 2)), np.ones(10, int),
                                        np.ones((10, 2, 2)), None)
    assert nmat == 3 and d is None and args[0].size == 20


@pytest.mark.parametrize("bad", ["table", "chi", "mat", "sigs", "dc"])
def test_xs_args_rejects_a_wrong_size(bad):
    f = _fake()
    tabs, chi, mat = _tables(10, 2), np.ones((3, 2)), np.ones(10, int)
    sigs, dc = np.ones((10, 2, 2)), np.ones((10, 2, 6))
    if bad == "table":
        tabs[2] = np.ones((9, 2))
    elif bad == "chi":
        chi = np.ones(5)
    elif bad == "mat":
        mat = np.ones(9, int)
    elif bad == "sigs":
        sigs = np.ones((10, 2))
    else:
        dc = np.ones((10, 2, 5))
    with pytest.raises(AdpError) as e:
        Core._xs_args(f, "node", tabs, chi, mat, sigs, dc)
    assert e.value.status == ADP_ERR_INPUT


def test_sized_checks_the_value_count():
    f = _fake(nnod=4, ng=2)
    a = np.ones((4, 2))
    assert Core._sized(f, a, 8, "af") is a
    for bad in (np.ones((4, 3)), None, np.ones(7)):
        with pytest.raises(AdpError) as e:
            Core._sized(f, bad, 8, "af")
        assert e.value.status == ADP_ERR_INPUT


class _StubLib:
    """Stands in for the C library: every entry point returns ADP_OK, so
    only the Python side's marshalling runs."""

    def __getattr__(self, name):
        return lambda *a, **k: 0


def test_host_entry_points_marshal_a_deck_without_a_device():
    from adpres_gb300 import deck, synth
    dk = deck.parse(synth.rod_ejection_3d(0, n=9, planes=6))
    c = Core.__new__(Core)
    c.L, c.h, c.nnod, c.ng, c._fb_cards = _StubLib(), None, dk.nnod, dk.ng, []
    m = dk.mat - 1
    c.xs_updt(dk.xsigtr, dk.xsiga, dk.xnuf, dk.xsigf, dk.chi, dk.mat, dk.xsigs, dk.dc)
    c.xs_updt_nodes(dk.xsigtr[m], dk.xsiga[m], dk.xnuf[m], dk.xsigf[m], dk.chi, dk.mat, dk.xsigs[m], dk.dc)
    c.set_xs(dk.xsigtr[m], dk.xsiga[m], dk.xnuf[m], dk.xsigf[m], dk.chi, dk.mat, dk.xsigs[m], dk.dc)
    c.fb_set(dk)
    assert c._fb_cards == [nm for nm in ("bcon", "ftem", "mtem", "cden") if nm in dk.feedback]
    c.fb_updt(dk)
    c.fb_updt(dk, bcon=1000.0, bpos=np.array(dk.feedback["crod"]["bpos"], float))
    with pytest.raises(AdpError):
        c.fb_updt(dk, bpos=np.zeros(int(dk.feedback["crod"]["nb"]) + 1))
    af = np.ones((dk.nnod, dk.ng))
    tr = dk.trans
    c.trans_init(tr["beta"], tr["lamb"], tr["velo"], tr["theta"], tr["extr"], af)
    with pytest.raises(AdpError):
        c.trans_init(tr["beta"], tr["lamb"], tr["velo"], tr["theta"], tr["extr"], af[:-1])
    c.set_state(f0=af, fs0=np.ones(dk.nnod), keff=1.0, dn=np.zeros((dk.nnod, dk.ng, 6)))
    c.reactivity(af)
    c.reactivity(af, af)
    c.core_beta(af, np.full((dk.chi.shape[0], 6), 1e-3), dk.mat)
