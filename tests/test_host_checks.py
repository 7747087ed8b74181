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
