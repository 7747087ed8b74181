"""The oracle against the reference's own golden output.

The pin is the IAEA3D convergence trace printed in docs/quick-guides.md:161-191
(fixture tests/golden/iaea3d_trace.json, made by tests/golden/make_golden.py):
every printed digit of k, fission-source error and flux error, the
extrapolation events, the nodal-update record and the final k.
"""
import json
import os

import numpy as np
import pytest

import oracle
from conftest import GOLDEN, reference_deck


def _trace():
    with open(os.path.join(GOLDEN, "iaea3d_trace.json")) as f:
        return json.load(f)


def test_iaea3d_trace_every_printed_digit():
    gold = _trace()
    o = oracle.Oracle(reference_deck("IAEA3Ds"))
    o.run()
    tr = {r.p: r for r in o.trace()}
    assert len(gold["rows"]) == 17
    for row in gold["rows"]:
        r = tr[row["p"]]
        # the reference prints with FORMAT (I5,F13.6,2ES15.5), mod_cmfd.f90:492
        assert "%.6f" % r.k == row["k"], row
        assert "%.5E" % r.ser == row["ser"], row
        assert "%.5E" % r.fer == row["fer"], row
    assert o.geti("outers") == gold["outers"] == 129
    assert "%.6f" % o.getd("Ke") == gold["keff"]
    nod = [r for r in o.trace() if r.nodal]
    assert nod[0].p == gold["nodal_at"]
    assert "%.5E" % nod[0].ndmax == gold["nodal"]["ndmax"]
    assert list(nod[0].loc) == gold["nodal"]["loc"]
    # extrapolation is printed before the row of outers 5, 20 (every nac=5)
    for p in gold["extrapolated_at"]:
        assert tr[p].extrapolated


@pytest.mark.parametrize("name", ["IAEA3Ds", "adjoint", "PNM", "FDM-1D", "DVP", "IAEA2D", "BIBLIS", "KOEBERG"])
def test_fixture_matches_fresh_oracle(name):
    fx = np.load(os.path.join(GOLDEN, "decks", name + ".npz"))
    o = oracle.Oracle(reference_deck(name))
    o.run()
    assert o.getd("Ke") == float(fx["out_k"])
    assert o.geti("outers") == int(fx["out_outers"])
    np.testing.assert_array_equal(o.powdis(), fx["out_power"])


@pytest.mark.parametrize("name,kref,tol_pcm", [("IAEA2D", 1.029585, 3.0), ("BIBLIS", 1.02511, 3.0),
                                                ("KOEBERG", 1.007954, 6.0)])
def test_benchmark_k_physics(name, kref, tol_pcm):
    """Benchmark k values quoted in the deck headers pin physics to ~pcm."""
    fx = np.load(os.path.join(GOLDEN, "decks", name + ".npz"))
    assert abs(float(fx["out_k"]) - kref) / kref * 1e5 < tol_pcm


def test_iaea3d_fixture_is_the_pinned_run():
    gold = _trace()
    fx = np.load(os.path.join(GOLDEN, "decks", "IAEA3Ds.npz"))
    k = fx["out_trace_k"]
    for row in gold["rows"]:
        assert "%.6f" % k[row["p"] - 1] == row["k"]


def test_out_of_scope_cards_are_rejected():
    with pytest.raises(oracle.OracleError) as e:
        oracle.Oracle(reference_deck("fixed_source"))
    assert e.value.code == oracle.ORA_ERR_UNSUPPORTED
