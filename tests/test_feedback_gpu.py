"""Critical boron search on the GPU (th::cbsearch, mod_th.f90:752-837)
against the oracle's search on the sample deck CBCsearch: each step is
XS_updt at the iterate on the device (adp_fb_updt) and a warm-started
adp_outer(popt = 0) through the C ABI.  The device update is checked
against the host restatement of XS_updt (feedback.xs_update) to the bit.

Bar, FP64 path: the same number of iterates; each iterate's boron within
0.01 ppm and k within 0.1 pcm of the oracle's; final nodal power within
1e-6 or 4x the oracle's own rounding sensitivity on this deck (the oracle
rebuilt with multiply-add contraction moves the final power by 1e-4: the
last step stops at ser < 1e-5).  Mixed path: the search converges (|k - 1|
< 1e-5) at a boron within 0.5 ppm of the oracle's (k's slope is about
10 pcm/ppm here).
"""
import copy

import numpy as np
import pytest

from adpres_gb300 import feedback
from adpres_gb300.core import Core, solve_deck
from feedback_fixture import deck_from_fixture, fixture

pytestmark = pytest.mark.gpu


def _max_rel(a, b):
    m = np.abs(b) > 0
    return float(np.max(np.abs(a[m] - b[m]) / np.abs(b[m])))


def test_cbsearch_fp64_matches_oracle():
    fx = fixture()
    dk = deck_from_fixture(fx)
    rep, p, core = solve_deck(dk, precision="fp64")
    it = core.bcsearch
    assert len(it) == len(fx["out_bcon"])
    bc = np.array([r[0] for r in it])
    k = np.array([r[1] for r in it])
    np.testing.assert_allclose(bc, fx["out_bcon"], rtol=0, atol=0.01)
    np.testing.assert_allclose(k, fx["out_k"], rtol=1e-6, atol=0)
    assert abs(rep.keff - 1.0) < 1e-5 and rep.ser < 1e-5 and rep.fer < 1e-5
    assert _max_rel(p, fx["out_power"]) <= max(1e-6, 4.0 * float(fx["sens_power_rel"]))
    # the first step starts cold and must take the oracle's outer count
    assert it[0][2] == int(fx["out_outers"][0])


def test_cbsearch_mixed_converges_to_the_same_boron():
    fx = fixture()
    dk = deck_from_fixture(fx)
    core = Core.from_deck(dk, precision="mixed")
    it = feedback.cbsearch(core, dk)
    b, k, _ = it[-1]
    assert abs(k - 1.0) < 1e-5
    assert abs(b - float(fx["out_bcon"][-1])) <= 0.5


def test_forward_deck_with_feedback_cards():
    """A FORWARD deck with the same cards solves once at the %CBCS reference
    boron (XS_updt(bcon, ftem, mtem, cden, bpos) before outer), which is the
    search's first step."""
    fx = fixture()
    dk = deck_from_fixture(fx, mode="FORWARD")
    rep, p, core = solve_deck(dk, precision="fp64")
    assert rep.converged
    assert abs(rep.keff - float(fx["out_k"][0])) / float(fx["out_k"][0]) * 1e5 <= 0.1
    assert rep.outers == int(fx["out_outers"][0])


def test_cbsearch_synthetic_core_matches_oracle():
    """The seeded full-core search deck (boron, temperatures, density, two rod
    banks with tips inside nodes), at a 9x9-assembly, 6-plane size."""
    import oracle
    from adpres_gb300 import deck, synth
    text = synth.boron_search_3d(0, n=9, planes=6)
    ref = oracle.Oracle(text=text).cbsearch()
    rep, p, core = solve_deck(deck.parse(text), precision="fp64")
    it = core.bcsearch
    assert len(it) == len(ref)
    np.testing.assert_allclose([r[0] for r in it], [r[0] for r in ref], rtol=0, atol=0.01)
    np.testing.assert_allclose([r[1] for r in it], [r[1] for r in ref], rtol=1e-6, atol=0)
    assert it[0][2] == ref[0][2]


def _solve_pair(dk, bcon, bpos):
    """The same solve with the node tables of the host restatement
    (feedback.xs_update + adp_xs_updt_nodes) and of the device update
    (adp_fb_set + adp_fb_updt)."""
    a = Core.from_deck(dk, precision="fp64")
    t = feedback.xs_update(dk, bcon, bpos)
    a.xs_updt_nodes(t["sigtr"], t["siga"], t["nuf"], t["sigf"], dk.chi, dk.mat, t["sigs"], dk.dc)
    ra = a.outer(popt=0, trace=False)
    b = Core.from_deck(dk, precision="fp64")
    b.fb_set(dk)
    b.fb_updt(dk, bcon=bcon, bpos=bpos)
    rb = b.outer(popt=0, trace=False)
    return ra, a.power(), rb, b.power()


@pytest.mark.parametrize("case", ["card", "partial", "all_in", "all_out", "clamped"])
def test_device_feedback_update_is_bit_identical(case):
    """adp_fb_updt forms the node tables with the operations of the host
    restatement in the same order: the solves agree to the bit, at the card's
    bank positions, with tips inside nodes, fully inserted and withdrawn
    banks, and with rod changes that drive rodded entries negative (clamped
    to 0)."""
    from adpres_gb300 import deck, synth
    dk = deck.parse(synth.boron_search_3d(1, n=9, planes=6))
    cr = dk.feedback["crod"]
    bpos = np.array(cr["bpos"], dtype=np.float64)
    bcon = 1234.5
    if case == "partial":
        bpos = bpos * 0.37 + 3.3
    elif case == "all_in":
        bpos[:] = 0.0
    elif case == "all_out":
        bpos[:] = float(cr["nstep"])
    elif case == "clamped":
        # rodded nodes lose their fission and scattering entirely
        ch = dict(cr["changes"])
        ch["nuf"] = ch["nuf"] - 10.0 * np.abs(dk.xnuf).max()
        ch["sigf"] = ch["sigf"] - 10.0 * np.abs(dk.xsigf).max()
        ch["sigs"] = ch["sigs"] - 10.0 * np.abs(dk.xsigs).max()
        cr["changes"] = ch
        bpos = bpos * 0.5
    ra, pa, rb, pb = _solve_pair(dk, bcon, bpos)
    assert ra.outers == rb.outers
    assert ra.keff == rb.keff
    assert np.array_equal(pa, pb)


def test_device_feedback_update_errors():
    from adpres_gb300 import deck, synth
    from adpres_gb300._lib import AdpError, ADP_ERR_INPUT, ADP_ERR_STATE
    dk = deck.parse(synth.boron_search_3d(0, n=9, planes=6))
    core = Core.from_deck(dk, precision="fp64")
    fresh = Core(dk.nxx, dk.nyy, dk.nzz, dk.ix, dk.iy, dk.iz, dk.xdel, dk.ydel, dk.zdel, dk.bc, dk.ng)
    with pytest.raises(AdpError) as e:
        fresh.fb_updt(dk)
    assert e.value.status == ADP_ERR_STATE
    # a non-finite bank position or a negative fuel temperature is an input error
    with pytest.raises(AdpError) as e:
        core.fb_updt(dk, bpos=np.full(int(dk.feedback["crod"]["nb"]), np.nan))
    assert e.value.status == ADP_ERR_INPUT
    ft = dict(dk.feedback["ftem"])
    ft["value"] = -1.0
    neg = dict(dk.feedback)
    neg["ftem"] = ft
    dkn = copy.copy(dk)
    dkn.feedback = neg
    with pytest.raises(AdpError) as e:
        core.fb_updt(dkn)
    assert e.value.status == ADP_ERR_INPUT
    core.fb_updt(dk)   # the handle stays usable
    assert core.outer(popt=0, trace=False).converged
    bad = dict(dk.feedback["crod"])
    bad["fbmap"] = np.asarray(bad["fbmap"]).copy()
    bad["fbmap"][0, 0] = int(bad["nb"]) + 1
    dk.feedback["crod"] = bad
    with pytest.raises(AdpError) as e:
        core.fb_set(dk)
    assert e.value.status == ADP_ERR_INPUT
