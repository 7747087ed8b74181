"""Output edits AsmPow, AxiPow and AsmFlux (mod_io.f90:3267-3644).

GPU: the device edits of the oracle's own converged flux (handed over with
adp_set_state) against the oracle's restatement of the edits, and on the
GPU's own solution.  The column and assembly sums follow the reference's
order; only PowDis's total and the per-plane sums of AxiPow are grouped
differently, so the bar is 1e-12 relative.
"""
import numpy as np
import pytest

import oracle
from adpres_gb300 import deck, synth

pytestmark = pytest.mark.gpu

DECKS = [lambda: synth.small_core(seed=3, ng=4, adf=True), lambda: synth.quarter_core_2d(0),
         lambda: synth.full_core_3d(0)]


def _pair(text):
    from adpres_gb300.core import Core
    o = oracle.Oracle(text=text)
    o.run()
    c = Core.from_deck(deck.parse(text))
    nn, ng = o.geti("nnod"), o.geti("ng")
    c.set_state(f0=o.fortran("f0", (nn, ng)), keff=o.getd("Ke"))
    return o, c


@pytest.mark.parametrize("mk", DECKS)
def test_edits_match_oracle_on_the_same_flux(mk):
    o, c = _pair(mk())
    p = o.powdis()
    fa_o, loc_o = o.asmpow(p)
    fa_g, loc_g = c.asmpow()
    np.testing.assert_allclose(fa_g, fa_o, rtol=1e-12, atol=1e-15)
    assert loc_g == loc_o
    ax_o, k_o = o.axipow(p)
    ax_g, k_g = c.axipow()
    np.testing.assert_allclose(ax_g, ax_o, rtol=1e-12)
    assert k_g == k_o
    ff_o, neg_o = o.asmflux(norm=1.0)
    ff_g, neg_g = c.asmflux(norm=1.0)
    np.testing.assert_allclose(ff_g, ff_o, rtol=1e-12, atol=1e-300)
    assert neg_g == neg_o


def test_edits_on_gpu_solution_close_to_oracle():
    text = synth.quarter_core_2d(1)
    from adpres_gb300.core import Core
    o = oracle.Oracle(text=text)
    o.run()
    c = Core.from_deck(deck.parse(text))
    c.outer(trace=False)
    fa_o, loc_o = o.asmpow(o.powdis())
    fa_g, loc_g = c.asmpow()
    np.testing.assert_allclose(fa_g, fa_o, rtol=1e-6, atol=1e-9)
    ax_o, _ = o.axipow(o.powdis())
    ax_g, _ = c.axipow()
    np.testing.assert_allclose(ax_g, ax_o, rtol=1e-6)


def test_edit_rejects_bad_divisions():
    from adpres_gb300._lib import AdpError, ADP_ERR_INPUT
    o, c = _pair(synth.small_core(seed=1, ng=2))
    dk = c.deck
    bad = list(dk.extra["xdiv"])
    bad[0] += 1
    with pytest.raises(AdpError) as e:
        c.asmpow(xdiv=bad)
    assert e.value.status == ADP_ERR_INPUT


def test_reactivity_and_beta_match_oracle():
    """adp_reactivity / adp_core_beta on the oracle's converged state against
    the oracle's restatement (weights: the reference's own adjoint flux and
    a seeded field)."""
    text = synth.small_core(seed=7, ng=3, adf=True)
    o, c = _pair(text)
    nn, ng, nm = o.geti("nnod"), o.geti("ng"), o.geti("nmat")
    # the GPU handle needs the oracle's dn and fission source for the leakage and sources
    c.set_state(f0=o.fortran("f0", (nn, ng)), fs0=o.array("fs0"), keff=o.getd("Ke"),
                dn=o.fortran("dn", (nn, ng, 6)))
    c.outer(frozen_dn=True, trace=False)   # df/A on the handle; one frozen solve from the oracle's state
    c.set_state(f0=o.fortran("f0", (nn, ng)), fs0=o.array("fs0"), keff=o.getd("Ke"),
                dn=o.fortran("dn", (nn, ng, 6)))
    rng = np.random.default_rng(3)
    for af in (np.ones((nn, ng)), rng.uniform(0.2, 3.0, (nn, ng))):
        assert abs(c.reactivity(af) - o.reactivity(af)) <= 1e-12 * max(1.0, abs(o.reactivity(af)))
    ib = rng.uniform(1e-4, 2e-3, (nm, 6))
    af = rng.uniform(0.2, 3.0, (nn, ng))
    dk = c.deck
    assert abs(c.core_beta(af, ib, dk.mat) - o.calc_beta(af, ib)) <= 1e-13


def test_reactivity_static_identity_on_gpu_solution():
    from adpres_gb300.core import Core
    c = Core.from_deck(deck.parse(synth.quarter_core_2d(0)), serc=1e-12, ferc=1e-12)
    rep = c.outer(trace=False)
    S, psi, _ = c.adjoint_sens(tol=1e-12, frozen_dn=True)
    nn, ng = c.nnod, c.ng
    for af in (np.ones((nn, ng)), psi):
        assert abs(c.reactivity(af) - (1 - 1 / rep.keff)) < 1e-9
