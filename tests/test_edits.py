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
