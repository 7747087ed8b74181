"""Rod ejection transient on the GPU (rod_eject, mod_trans.f90:17-160):
the steady state, KNE1, the adjoint weight, then every time step's
outer_tr on the FP64 kernel (the mixed kernel for a mixed-precision
handle) with the nodal update in its transient form, against the oracle.

Bar: the reactivity at t = 0 within 1e-8 (absolute); per step the relative
power within 1e-6 or 4x the oracle's own rounding sensitivity (the oracle
rebuilt with multiply-add contraction: each step stops at ser, fer < 1e-5,
and on LMW that moves the power by up to 3.3e-3 over 240 steps), the
reactivity in dollars likewise; no step reaches nout where the oracle's
does not.
"""
import numpy as np
import pytest

from adpres_gb300 import deck, synth
from adpres_gb300._lib import AdpError, ADP_ERR_STATE
from adpres_gb300.core import Core
from adpres_gb300.transient import rod_eject
from feedback_fixture import deck_from_fixture, fixture

pytestmark = pytest.mark.gpu


def _compare(rec, t, rho, pw, sens_rho, sens_pow):
    assert len(rec) == len(t)
    np.testing.assert_allclose([r[0] for r in rec], t, rtol=0, atol=1e-12)
    assert abs(rec[0][1] - rho[0]) <= 1e-8
    got_p = np.array([r[2] for r in rec])
    got_r = np.array([r[1] for r in rec[1:]])
    tol_p = max(1e-6, 4.0 * sens_pow)
    tol_r = max(1e-6, 4.0 * sens_rho)
    assert float(np.max(np.abs(got_p - pw) / pw)) <= tol_p
    assert float(np.max(np.abs(got_r - rho[1:]))) <= tol_r


def test_lmw_matches_oracle():
    fx = fixture("LMW")
    dk = deck_from_fixture(fx, mode="RODEJECT")
    core = Core.from_deck(dk, precision="fp64")
    rec = rod_eject(core, dk)
    sens_pow = float(np.max(np.abs(fx["sens_pow"] - fx["out_pow"]) / fx["out_pow"]))
    sens_rho = float(np.max(np.abs(fx["sens_rho"][1:] - fx["out_rho"][1:])))
    _compare(rec, fx["out_t"], fx["out_rho"], fx["out_pow"], sens_rho, sens_pow)
    assert not any(r[3] for r in rec) and not fx["out_maxi"].any()


@pytest.mark.parametrize("extr", [False, True])
def test_synthetic_ejection_matches_oracle(extr):
    """With %EXTR the steps also carry the exponential flux extrapolation:
    omega = ln(f0 / ft) / dt from the second step on (rod_eject,
    mod_trans.f90:120-156), used by trans_calc's removal and sources."""
    import oracle
    text = synth.rod_ejection_3d(0, n=9, planes=6, extr=extr)
    ref = oracle.Oracle(text=text).rodeject()
    sens = oracle.Oracle(text=text, variant="fma").rodeject()
    pw = np.array([r[2] for r in ref])
    rho = np.array([r[1] for r in ref])
    sens_pow = float(np.max(np.abs(np.array([r[2] for r in sens]) - pw) / pw))
    sens_rho = float(np.max(np.abs(np.array([r[1] for r in sens[1:]]) - rho[1:])))
    dk = deck.parse(text)
    core = Core.from_deck(dk, precision="fp64")
    rec = rod_eject(core, dk)
    _compare(rec, [r[0] for r in ref], rho, pw, sens_rho, sens_pow)


def test_lmw_mixed_matches_oracle_within_its_rounding_sensitivity():
    """A mixed-precision handle runs its transient steps on the mixed
    kernel (FP32 Krylov steps, double-float defect with the step's external
    source; nodal update in FP64).  On LMW, whose 241 loosely converged
    steps move the oracle's own power by 3.3e-3 under a change of rounding,
    it stays within the FP64 path's bars (4x that sensitivity)."""
    fx = fixture("LMW")
    dk = deck_from_fixture(fx, mode="RODEJECT")
    core = Core.from_deck(dk, precision="mixed")
    rec = rod_eject(core, dk)
    sens_pow = float(np.max(np.abs(fx["sens_pow"] - fx["out_pow"]) / fx["out_pow"]))
    sens_rho = float(np.max(np.abs(fx["sens_rho"][1:] - fx["out_rho"][1:])))
    _compare(rec, fx["out_t"], fx["out_rho"], fx["out_pow"], sens_rho, sens_pow)
    assert not any(r[3] for r in rec)


@pytest.mark.parametrize("extr", [False, True])
def test_synthetic_ejection_mixed_matches_fp64(extr):
    """Mixed against FP64 handles on the synthetic ejection: the same
    outers, power within 1e-6 and reactivity within 1e-8 dollars at every
    step (measured: 1e-8 and 8e-10)."""
    dk = deck.parse(synth.rod_ejection_3d(0, n=9, planes=6, extr=extr))
    out = {}
    for prec in ("fp64", "mixed"):
        core = Core.from_deck(dk, precision=prec)
        out[prec] = rod_eject(core, dk)
        core.close()
    a, b = out["fp64"], out["mixed"]
    assert len(a) == len(b)
    pa, pb = np.array([r[2] for r in a]), np.array([r[2] for r in b])
    assert float(np.max(np.abs(pb - pa) / pa)) <= 1e-6
    assert float(np.max(np.abs(np.array([r[1] for r in b]) - np.array([r[1] for r in a])))) <= 1e-8
    assert [r[4] for r in a] == [r[4] for r in b]
    assert not any(r[3] for r in b)


def test_step_before_init_is_refused():
    dk = deck.parse(synth.rod_ejection_3d(0, n=9, planes=6))
    core = Core.from_deck(dk, precision="fp64")
    core.outer(popt=0, trace=False)
    with pytest.raises(AdpError) as e:
        core.trans_step(0.01, 0)
    assert e.value.status == ADP_ERR_STATE
