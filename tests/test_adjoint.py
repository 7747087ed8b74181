"""Discrete adjoint and dk/dSigma on the GPU, through the C ABI.

Checks, on the same inputs:
  * dk/dp at frozen dn (adp_adjoint_sens_frozen) against the dense restatement (tests/adjoint_ref.py)
    built from the oracle's assembled operators: every entry, 1e-6 of the
    largest entry of its kind;
  * against central finite differences of k at dn frozen (relative step
    1e-4): dense eigenvalues on small cores, warm-started GPU solves
    (ADP_FROZEN_DN) on the 34x34x22 two-group full core, <= 1e-3 relative;
  * for the FDM kernel (dn = 0, so frozen and full solves coincide): the
    adjoint flux against the reference's own adjoint (outer_ad) as
    psi = V phi*, and dk/dp against finite differences of the oracle's full
    solve, <= 1e-3 relative.
"""
import numpy as np
import pytest

import oracle
from adpres_gb300 import deck, synth
from adjoint_ref import Dense

pytestmark = pytest.mark.gpu

TIGHT = 1e-12
KINDS = ("D", "siga", "nuf", "sigtr")


def _gpu(text, precision="fp64", tol=TIGHT, **over):
    from adpres_gb300.core import Core
    dk = deck.parse(text)
    c = Core.from_deck(dk, precision=precision, serc=tol, ferc=tol, **over)
    rep = c.outer()
    assert rep.converged
    return dk, c, rep


def _oracle(text, tol=TIGHT):
    o = oracle.Oracle(text=text)
    o.setd("serc", tol)
    o.setd("ferc", tol)
    o.run()
    return o


def _node_tables(dk):
    m = dk.mat - 1
    return dict(sigtr=dk.xsigtr[m].copy(), siga=dk.xsiga[m].copy(), nuf=dk.xnuf[m].copy(), sigf=dk.xsigf[m].copy(),
                sigs=dk.xsigs[m].copy())


CASES = [("FDM", 6, 2, False), ("SANM", 1, 2, False), ("PNM", 4, 2, True), ("SANM", 3, 4, True)]


@pytest.mark.parametrize("kern,seed,ng,adf", CASES)
def test_sens_matches_dense_restatement(kern, seed, ng, adf):
    text = synth.small_core(seed=seed, ng=ng, kern=kern, adf=adf)
    dk, c, rep = _gpu(text)
    S, psi, arep = c.adjoint_sens(tol=TIGHT, frozen_dn=True)
    assert arep.converged
    # the discrete adjoint has the forward eigenvalue
    assert abs(arep.keff - rep.keff) <= 1e-10 * rep.keff
    o = _oracle(text)
    d = Dense(o)
    k, phi_d, psi_d = d.eig()
    assert abs(k - rep.keff) <= 1e-10 * k
    a, b = psi / psi.sum(), psi_d / psi_d.sum()   # both (nnod, ng)
    assert np.max(np.abs(a - b)) <= 1e-8 * np.max(np.abs(b))
    ref = d.analytic_sens(k, phi_d, psi_d)
    for cidx in range(4 + ng):
        scale = np.max(np.abs(ref[:, :, cidx]))
        if scale == 0:
            assert np.all(S[:, :, cidx] == 0)
            continue
        assert np.max(np.abs(S[:, :, cidx] - ref[:, :, cidx])) <= 1e-6 * scale, cidx


@pytest.mark.parametrize("kern,seed,ng,adf", CASES[:3])
def test_sens_matches_dense_fd_frozen_dn(kern, seed, ng, adf):
    """Central differences (relative step 1e-4) of the dense eigenvalue with
    the oracle's converged dn held fixed.  Only parameters whose k change at
    that step exceeds 1e-11 (1000x the dense eigenvalue's rounding) are
    compared."""
    text = synth.small_core(seed=seed, ng=ng, kern=kern, adf=adf)
    dk, c, rep = _gpu(text)
    S, _, _ = c.adjoint_sens(tol=TIGHT, frozen_dn=True)
    d = Dense(_oracle(text))
    rng = np.random.default_rng(100 + seed)
    checked, worst = 0, 0.0
    while checked < 16:
        n, g = int(rng.integers(d.nn)), int(rng.integers(d.ng))
        kind = KINDS[int(rng.integers(4))]
        p = d.o.fortran(kind, (d.nn, d.ng))[n, g]
        if p == 0 or abs(S[n, g, KINDS.index(kind)] * p * 1e-4) < 1e-11:
            continue
        fd = d.fd(kind, n, g, rel=1e-4)
        worst = max(worst, abs(S[n, g, KINDS.index(kind)] - fd) / abs(fd))
        checked += 1
    assert worst <= 1e-3, worst


def test_fdm_adjoint_flux_is_reference_adjoint_times_volume():
    """For the FDM kernel the discrete adjoint is psi = V phi*, phi* the
    reference's outer_ad flux: V A_g is symmetric and the local terms commute
    with V.  Normalised inner-product agreement 1 - cos <= 1e-6 (measured far
    below), and pointwise after normalisation."""
    for seed, ng in ((6, 2), (7, 4)):
        text = synth.small_core(seed=seed, ng=ng, kern="FDM")
        dk, c, rep = _gpu(text)
        _, psi, _ = c.adjoint_sens(tol=TIGHT)
        o = oracle.Oracle(text=text)
        o.setd("serc", TIGHT)
        o.setd("ferc", TIGHT)
        o.xs_updt()
        o.outer(adjoint=True, popt=1)
        nn = o.geti("nnod")
        phis = o.fortran("f0", (nn, ng))
        vps = phis * o.array("vdel")[:, None]
        a, b = psi.ravel(), vps.ravel()
        cos = float(a @ b) / (np.linalg.norm(a) * np.linalg.norm(b))
        assert 1.0 - cos <= 1e-6
        a, b = a / a.sum(), b / b.sum()
        assert np.max(np.abs(a - b)) <= 1e-6 * np.max(np.abs(b))


def test_fdm_sens_matches_fd_of_full_oracle_solve():
    """FDM: dn = 0, so dk/dp is the derivative of the reference's full solve.
    Central differences of the oracle's k (warm-started outer(), relative step
    1e-4, 1e-12 criteria)."""
    text = synth.small_core(seed=6, ng=2, kern="FDM")
    dk, c, rep = _gpu(text)
    S, _, _ = c.adjoint_sens(tol=TIGHT)
    o = _oracle(text)
    base = {a: o.array(a).copy() for a in ("f0", "fs0", "D", "sigr", "siga", "sigtr", "nuf", "sigs")}
    k0 = o.getd("Ke")
    nn, ng = o.geti("nnod"), o.geti("ng")

    def k_at(kind, n, g, rel):
        for a, v in base.items():
            o.set_array(a, v)
        o.setd("Ke", k0)
        a = o.fortran(kind, (nn, ng)).copy()
        a[n, g] *= 1.0 + rel
        o.set_array(kind, a.reshape(-1, order="F"))
        if kind != "nuf":
            o.dsigr_updt()
        o.outer(popt=1)
        return o.getd("Ke")

    rng = np.random.default_rng(7)
    checked, worst = 0, 0.0
    while checked < 12:
        n, g = int(rng.integers(nn)), int(rng.integers(ng))
        kind = ("siga", "nuf", "sigtr")[int(rng.integers(3))]
        p = o.fortran(kind, (nn, ng))[n, g]
        ci = KINDS.index(kind)
        if p == 0 or abs(S[n, g, ci] * p * 1e-4) < 1e-10:
            continue
        fd = (k_at(kind, n, g, 1e-4) - k_at(kind, n, g, -1e-4)) / (2e-4 * p)
        worst = max(worst, abs(S[n, g, ci] - fd) / abs(fd))
        checked += 1
    assert worst <= 1e-3, worst


def _frozen_fd(c, dk, tabs, state, kind, n, g, rel, h=None):
    """k of the GPU solve at dn frozen with one node parameter scaled by 1 + rel,
    warm-started from the converged state."""
    t = {a: v.copy() for a, v in tabs.items()}
    if kind == "sigs":
        t["sigs"][n, g, h] *= 1.0 + rel
    else:
        t[kind][n, g] *= 1.0 + rel
    c.xs_updt_nodes(t["sigtr"], t["siga"], t["nuf"], t["sigf"], dk.chi, dk.mat, t["sigs"], dk.dc)
    f0, fs0, k0, dn = state
    c.set_state(f0=f0, fs0=fs0, keff=k0, dn=dn)
    rep = c.outer(frozen_dn=True, trace=False)
    assert rep.converged
    return rep.keff


def test_full_core_3d_sens_matches_frozen_fd():
    """The 34x34x22-node two-group full core: 64 seeded parameters
    (D via sigtr, siga, nuf, sigs(1->2)), central differences at relative
    step 1e-4 of warm-started GPU FP64 solves with dn frozen, <= 1e-3."""
    text = synth.full_core_3d(0)
    dk, c, rep = _gpu(text, tol=1e-13)
    S, psi, arep = c.adjoint_sens(tol=1e-13, frozen_dn=True)
    assert arep.converged
    state = c.state()
    tabs = _node_tables(dk)
    nn, ng = len(dk.mat), dk.ng
    rng = np.random.default_rng(2024)
    worst, checked = 0.0, 0
    rows = []
    while checked < 64:
        n, g = int(rng.integers(nn)), int(rng.integers(ng))
        kind = ("sigtr", "siga", "nuf", "sigs")[checked % 4]
        h = None
        if kind == "sigs":
            g, h = 0, 1
            p = tabs["sigs"][n, g, h]
            an = S[n, g, 4 + h]
        else:
            p = tabs[kind][n, g]
            an = S[n, g, {"sigtr": 3, "siga": 1, "nuf": 2}[kind]]
        if p == 0 or abs(an * p * 1e-4) < 1e-12:
            continue
        kp = _frozen_fd(c, dk, tabs, state, kind, n, g, 1e-4, h)
        km = _frozen_fd(c, dk, tabs, state, kind, n, g, -1e-4, h)
        fd = (kp - km) / (2e-4 * p)
        err = abs(an - fd) / abs(fd)
        rows.append((kind, n, g, an, fd, err))
        worst = max(worst, err)
        checked += 1
    print("full_core_3d frozen-dn FD: worst relative error %.3e over %d parameters" % (worst, checked))
    assert worst <= 1e-3, [r for r in rows if r[-1] > 1e-3]


def test_mixed_precision_sens_close_to_fp64():
    text = synth.quarter_core_2d(1)
    _, c64, _ = _gpu(text, "fp64", tol=1e-10)
    S64, _, _ = c64.adjoint_sens(tol=1e-10, frozen_dn=True)
    _, c32, _ = _gpu(text, "mixed", tol=1e-10)
    S32, _, _ = c32.adjoint_sens(tol=1e-10, frozen_dn=True)
    for ci in range(S64.shape[2]):
        scale = np.max(np.abs(S64[:, :, ci]))
        if scale:
            assert np.max(np.abs(S32[:, :, ci] - S64[:, :, ci])) <= 1e-4 * scale, ci


def test_adjoint_requires_converged_forward():
    from adpres_gb300._lib import AdpError, ADP_ERR_STATE
    from adpres_gb300.core import Core
    dk = deck.parse(synth.small_core(seed=2, ng=2))
    c = Core.from_deck(dk)
    with pytest.raises(AdpError) as e:
        c.adjoint_sens()
    assert e.value.status == ADP_ERR_STATE
    c.outer()
    c.adjoint_sens()
    c.xs_updt(dk.xsigtr, dk.xsiga, dk.xnuf, dk.xsigf, dk.chi, dk.mat, dk.xsigs, dk.dc)
    with pytest.raises(AdpError) as e:
        c.adjoint_sens()
    assert e.value.status == ADP_ERR_STATE


def _cos(a, b):
    a, b = np.ravel(a), np.ravel(b)
    return float(a @ b) / (np.linalg.norm(a) * np.linalg.norm(b))


@pytest.mark.parametrize("kern,seed,ng,adf", [("SANM", 1, 2, False), ("PNM", 2, 2, True), ("SANM", 3, 4, True),
                                              ("FDM", 6, 2, False)])
def test_reference_adjoint_flux_inner_product(kern, seed, ng, adf):
    """The reference's own adjoint calculation (outer_ad with the adjoint
    nodal update, mod_cmfd.f90:602-699 and mod_nodal.f90:1392-1402), run on
    the GPU by adp_outer(ADP_ADJOINT), against the oracle's: normalised
    inner product 1 - cos <= 1e-6 (measured near rounding).  Beside it, the
    discrete adjoint psi of adp_adjoint_sens against V phi* of that
    reference adjoint: equal for FDM; for SANM/PNM the two are adjoints of
    different operators (the reference's physical adjoint takes the
    untransposed matrix with coupling coefficients from its own adjoint
    two-node problems, and its eigenvalue differs from the forward k), so
    1 - cos is printed and bounded at the value the dense restatement gives."""
    text = synth.small_core(seed=seed, ng=ng, kern=kern, adf=adf)
    o = oracle.Oracle(text=text)
    o.setd("serc", TIGHT)
    o.setd("ferc", TIGHT)
    o.xs_updt()
    o.outer(adjoint=True, popt=1)
    nn = o.geti("nnod")
    phis = o.fortran("f0", (nn, ng))
    from adpres_gb300.core import Core
    c = Core.from_deck(deck.parse(text), serc=TIGHT, ferc=TIGHT)
    rep = c.outer(adjoint=True, popt=1)
    assert rep.converged
    f0, _, _, _ = c.state()
    one_minus = 1.0 - _cos(f0, phis)
    assert one_minus <= 1e-6, one_minus
    # the discrete adjoint of the forward problem against V phi*
    c.reset()
    c.outer()
    _, psi, _ = c.adjoint_sens(tol=TIGHT, frozen_dn=True)
    d = Dense(_oracle(text))
    _, _, psi_d = d.eig()
    vps = phis * o.array("vdel")[:, None]
    gpu_gap, dense_gap = 1.0 - _cos(psi, vps), 1.0 - _cos(psi_d, vps)
    print("%s seed %d: reference adjoint GPU vs oracle 1-cos %.1e; discrete adjoint vs reference adjoint "
          "1-cos %.2e (dense restatement %.2e)" % (kern, seed, one_minus, gpu_gap, dense_gap))
    assert abs(gpu_gap - dense_gap) <= 1e-9
    if kern == "FDM":
        assert gpu_gap <= 1e-12
