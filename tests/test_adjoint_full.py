"""dk/dSigma through the nodal update on the GPU, through the C ABI.

* adp_nodal_vjp (the reverse-mode derivative of one nodal update) against
  torch.autograd of the restated update (tests/nodal_ref.py) at the
  oracle's converged state: the adjoints of the flux, the coupling
  coefficients, k and the cross sections, on small cores with every
  boundary condition, ADFs, PNM and 4 groups; each output within 1e-9 of
  its largest entry.
* adp_adjoint_sens against the dense fixed-point derivative
  (tests/adjoint_full_ref.py, itself checked against the oracle's full-solve
  differences on the CPU): every entry within 1e-6 of its kind's largest.
* the 34x34x22-node two-group full core: 64 seeded parameters against
  central differences of the oracle's full solve (nodal update re-converged,
  tests/golden/adjoint_fd_full_core_3d.json): relative error <= 1e-3.
"""
import json
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import oracle
from adpres_gb300 import deck, synth
from adjoint_full_ref import FullAdjoint, converge_fixed_point, dkdp_layout
from nodal_ref import NodalRef

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
CORES = [("SANM", 1, 2, False, None), ("PNM", 4, 2, True, None), ("SANM", 3, 4, True, None),
         ("SANM", 5, 2, True, (2, 2, 2, 0, 2, 0)), ("SANM", 8, 2, False, (1, 1, 1, 1, 1, 1)),
         ("SANM", 9, 3, True, (0, 0, 0, 0, 0, 0)), ("PNM", 10, 1, False, None)]


def _core(text, **over):
    from adpres_gb300.core import Core
    return Core.from_deck(deck.parse(text), **over)


@pytest.mark.parametrize("kern,seed,ng,adf,bc", CORES)
def test_nodal_vjp_matches_autograd(kern, seed, ng, adf, bc):
    text = synth.small_core(seed=seed, ng=ng, kern=kern, adf=adf, bc=bc)
    o = oracle.Oracle(text=text)
    o.setd("serc", 1e-9)
    o.setd("ferc", 1e-9)
    o.run()
    R = NodalRef(o)
    phi, dnc, k = R.state()
    p = {a: v.clone().requires_grad_(True) for a, v in R.params().items()}
    phi_t = phi.clone().requires_grad_(True)
    dnc_t = dnc.clone().requires_grad_(True)
    k_t = torch.tensor(k, dtype=torch.float64, requires_grad=True)
    rng = np.random.default_rng(seed)
    lam = torch.tensor(rng.standard_normal((R.nn, R.ng, 6))) * R.canon[:, None, :]
    new = R.update(phi_t, dnc_t, k_t, p)
    (new * lam).sum().backward()
    ref_phi = phi_t.grad.numpy()
    ref_dn = (dnc_t.grad * R.canon[:, None, :]).numpy()
    ref_sig = dkdp_layout(p["D"].detach(), {a: v.grad for a, v in p.items()})
    c = _core(text)
    nn = R.nn
    c.set_state(f0=o.fortran("f0", (nn, ng)), fs0=o.array("fs0"), keff=k, dn=o.fortran("dn", (nn, ng, 6)))
    pb, db, kb, sb, res = c.nodal_vjp(lam.numpy())
    # the fixed-point residual max |N(state) - d| of the forward recompute
    ref_res = float((new.detach() - dnc).abs().max())
    assert abs(res - ref_res) <= 1e-10 * float(dnc.abs().max()), (res, ref_res)

    def close(a, b, what):
        scale = np.max(np.abs(b))
        assert np.max(np.abs(a - b)) <= 1e-9 * scale, (what, np.max(np.abs(a - b)), scale)

    close(pb, ref_phi, "phi")
    close(db, ref_dn, "dn")
    assert abs(kb - float(k_t.grad)) <= 1e-9 * abs(float(k_t.grad)) + 1e-15
    for col in range(4 + ng):
        if np.max(np.abs(ref_sig[:, :, col])) > 0:
            close(sb[:, :, col], ref_sig[:, :, col], "sigma column %d" % col)
        else:
            assert np.max(np.abs(sb[:, :, col])) == 0.0


@pytest.mark.parametrize("kern,seed,ng,adf,bc", CORES[:3] + CORES[4:6])
def test_fixed_point_sens_matches_dense_reference(kern, seed, ng, adf, bc):
    text = synth.small_core(seed=seed, ng=ng, kern=kern, adf=adf, bc=bc)
    o = oracle.Oracle(text=text)
    converge_fixed_point(o)
    A = FullAdjoint(o)
    ref, frozen, _ = A.sens()
    c = _core(text, serc=1e-12, ferc=1e-12)
    rep = c.outer(trace=False)
    assert rep.converged and abs(rep.keff - A.k) <= 1e-10
    S, psi, arep = c.adjoint_sens(tol=1e-12)
    assert arep.converged and arep.ndmax <= 1e-7
    print("%s seed %d: %d rounds, %d outers, fixed-point residual %.1e" % (kern, seed, arep.nodal_updates,
                                                                           arep.outers, arep.ndmax))
    for col in range(4 + ng):
        scale = np.max(np.abs(ref[:, :, col]))
        if scale == 0:
            assert np.max(np.abs(S[:, :, col])) == 0.0
            continue
        err = np.max(np.abs(S[:, :, col] - ref[:, :, col]))
        assert err <= 1e-6 * scale, (col, err / scale)
        # and it is not the frozen-dn derivative
        assert np.max(np.abs(frozen[:, :, col] - ref[:, :, col])) > 1e-3 * scale or col >= 4


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_full_core_3d_matches_full_solve_differences(precision):
    """34x34x22 nodes, 2 groups, SANM: 64 seeded parameters (sigtr, siga,
    nuf, sigs(1->2) of fuel nodes) against the oracle's central differences
    with the nodal update re-converged; bar 1e-3 relative.  The mixed
    handle runs its forward, adjoint and generalized-adjoint outers in the
    mixed kernel."""
    with open(os.path.join(HERE, "golden", "adjoint_fd_full_core_3d.json")) as f:
        fx = json.load(f)
    c = _core(synth.full_core_3d(0), serc=1e-12, ferc=1e-12, precision=precision)
    rep = c.outer(trace=False)
    assert rep.converged
    assert abs(rep.keff - fx["keff"]) <= 1e-10 * fx["keff"]
    S, _, arep = c.adjoint_sens(tol=1e-10)
    Sf, _, _ = c.adjoint_sens(tol=1e-12, frozen_dn=True)
    col = {"sigtr": 3, "siga": 1, "nuf": 2}
    worst, worst_frozen, rows = 0.0, 0.0, []
    for r in fx["params"]:
        n, g, h = r["n"], r["g"], r["h"]
        ci = 4 + h if r["kind"] == "sigs" else col[r["kind"]]
        an, fz = S[n, g, ci], Sf[n, g, ci]
        err = abs(an - r["fd"]) / abs(r["fd"])
        worst = max(worst, err)
        worst_frozen = max(worst_frozen, abs(fz - r["fd"]) / abs(r["fd"]))
        rows.append((r["kind"], n, g, an, r["fd"], err))
    print("full_core_3d %s: %d parameters, worst relative error %.2e (frozen dn %.2e); %d rounds, %d outers, "
          "%.1f ms" % (precision, len(rows), worst, worst_frozen, arep.nodal_updates, arep.outers, arep.device_ms))
    assert len(rows) == 64
    assert worst <= 1e-3, [x for x in rows if x[-1] > 1e-3]
