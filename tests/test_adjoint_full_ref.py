"""CPU checks of the derivative through the nodal update (no GPU).

* tests/nodal_ref.py restates nodal_update / nodal_update_pnm
  (mod_nodal.f90:18-278) with torch tensors; its new dn equals the oracle's
  nodal_upd on SANM, PNM, ADF and 4-group cores with every boundary
  condition, to rounding.
* tests/adjoint_full_ref.py forms dk/dSigma of the nonlinear fixed point
  (CMFD eigenproblem + two-node update) from autograd partials and dense
  solves; it matches central differences of the oracle's full solve
  (relative step 1e-4, re-converged dn) to 1e-3, while the frozen-dn
  derivative misses them by 5 % to over 100 % on the same cores.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import oracle
from adpres_gb300 import synth
from adjoint_full_ref import STATE, FullAdjoint, converge_fixed_point, full_fd
from nodal_ref import NodalRef

CORES = [("SANM", 1, 2, False, None), ("PNM", 4, 2, True, None), ("SANM", 3, 4, True, None),
         ("SANM", 5, 2, True, (2, 2, 2, 0, 2, 0)), ("SANM", 8, 2, False, (1, 1, 1, 1, 1, 1)),
         ("SANM", 9, 3, True, (0, 0, 0, 0, 0, 0))]


@pytest.mark.parametrize("kern,seed,ng,adf,bc", CORES)
def test_torch_nodal_update_matches_oracle(kern, seed, ng, adf, bc):
    o = oracle.Oracle(text=synth.small_core(seed=seed, ng=ng, kern=kern, adf=adf, bc=bc))
    o.setd("serc", 1e-8)
    o.setd("ferc", 1e-8)
    o.run()
    R = NodalRef(o)
    phi, dnc, k = R.state()
    new = R.update(phi, dnc, k, R.params())
    o.nodal_upd(1)
    ref = R.to_canon(torch.tensor(o.fortran("dn", (R.nn, R.ng, 6))))
    assert float((new - ref).abs().max()) <= 1e-12 * float(ref.abs().max())
    # interior faces carry one coefficient in both nodes' slots
    assert float((R.expand(ref) - torch.tensor(o.fortran("dn", (R.nn, R.ng, 6)))).abs().max()) == 0.0


KIND_COL = {"sigtr": 3, "siga": 1, "nuf": 2}


def _pick(o, S, rng, nn, ng, count, floor):
    """Seeded parameters whose k change at the step is above the noise floor."""
    out = []
    tries = 0
    while len(out) < count and tries < 2000:
        tries += 1
        n, g = int(rng.integers(nn)), int(rng.integers(ng))
        kind = ("sigtr", "siga", "nuf", "sigs")[len(out) % 4]
        h = None
        if kind == "sigs":
            g, h = 0, 1
            p = o.fortran("sigs", (nn, ng, ng))[n, g, h]
            an = S[n, g, 4 + h]
        else:
            p = o.fortran(kind, (nn, ng))[n, g]
            an = S[n, g, KIND_COL[kind]]
        if p == 0 or abs(an * p * 1e-4) < floor:
            continue
        out.append((kind, n, g, h))
    return out


@pytest.mark.parametrize("kern,seed,ng,adf,bc", CORES[:3])
def test_full_derivative_matches_fd_of_full_oracle_solve(kern, seed, ng, adf, bc):
    o = oracle.Oracle(text=synth.small_core(seed=seed, ng=ng, kern=kern, adf=adf, bc=bc))
    converge_fixed_point(o)
    A = FullAdjoint(o)
    assert abs(A.k - A.k_oracle) <= 1e-11
    assert A.nodal_residual() <= 1e-7
    S, KS, _ = A.sens()
    base = {a: o.array(a).copy() for a in STATE}
    k0 = o.getd("Ke")
    rng = np.random.default_rng(seed)
    worst, worst_frozen = 0.0, 0.0
    for kind, n, g, h in _pick(o, S, rng, A.nn, ng, 8, 1e-9):
        fd = full_fd(o, kind, n, g, 1e-4, base, k0, h=h)
        col = 4 + h if kind == "sigs" else KIND_COL[kind]
        worst = max(worst, abs(S[n, g, col] - fd) / abs(fd))
        worst_frozen = max(worst_frozen, abs(KS[n, g, col] - fd) / abs(fd))
    print("%s seed %d: full %.2e, frozen-dn %.2e (relative to full-solve differences)" % (kern, seed, worst,
                                                                                         worst_frozen))
    assert worst <= 1e-3
    assert worst_frozen > 1e-2
