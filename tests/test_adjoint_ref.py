"""CPU checks of the dk/dSigma formula that the adjoint kernels implement.

The dense restatement (tests/adjoint_ref.py) contracts the left and right
eigenvectors of the oracle's assembled CMFD operators; here it is checked
against central differences of the dense eigenvalue with dn frozen, and,
for the FDM kernel (dn = 0), against differences of the oracle's full
solve.  The derivative through the nodal update (SANM/PNM), which the
frozen-dn formula leaves out, is checked in tests/test_adjoint_full_ref.py.
"""
import numpy as np
import pytest

import oracle
from adpres_gb300 import synth
from adjoint_ref import Dense

KINDS = ("D", "siga", "nuf", "sigtr")


def _dense(kern, seed, ng, tol=1e-12, **kw):
    o = oracle.Oracle(text=synth.small_core(seed=seed, ng=ng, kern=kern, **kw))
    o.setd("serc", tol)
    o.setd("ferc", tol)
    o.run()
    return Dense(o)


@pytest.mark.parametrize("kern,seed", [("FDM", 6), ("SANM", 1)])
def test_formula_matches_dense_fd_frozen_dn(kern, seed):
    d = _dense(kern, seed, 2)
    k, phi, psi = d.eig()
    assert abs(k - d.o.getd("Ke")) <= 1e-11
    S = d.analytic_sens(k, phi, psi)
    rng = np.random.default_rng(seed)
    checked = 0
    while checked < 8:
        n, g = int(rng.integers(d.nn)), int(rng.integers(d.ng))
        kind = KINDS[checked % 4]
        p = d.o.fortran(kind, (d.nn, d.ng))[n, g]
        if p == 0 or abs(S[n, g, KINDS.index(kind)] * p * 1e-3) < 1e-11:
            continue
        fd = d.fd(kind, n, g, rel=1e-3)
        assert abs(S[n, g, KINDS.index(kind)] - fd) <= 1e-3 * abs(fd), (kind, n, g)
        checked += 1
    # the g -> h scattering enters sigr and the scattering source
    n = int(np.argmax(phi[:, 0]))
    fd = d.fd("sigs", n, 0, rel=1e-3, h=1)
    assert abs(S[n, 0, 5] - fd) <= 1e-3 * abs(fd)


def _full_fd(d, kind, n, g, rel, base, k0):
    o = d.o
    out = []
    for r in (rel, -rel):
        for a, v in base.items():
            o.set_array(a, v)
        o.setd("Ke", k0)
        a = o.fortran(kind, (d.nn, d.ng)).copy()
        a[n, g] *= 1.0 + r
        o.set_array(kind, a.reshape(-1, order="F"))
        if kind != "nuf":
            o.dsigr_updt()
        o.outer(popt=1)
        out.append(o.getd("Ke"))
    p = base[kind].reshape((d.nn, d.ng), order="F")[n, g]
    for a, v in base.items():
        o.set_array(a, v)
    return (out[0] - out[1]) / (2.0 * rel * p)


def test_fdm_formula_matches_fd_of_full_solve():
    d = _dense("FDM", 6, 2)
    k, phi, psi = d.eig()
    S = d.analytic_sens(k, phi, psi)
    base = {a: d.o.array(a).copy() for a in ("f0", "fs0", "D", "sigr", "siga", "sigtr", "nuf", "sigs")}
    k0 = d.o.getd("Ke")
    for n, g, kind in ((int(np.argmax(phi[:, 1])), 1, "siga"), (int(np.argmax(phi[:, 0])), 0, "nuf"),
                       (int(np.argmax(phi[:, 0])), 0, "sigtr")):
        fd = _full_fd(d, kind, n, g, 1e-3, base, k0)
        assert abs(S[n, g, KINDS.index(kind)] - fd) <= 1e-3 * abs(fd), kind
