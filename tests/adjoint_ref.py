"""Dense numpy restatement of the discrete adjoint, for tests only.

The operators come from the oracle: after a converged forward outer() its
assembled CMFD matrix (matrix_setup, mod_cmfd.f90:217-304, with the nodal
dn of the last update) is read back with ``matrix7``, and the scattering and
fission terms of TSrc (mod_cmfd.f90:1006-1033) are added from its node
cross sections, giving the generalized eigenproblem

    M phi = (1/k) F phi,   M = blockdiag(A_g) - S,   F = chi nuf^T (per node).

The fundamental mode and its left eigenvector come from a dense solve, so
k is exact to rounding and finite differences of k with dn frozen are
reliable at a relative step of 1e-4.  ``analytic_sens`` restates
dk/dp = k^2 psi^T (dF/dp / k - dM/dp) phi / (psi^T F phi) in plain loops.
"""
from __future__ import annotations

import numpy as np
import scipy.linalg

FACES = ((1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1))   # X+ X- Y+ Y- Z+ Z-


class Dense:
    def __init__(self, o):
        self.o = o
        self.ng, self.nn = o.geti("ng"), o.geti("nnod")
        self.ix, self.iy, self.iz = (o.array(a).astype(int) for a in ("ix", "iy", "iz"))
        self.pos = {(int(i), int(j), int(k)): n for n, (i, j, k) in enumerate(zip(self.ix, self.iy, self.iz))}
        self.xdel, self.ydel, self.zdel = o.array("xdel"), o.array("ydel"), o.array("zdel")
        self.bc = [o.geti(s) for s in ("xeast", "xwest", "ynorth", "ysouth", "ztop", "zbott")]
        # neighbour of each node across each face (-1 at the outline)
        self.nbr = np.full((self.nn, 6), -1, dtype=int)
        for n in range(self.nn):
            for f, (di, dj, dk) in enumerate(FACES):
                self.nbr[n, f] = self.pos.get((self.ix[n] + di, self.iy[n] + dj, self.iz[n] + dk), -1)

    def h(self, n, u):
        return (self.xdel[self.ix[n] - 1], self.ydel[self.iy[n] - 1], self.zdel[self.iz[n] - 1])[u]

    def operators(self):
        o, ng, nn = self.o, self.ng, self.nn
        A7 = o.matrix7()                                    # (ng, nn, 7): z- y- x- diag x+ y+ z+
        slot_face = {0: 5, 1: 3, 2: 1, 4: 0, 5: 2, 6: 4}
        M = np.zeros((ng * nn, ng * nn))
        for g in range(ng):
            for n in range(nn):
                r = g * nn + n
                M[r, r] = A7[g, n, 3]
                for c, f in slot_face.items():
                    m = self.nbr[n, f]
                    if m >= 0:
                        M[r, g * nn + m] += A7[g, n, c]
        sigs = o.fortran("sigs", (nn, ng, ng))               # sigs(n, g, h): g -> h
        nuf = o.fortran("nuf", (nn, ng))
        chi = o.fortran("chi", (o.geti("nmat"), ng))
        mat = o.array("mat").astype(int) - 1
        F = np.zeros_like(M)
        for g in range(ng):
            for h in range(ng):
                idx = np.arange(nn)
                if h != g:
                    M[g * nn + idx, h * nn + idx] -= sigs[:, h, g]
                F[g * nn + idx, h * nn + idx] = chi[mat, g] * nuf[:, h]
        return M, F

    def eig(self):
        """(k, phi, psi) of the fundamental mode, as (nn, ng) arrays."""
        M, F = self.operators()
        w, vl, vr = scipy.linalg.eig(F, M, left=True, right=True)
        w = np.real_if_close(w)
        i = int(np.argmax(np.where(np.isfinite(w.real), w.real, -np.inf)))
        k = float(w[i].real)
        phi = np.real(vr[:, i])
        psi = np.real(vl[:, i])
        phi = phi * np.sign(phi.sum())
        psi = psi * np.sign(psi.sum())
        return k, phi.reshape(self.ng, self.nn).T, psi.reshape(self.ng, self.nn).T

    def k_only(self):
        M, F = self.operators()
        w = scipy.linalg.eigvals(F, M)
        w = w[np.isfinite(w)]
        return float(np.max(w.real))

    # -- perturbations with dn frozen (matrix_setup(1) keeps nod%dn) ----------
    def perturbed_k(self, kind, n, g, rel, h=None):
        o, nn, ng = self.o, self.nn, self.ng
        names = {"D": "D", "siga": "siga", "nuf": "nuf", "sigtr": "sigtr", "sigs": "sigs"}
        name = names[kind]
        shape = (nn, ng, ng) if kind == "sigs" else (nn, ng)
        base = o.fortran(name, shape).copy()
        saved = {a: o.array(a).copy() for a in ("D", "sigr")}
        a = base.copy()
        if kind == "sigs":
            a[n, g, h] *= 1.0 + rel
        else:
            a[n, g] *= 1.0 + rel
        o.set_array(name, a.reshape(-1, order="F"))
        if kind in ("siga", "sigtr", "sigs"):
            o.dsigr_updt()                                  # D = 1/(3 sigtr), sigr = siga + sum sigs
        o.matrix_setup(1)
        k = self.k_only()
        o.set_array(name, base.reshape(-1, order="F"))
        for nm, v in saved.items():
            o.set_array(nm, v)
        o.matrix_setup(1)
        return k

    def fd(self, kind, n, g, rel=1e-4, h=None):
        """Central difference dk/dp with dn frozen."""
        shape = (self.nn, self.ng, self.ng) if kind == "sigs" else (self.nn, self.ng)
        p = self.o.fortran(kind, shape)[(n, g, h) if kind == "sigs" else (n, g)]
        kp = self.perturbed_k(kind, n, g, rel, h)
        km = self.perturbed_k(kind, n, g, -rel, h)
        return (kp - km) / (2.0 * rel * p)

    # -- the contraction, in loops -------------------------------------------
    def analytic_sens(self, k, phi, psi):
        o, nn, ng = self.o, self.nn, self.ng
        D = o.fortran("D", (nn, ng))
        nuf = o.fortran("nuf", (nn, ng))
        chi = o.fortran("chi", (o.geti("nmat"), ng))
        mat = o.array("mat").astype(int) - 1
        chin = chi[mat]
        den = float(np.sum((chin * psi).sum(1) * (nuf * phi).sum(1)))
        scale = k * k / den
        out = np.zeros((nn, ng, 4 + ng))
        for n in range(nn):
            fsa = float(np.dot(chin[n], psi[n]))
            for g in range(ng):
                nD = 0.0
                for f in range(6):
                    u = f // 2
                    hn = self.h(n, u)
                    m = self.nbr[n, f]
                    Dn = D[n, g]
                    if m >= 0:
                        Dm, hm = D[m, g], self.h(m, u)
                        d = 2.0 * Dm * Dm * hn / (Dn * hm + Dm * hn) ** 2
                        nD += d * (psi[n, g] * (phi[n, g] - phi[m, g]) / hn + psi[m, g] * (phi[m, g] - phi[n, g]) / hm)
                    else:
                        bc = self.bc[f]
                        if bc == 0:
                            alb = 1e30
                            d = 2.0 * alb * alb * hn / (2.0 * Dn + alb * hn) ** 2
                        elif bc == 1:
                            d = 0.5 * hn / (2.0 * Dn + 0.5 * hn) ** 2
                        else:
                            d = 0.0
                        nD += d * psi[n, g] * phi[n, g] / hn
                out[n, g, 0] = -nD * scale
                out[n, g, 1] = -psi[n, g] * phi[n, g] * scale
                out[n, g, 2] = fsa * phi[n, g] * scale / k
                out[n, g, 3] = -3.0 * D[n, g] ** 2 * out[n, g, 0]
                for h in range(ng):
                    if h != g:
                        out[n, g, 4 + h] = -(psi[n, g] - psi[n, h]) * phi[n, g] * scale
        return out
