"""Dense restatement of dk/dSigma through the nodal update, for tests only.

The converged SANM/PNM state is the fixed point of two coupled equations
(mod_cmfd.f90:415-509 with the nodal update every nupd outers):

    M(Sigma, d) phi = (1/k) F(Sigma) phi          (CMFD eigenproblem, d frozen)
    d = N(phi, d, k; Sigma)                        (nodal_update, mod_nodal.f90)

with d the coupling coefficients of the faces.  With K(d, Sigma) the CMFD
eigenvalue and Phi(d, Sigma) its eigenvector, the fixed point is
d = G(d) = N(Phi(d), d, K(d)) and k = K(d*).  Its total derivative is

    dk/dSigma = K_S (1 + s) + N_S^T lam - Gam^T (M_S - F_S / k) phi
    lam = K_d^T (1 + s) + N_d^T lam - [Gam^T M_d phi]             (per face)
    (M - F/k)^T Gam = N_phi^T lam,   Gam^T F phi = 0,   s = N_k^T lam

where K_x = -k^2 psi^T (M_x - F_x/k) phi / (psi^T F phi) is the frozen-d
derivative and Gam the generalized adjoint of the eigenvector's response
(N is homogeneous of degree 0 in phi, so N_phi^T lam is orthogonal to phi
and the singular system has a solution).  Every partial derivative here
comes from torch.autograd through tests/nodal_ref.py; the eigenvectors and
Gam from dense solves; lam from GMRES.  It is the reference the CUDA
adjoint (adp_adjoint_sens in its full mode) is compared with, and it is
itself checked against central differences of the oracle's full solve.
"""
from __future__ import annotations

import numpy as np
import scipy.linalg
import scipy.sparse.linalg as sla
import torch

from nodal_ref import NodalRef


def _eig(M, F):
    w, vl, vr = scipy.linalg.eig(F, M, left=True, right=True)
    w = np.where(np.isfinite(w.real), w.real, -np.inf)
    i = int(np.argmax(w))
    phi, psi = np.real(vr[:, i]), np.real(vl[:, i])
    return float(w[i]), phi * np.sign(phi.sum()), psi * np.sign(psi.sum())


class FullAdjoint:
    def __init__(self, o):
        self.R = NodalRef(o)
        R = self.R
        self.nn, self.ng = R.nn, R.ng
        self.p = R.params()
        phi_o, self.dnc, k_o = R.state()
        M, F = R.operators(self.p, self.dnc)
        self.M, self.F = M.numpy(), F.numpy()
        k, phi, psi = _eig(self.M, self.F)
        self.k = k
        # the oracle's flux and the dense eigenvector agree to its convergence
        self.phi_vec = phi
        self.psi_vec = psi
        self.phi = torch.tensor(phi.reshape(self.ng, self.nn).T.copy())
        self.psi = torch.tensor(psi.reshape(self.ng, self.nn).T.copy())
        self.k_oracle = k_o
        self.Fphi = self.F @ phi

    # residual of the fixed point d = N(phi, d, k) at the state
    def nodal_residual(self):
        with torch.no_grad():
            new = self.R.update(self.phi, self.dnc, self.k, self.p)
        return float((new - self.dnc).abs().max())

    def _vec(self, a):
        return a.T.reshape(-1)    # (nn, ng) -> group-major vector

    def _mat(self, v):
        return torch.tensor(np.asarray(v).reshape(self.ng, self.nn).T.copy())

    # w^T (M - c F) phi and its gradient with respect to Sigma and d
    def contraction(self, w, c):
        p = {a: v.clone().requires_grad_(True) for a, v in self.p.items()}
        dnc = self.dnc.clone().requires_grad_(True)
        M, F = self.R.operators(p, dnc)
        wv = torch.tensor(self._vec(w).numpy() if isinstance(w, torch.Tensor) else w)
        phv = torch.tensor(self.phi_vec)
        val = wv @ (M @ phv) - c * (wv @ (F @ phv))
        val.backward()
        return {a: v.grad.detach() for a, v in p.items()}, dnc.grad.detach() * self.R.canon[:, None, :]

    def nvjp(self, lam):
        """lam^T N: gradients with respect to phi, d, k and Sigma."""
        p = {a: v.clone().requires_grad_(True) for a, v in self.p.items()}
        phi = self.phi.clone().requires_grad_(True)
        dnc = self.dnc.clone().requires_grad_(True)
        k = torch.tensor(self.k, dtype=torch.float64, requires_grad=True)
        new = self.R.update(phi, dnc, k, p)
        (new * lam).sum().backward()
        return (phi.grad.detach(), dnc.grad.detach() * self.R.canon[:, None, :], float(k.grad),
                {a: v.grad.detach() for a, v in p.items()})

    def gpt(self, v):
        """Gam with (M - F/k)^T Gam = v and Gam^T F phi = 0 (bordered dense solve)."""
        N = self.M.shape[0]
        Bm = np.zeros((N + 1, N + 1))
        Bm[:N, :N] = (self.M - self.F / self.k).T
        Bm[:N, N] = self.Fphi
        Bm[N, :N] = self.Fphi
        rhs = np.concatenate([v, [0.0]])
        x = np.linalg.solve(Bm, rhs)
        return x[:N]

    def sens(self, tol=1e-12):
        """(dk/dp (nn, ng, 4 + ng) through the nodal update, frozen-d part, lam)."""
        nn, ng = self.nn, self.ng
        k = self.k
        den = float(self.psi_vec @ self.Fphi)
        scale = -k * k / den
        gS, gd = self.contraction(self.psi, 1.0 / k)
        KS = {a: scale * v for a, v in gS.items()}
        Kd = scale * gd
        canon = self.R.canon[:, None, :].expand(nn, ng, 6)
        cidx = canon.reshape(-1).nonzero().squeeze(1)

        def unpack(x):
            out = torch.zeros(nn * ng * 6, dtype=torch.float64)
            out[cidx] = torch.tensor(x)
            return out.reshape(nn, ng, 6)

        def pack(t):
            return t.reshape(-1)[cidx].numpy()

        def gam_of(lam):
            vphi, vd, vk, vS = self.nvjp(lam)
            v = self._vec(vphi).numpy()
            return self.gpt(v), vd, vk, vS

        def op(x):
            lam = unpack(x)
            gam, vd, vk, _ = gam_of(lam)
            _, gdg = self.contraction(self._mat(gam), 0.0)
            return x - pack(Kd * vk + vd - gdg)

        n = len(cidx)
        A = sla.LinearOperator((n, n), matvec=op, dtype=np.float64)
        b = pack(Kd)
        x, info = sla.gmres(A, b, rtol=tol, atol=0.0, restart=200, maxiter=2000)
        if info != 0:
            raise RuntimeError("GMRES did not converge (%d)" % info)
        lam = unpack(x)
        gam, vd, s, vS = gam_of(lam)
        gG, _ = self.contraction(self._mat(gam), 1.0 / k)
        tot = {a: KS[a] * (1.0 + s) + vS[a] - gG[a] for a in KS}
        return self.layout(tot), self.layout(KS), lam

    def layout(self, g):
        return dkdp_layout(self.p["D"], g)


def dkdp_layout(D, g):
    """Gradients with respect to D, siga, nuf (nn, ng) and sigs (nn, ng, ng)
    in the dkdp layout (nn, ng, 4 + ng) of adp_adjoint_sens."""
    D = D.numpy()
    nn, ng = D.shape
    out = np.zeros((nn, ng, 4 + ng))
    out[:, :, 0] = g["D"].numpy()
    out[:, :, 1] = g["siga"].numpy()
    out[:, :, 2] = g["nuf"].numpy()
    out[:, :, 3] = -3.0 * D * D * out[:, :, 0]
    sg = g["sigs"].numpy()
    for h in range(ng):
        col = sg[:, :, h].copy()
        col[:, h] = 0.0
        out[:, :, 4 + h] = col
    return out


def converge_fixed_point(o, tol=1e-12, nupd=None):
    """Converge the oracle to the nonlinear fixed point: the deck's iteration,
    then, warm-started, with tight criteria (and nodal updates every `nupd`
    outers, the deck's interval by default: at every outer the two-node
    iteration of some cores is not stable, mod_nodal.f90:131-142)."""
    o.run()
    if nupd:
        o.seti("nupd", nupd)
    o.setd("serc", tol)
    o.setd("ferc", tol)
    o.outer(popt=1)


def full_fd(o, kind, n, g, rel, base, k0, h=None):
    """Central difference of the oracle's full solve (the criteria and nodal
    interval converge_fixed_point left set), warm-started from the fixed
    point in `base`."""
    nn, ng = o.geti("nnod"), o.geti("ng")
    out = []
    for r in (rel, -rel):
        for a, v in base.items():
            o.set_array(a, v)
        o.setd("Ke", k0)
        if kind == "sigs":
            a = o.fortran("sigs", (nn, ng, ng)).copy()
            a[n, g, h] *= 1.0 + r
        else:
            a = o.fortran(kind, (nn, ng)).copy()
            a[n, g] *= 1.0 + r
        o.set_array(kind, a.reshape(-1, order="F"))
        if kind != "nuf":
            o.dsigr_updt()
        o.outer(popt=1)
        out.append(o.getd("Ke"))
    for a, v in base.items():
        o.set_array(a, v)
    o.setd("Ke", k0)
    if kind == "sigs":
        p = base["sigs"].reshape((nn, ng, ng), order="F")[n, g, h]
    else:
        p = base[kind].reshape((nn, ng), order="F")[n, g]
    return (out[0] - out[1]) / (2.0 * rel * p)


STATE = ("f0", "fs0", "dn", "D", "sigr", "siga", "sigtr", "nuf", "sigs")
