"""A thin torch.autograd.Function over the C ABI (test harness only).

forward: adp_xs_updt_nodes + adp_outer -> k.  backward: adp_adjoint_sens
(dk/dp at dn frozen) contracted with the incoming gradient.  The check
differentiates k with respect to per-material log-scalings of siga, nuf and
sigtr through ordinary torch operations, and compares with central
differences of full solves; the FDM kernel is used so that the frozen-dn
gradient is the full solve's gradient.
"""
import numpy as np
import pytest

from adpres_gb300 import deck, synth

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = 1e-12


class Keff(torch.autograd.Function):
    @staticmethod
    def forward(ctx, sigtr, siga, nuf, sigs, core, dk):
        core.xs_updt_nodes(sigtr.detach().numpy(), siga.detach().numpy(), nuf.detach().numpy(),
                           dk.xsigf[dk.mat - 1], dk.chi, dk.mat, sigs.detach().numpy(), dk.dc)
        core.reset()
        rep = core.outer(trace=False)
        S, _, _ = core.adjoint_sens(tol=TOL)
        ctx.save_for_backward(torch.from_numpy(S))
        return torch.tensor(rep.keff, dtype=torch.float64)

    @staticmethod
    def backward(ctx, gk):
        (S,) = ctx.saved_tensors
        return gk * S[:, :, 3], gk * S[:, :, 1], gk * S[:, :, 2], gk * S[:, :, 4:], None, None


def _k_of_theta(theta, base, core, dk):
    m = torch.from_numpy(dk.mat - 1)
    f = torch.exp(theta)                                 # (nmat, 3)
    sigtr = base["sigtr"] * f[m, 0:1]
    siga = base["siga"] * f[m, 1:2]
    nuf = base["nuf"] * f[m, 2:3]
    return Keff.apply(sigtr, siga, nuf, base["sigs"], core, dk)


def test_autograd_gradient_matches_fd_of_full_solves():
    from adpres_gb300.core import Core
    dk = deck.parse(synth.small_core(seed=6, ng=2, kern="FDM"))
    core = Core.from_deck(dk, serc=TOL, ferc=TOL)
    m = dk.mat - 1
    base = {k: torch.from_numpy(np.ascontiguousarray(v[m])) for k, v in
            (("sigtr", dk.xsigtr), ("siga", dk.xsiga), ("nuf", dk.xnuf), ("sigs", dk.xsigs))}
    nmat = dk.xsigtr.shape[0]
    theta = torch.zeros((nmat, 3), dtype=torch.float64, requires_grad=True)
    k = _k_of_theta(theta, base, core, dk)
    k.backward()
    grad = theta.grad.numpy().copy()
    step = 1e-4
    for a in range(nmat):
        for b in range(3):
            if b == 2 and not np.any(dk.xnuf[a]):
                assert grad[a, b] == 0.0
                continue
            t = torch.zeros((nmat, 3), dtype=torch.float64)
            t[a, b] = step
            kp = float(_k_of_theta(t, base, core, dk))
            km = float(_k_of_theta(-t, base, core, dk))
            fd = (kp - km) / (2 * step)
            assert abs(grad[a, b] - fd) <= 1e-4 * abs(fd) + 1e-12, (a, b, grad[a, b], fd)
