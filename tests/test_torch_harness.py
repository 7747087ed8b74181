"""A thin torch.autograd.Function over the C ABI (test harness only).

forward: adp_xs_updt_nodes + adp_outer -> k.  backward: adp_adjoint_sens
(dk/dp of the fixed point, through the nodal update for SANM/PNM)
contracted with the incoming gradient.  The check differentiates k with
respect to per-material log-scalings of siga, nuf and sigtr through
ordinary torch operations, and compares with central differences of full
solves, for the FDM, SANM and PNM kernels.
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


@pytest.mark.parametrize("kern,seed,rtol", [("FDM", 6, 1e-4), ("SANM", 1, 1e-3), ("PNM", 4, 1e-3)])
def test_autograd_gradient_matches_fd_of_full_solves(kern, seed, rtol):
    """k through per-material log-scalings of sigtr, siga and nuf: the
    backward pass is adp_adjoint_sens (for SANM/PNM the derivative of the
    fixed point through the nodal update), the check central differences of
    full solves (cold start, criteria 1e-12; the nodal update re-converged
    in each)."""
    from adpres_gb300.core import Core
    dk = deck.parse(synth.small_core(seed=seed, ng=2, kern=kern, adf=(kern == "PNM")))
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
    worst = 0.0
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
            worst = max(worst, abs(grad[a, b] - fd) / abs(fd))
            assert abs(grad[a, b] - fd) <= rtol * abs(fd) + 1e-12, (a, b, grad[a, b], fd)
    print("%s: autograd vs full-solve differences, worst relative %.1e" % (kern, worst))
