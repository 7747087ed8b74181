"""CPU checks of the oracle's restatement of the output edits: the
normalisations of mod_io.f90 (assemblies or regions with power average 1;
the forward AsmFlux scaling makes each group's positive assemblies sum to
1), the first-maximum rule, and the layouts."""
import numpy as np

import oracle
from adpres_gb300 import synth


def _solved(text):
    o = oracle.Oracle(text=text)
    o.run()
    return o


def test_asmpow_and_axipow_normalisation():
    o = _solved(synth.small_core(seed=5, ng=2, nz=4))
    p = o.powdis()
    fa, (im, jm) = o.asmpow(p)
    assert fa.shape == (o.geti("nx"), o.geti("ny"))
    pos = fa[fa > 0]
    assert abs(pos.mean() - 1.0) < 1e-12
    assert fa[im - 1, jm - 1] == fa.max()
    ax, km = o.axipow(p)
    assert ax.shape == (o.geti("nz"),)
    assert abs(ax[ax > 0].mean() - 1.0) < 1e-12
    assert ax[km - 1] == ax.max()


def test_asmflux_forward_scaling():
    o = _solved(synth.small_core(seed=6, ng=3))
    fa, neg = o.asmflux(norm=1.0)
    assert not neg
    for g in range(o.geti("ng")):
        assert abs(fa[:, :, g][fa[:, :, g] > 0].sum() - 1.0) < 1e-12
    raw, _ = o.asmflux(norm=0.0)
    assert np.all(raw >= 0)


def test_reactivity_of_a_converged_state_is_one_minus_one_over_k():
    """mod_trans.f90:648-688: at the converged static state the weighted
    balance gives rho = 1 - 1/k whatever the weight."""
    o = oracle.Oracle(text=synth.small_core(seed=5, ng=2))
    o.setd("serc", 1e-12)
    o.setd("ferc", 1e-12)
    o.run()
    nn, ng = o.geti("nnod"), o.geti("ng")
    k = o.getd("Ke")
    rng = np.random.default_rng(0)
    for af in (np.ones((nn, ng)), rng.uniform(0.5, 2.0, (nn, ng))):
        assert abs(o.reactivity(af) - (1 - 1 / k)) < 1e-10


def test_calc_beta_uniform_fractions():
    o = _solved(synth.small_core(seed=5, ng=2))
    nn, ng, nm = o.geti("nnod"), o.geti("ng"), o.geti("nmat")
    ib = np.tile([0.0002, 0.001, 0.002], (nm, 1))
    assert abs(o.calc_beta(np.ones((nn, ng)), ib) - 0.0032) < 1e-15
