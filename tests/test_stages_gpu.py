"""Per-stage parity on tiny grids: each stage of the path on the GPU
against the oracle's routine on the same state, on 3x3x2-node cores with a
cut corner (ragged rows), ADFs != 1 and every combination of the three
boundary conditions on the six faces.

  matrix_setup(1) with coup_coef   adp_get_matrix        vs ora matrix7
  get_source / Lxyz                adp_get_nodal_sources vs S1, S2, S3
  one nodal update (get_B ... nodal_coup_upd, ndmax and its location)
                                   adp_nodal_step        vs nodal_upd(1)
  PowDis                           adp_power             vs powdis

The state is seeded and arbitrary (a positive flux, coupling coefficients
of either sign, k = 1.05): each routine is a function of it, so any state
exercises every branch that the geometry reaches.
"""
import itertools

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import oracle
from adpres_gb300 import deck, synth
from nodal_ref import NodalRef

pytestmark = pytest.mark.gpu

ALL_BC = list(itertools.product(range(3), repeat=6))


def _case(bc, ng, kern, seed):
    text = synth.small_core(seed=seed, ng=ng, kern=kern, nx=3, ny=3, nz=2, xdiv=1, ydiv=1, zdiv=1, ragged=True,
                            adf=True, bc=bc)
    o = oracle.Oracle(text=text)
    o.xs_updt()
    o.outer(popt=1, max_outers=1)        # allocates the state arrays; overwritten below
    R = NodalRef(o)
    nn = R.nn
    rng = np.random.default_rng(seed)
    f0 = rng.uniform(0.2, 2.0, (nn, ng))
    dnc = torch.tensor(rng.uniform(-0.05, 0.05, (nn, ng, 6))) * R.canon[:, None, :]
    dn = R.expand(dnc).numpy()
    k = 1.05
    o.set_array("f0", f0.reshape(-1, order="F"))
    o.set_array("fs0", np.ones(nn))
    o.set_array("dn", dn.reshape(-1, order="F"))
    o.setd("Ke", k)
    from adpres_gb300.core import Core
    c = Core.from_deck(deck.parse(text))
    c.set_state(f0=f0, fs0=np.ones(nn), keff=k, dn=dn)
    return o, c, nn


def _check_case(bc, ng, kern, seed):
    o, c, nn = _case(bc, ng, kern, seed)
    # matrix_setup(1)
    o.matrix_setup(1)
    ref = np.transpose(o.matrix7(), (1, 0, 2))            # (nn, ng, 7)
    A7 = c.matrix()
    assert np.max(np.abs(A7 - ref)) <= 1e-13 * np.max(np.abs(ref)), ("matrix", bc)
    # PowDis of the state
    np.testing.assert_allclose(c.power(), o.powdis(), rtol=1e-13, atol=0)
    # one nodal update
    rep = c.nodal_step()
    o.nodal_upd(1)
    S = c.nodal_sources()
    Sref = np.stack([o.fortran(n, (nn, ng)) for n in ("S1", "S2", "S3")], axis=2)
    assert np.max(np.abs(S - Sref)) <= 1e-12 * max(np.max(np.abs(Sref)), 1e-300), ("S", bc)
    dn_ref = o.fortran("dn", (nn, ng, 6))
    _, _, _, dn = c.state()
    assert np.max(np.abs(dn - dn_ref)) <= 1e-11 * np.max(np.abs(dn_ref)), ("dn", bc)
    nd = o.getd("ndmax")
    assert abs(rep.ndmax - nd) <= 1e-11 * nd, ("ndmax", bc)
    return rep.loc, (o.geti("im"), o.geti("jm"), o.geti("km"))


def test_every_boundary_combination_two_groups_sanm():
    """All 729 combinations of zero flux, zero incoming current and
    reflective on the six faces; the ndmax location must agree wherever the
    maximum is not tied (it is a first-maximum rule over the sweep order)."""
    same = 0
    for i, bc in enumerate(ALL_BC):
        loc, loc_ref = _check_case(bc, 2, "SANM", 100 + i)
        same += loc == loc_ref
    assert same >= 0.95 * len(ALL_BC), same


@pytest.mark.parametrize("ng,kern", [(1, "PNM"), (3, "PNM"), (4, "SANM"), (2, "PNM")])
def test_seeded_boundary_combinations(ng, kern):
    rng = np.random.default_rng(ng * 10 + len(kern))
    for j in rng.choice(len(ALL_BC), 40, replace=False):
        _check_case(ALL_BC[int(j)], ng, kern, 2000 + int(j))
