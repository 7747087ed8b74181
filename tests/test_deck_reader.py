"""The product's deck reader against the oracle's reader (two independent
restatements of mod_io.f90) on the reference sample decks and on synthetic
decks, plus its error behaviour."""
import numpy as np
import pytest

import oracle
from adpres_gb300 import deck, synth
from adpres_gb300._lib import ADP_ERR_INPUT, ADP_ERR_UNSUPPORTED
from conftest import reference_deck


def _compare(dk, o):
    ng, nn, nm = dk.ng, dk.nnod, dk.nmat
    assert (ng, nn, nm) == (o.geti("ng"), o.geti("nnod"), o.geti("nmat"))
    assert (dk.nxx, dk.nyy, dk.nzz) == (o.geti("nxx"), o.geti("nyy"), o.geti("nzz"))
    for name in ("ix", "iy", "iz", "mat"):
        np.testing.assert_array_equal(getattr(dk, name), o.array(name))
    for name in ("xdel", "ydel", "zdel"):
        np.testing.assert_array_equal(getattr(dk, name), o.array(name))
    assert tuple(dk.bc) == tuple(o.geti(k) for k in ("xeast", "xwest", "ynorth", "ysouth", "zbott", "ztop"))
    for name in ("xsigtr", "xsiga", "xnuf", "xsigf", "chi"):
        np.testing.assert_array_equal(getattr(dk, name), o.fortran(name, (nm, ng)))
    np.testing.assert_array_equal(dk.xsigs, o.fortran("xsigs", (nm, ng, ng)))
    np.testing.assert_array_equal(dk.dc, o.fortran("dc", (nn, ng, 6)))
    assert (dk.nin, dk.nout, dk.nac, dk.nupd) == tuple(o.geti(k) for k in ("nin", "nout", "nac", "nupd"))
    assert dk.serc == o.getd("serc") and dk.ferc == o.getd("ferc")
    assert dk.kern_code == o.geti("kern")
    assert int(dk.adjoint) == o.geti("adjoint")


@pytest.mark.parametrize("name", ["IAEA3Ds", "adjoint", "PNM", "FDM", "FDM-1D", "DVP", "IAEA2D", "BIBLIS", "KOEBERG",
                                  "MOX/part1_ari_helios", "MOX/part1_ari_serpent", "MOX/part1_aro_helios",
                                  "MOX/part1_aro_serpent"])
def test_reference_decks_match_oracle(name):
    path = reference_deck(name)
    _compare(deck.load(path), oracle.Oracle(path))


@pytest.mark.parametrize("fn", [synth.quarter_core_2d, synth.full_core_3d, synth.core_4g])
def test_synthetic_configs_match_oracle(fn):
    text = fn(0)
    _compare(deck.parse(text), oracle.Oracle(text=text))


@pytest.mark.parametrize("seed", range(6))
def test_small_cores_match_oracle(seed):
    text = synth.small_core(seed=seed, ng=1 + seed % 4, adf=True, kern=("SANM", "PNM", "FDM")[seed % 3])
    _compare(deck.parse(text), oracle.Oracle(text=text))


def test_batch_member_shapes():
    for i in range(5):
        dk = deck.parse(synth.batch_member(0, i))
        assert 20 <= dk.nxx <= 68 and dk.nxx == dk.nyy and 10 <= dk.nzz <= 40


def test_default_iteration_control():
    dk = deck.load(reference_deck("IAEA3Ds"))
    assert dk.nupd == 22             # ceiling((17+17+19)/2.5), mod_io.f90:1363
    assert dk.serc == float(np.float32(1e-5))


def test_out_of_scope_and_bad_cards():
    with pytest.raises(deck.DeckError) as e:
        deck.load(reference_deck("fixed_source"))
    assert e.value.status == ADP_ERR_UNSUPPORTED
    # the NEACRP decks include their cards by the author's absolute paths;
    # the include falls back to the file beside the deck, and both readers
    # then stop at the thermal-hydraulics card, outside this path
    path = reference_deck("NEACRP/A1")
    with pytest.raises(deck.DeckError) as e:
        deck.load(path)
    assert e.value.status == ADP_ERR_UNSUPPORTED and "THER" in str(e.value)
    with pytest.raises(oracle.OracleError) as e:
        oracle.Oracle(path)
    assert "THER" in str(e.value)
    bad = synth.small_core(seed=0).replace("%KERN", "%KERNEL")
    with pytest.raises(deck.DeckError) as e:
        deck.parse(bad)
    assert e.value.status == ADP_ERR_INPUT
    short = synth.small_core(seed=0).replace("%GEOM\n4 4 3", "%GEOM\n4 4")
    with pytest.raises(deck.DeckError):
        deck.parse(short)


def test_repeat_syntax_and_comments():
    text = synth.small_core(seed=1)
    text = text.replace("15.0 15.0 15.0 15.0", "4*15.0  ! four assemblies")
    dk = deck.parse(text)
    np.testing.assert_array_equal(dk.xdel, np.full(8, 7.5))
