"""Cross-section feedback and the critical boron search on the host: the
deck reader's feedback cards and adpres_gb300.feedback.xs_update against the
oracle's XS_updt (mod_xsec.f90:11-46), bit for bit, and the oracle's own
boron search (mod_th.f90:752-837) on the sample deck CBCsearch."""
import numpy as np
import pytest

import oracle
from adpres_gb300 import deck
from adpres_gb300.feedback import xs_update
from conftest import reference_deck
from feedback_fixture import deck_from_fixture, fixture

KEYS = ("sigtr", "siga", "nuf", "sigf", "sigs")


def test_fixture_xs_update_matches_oracle_bits():
    """Node tables from the fixture's cards equal the oracle's XS_updt at three
    boron concentrations (the control rods' clamp of negative entries included)."""
    fx = fixture()
    dk = deck_from_fixture(fx)
    for i, b in enumerate(fx["xs_bcon"]):
        t = xs_update(dk, float(b))
        for k in KEYS:
            np.testing.assert_array_equal(t[k], fx["xs_%d_%s" % (i, k)], err_msg="%s at %g ppm" % (k, b))


def test_rods_reach_the_core():
    """The deck's rods change the tables: without %CROD the nodes under a bank differ."""
    fx = fixture()
    dk = deck_from_fixture(fx)
    t = xs_update(dk, 1200.2)
    del dk.feedback["crod"]
    u = xs_update(dk, 1200.2)
    rodded = np.any(t["siga"] != u["siga"], axis=1)
    assert 0 < rodded.sum() < len(rodded)


def test_deck_reader_feedback_matches_oracle():
    path = reference_deck("CBCsearch")
    dk = deck.load(path)
    assert dk.mode == "BCSEARCH" and dk.bcbcs
    assert sorted(dk.feedback) == ["bcon", "cden", "crod", "ftem", "mtem"]
    o = oracle.Oracle(path)
    nn, ng = o.geti("nnod"), o.geti("ng")
    for b in (dk.feedback["bcon"]["ref"], 777.0):
        o.xs_updt_at(b)
        t = xs_update(dk, b)
        for k in KEYS:
            shape = (nn, ng, ng) if k == "sigs" else (nn, ng)
            np.testing.assert_array_equal(t[k], o.fortran(k, shape))


def test_oracle_cbsearch_matches_fixture():
    """The oracle's search on the sample deck: 4 iterates ending at k = 1 within 1e-5."""
    path = reference_deck("CBCsearch")
    fx = fixture()
    it = oracle.Oracle(path).cbsearch()
    assert len(it) == len(fx["out_bcon"]) == 4
    np.testing.assert_array_equal([r[0] for r in it], fx["out_bcon"])
    np.testing.assert_array_equal([r[1] for r in it], fx["out_k"])
    assert abs(it[-1][1] - 1.0) < 1e-5
    assert it[-1][0] == pytest.approx(1257.32, abs=0.01)


def _strip_card(text, name):
    """The deck without card %name (its lines up to the next card)."""
    out, skip = [], False
    for ln in text.splitlines():
        s = ln.strip()
        if s.startswith("%"):
            skip = s[1:].strip().upper() == name
        if not skip:
            out.append(ln)
    return "\n".join(out) + "\n"


def _card_body(text, name, first):
    """The records of card %name with its first record replaced by `first`."""
    out, on, seen = [], False, False
    for ln in text.splitlines():
        s = ln.strip()
        if s.startswith("%"):
            on = s[1:].strip().upper() == name
            continue
        if on and s and not s.startswith("!"):
            out.append(first if not seen else ln)
            seen = True
    return "\n".join(out) + "\n"


def _edit(text, old, new):
    assert old in text
    return text.replace(old, new, 1)


@pytest.mark.parametrize("case", ["no_cbcs", "bank_beyond_steps", "negative_bank", "bank_number", "cbcs_in_forward",
                                  "bcon_in_search"])
def test_deck_feedback_card_errors(case):
    """inp_crod's checks (mod_io.f90:2148-2328) and BCSEARCH's need of %CBCS:
    the deck reader and the oracle reject the same decks."""
    text = open(reference_deck("CBCsearch")).read()
    bpos = "100.00  200.00  100.00  200.00"
    bad = {"no_cbcs": (_strip_card(text, "CBCS"), "CBCS"),
           "bank_beyond_steps": (_edit(text, bpos, "300.00  200.00  100.00  200.00"), "number of steps"),
           "negative_bank": (_edit(text, bpos, "-1.00  200.00  100.00  200.00"), "negative"),
           "bank_number": (_edit(text, "\n 1  0  2  0  0  0  3", "\n 9  0  2  0  0  0  3"), "number of banks"),
           "cbcs_in_forward": (_edit(text, "BCSEARCH", "FORWARD"), "not necessary"),
           "bcon_in_search": (text + "%BCON\n" + _card_body(text, "CBCS", "1200.2 1200.2"), "must not present")}
    t, msg = bad[case]
    with pytest.raises(deck.DeckError, match=msg):
        deck.parse(t, "/nonexistent")
    with pytest.raises(oracle.OracleError, match=msg):
        oracle.Oracle(text=t)


def test_rod_tips_of_the_abi_match_the_host_restatement():
    """adp_fb_rod_tips (host arithmetic inside the C library, no device
    call) gives the plane and rodded fraction of feedback._rod_tip to the bit
    for bank positions across and beyond the core, on the sample deck's
    planes and on uneven ones."""
    import ctypes

    from adpres_gb300 import _lib
    from adpres_gb300._lib import dptr, iptr
    from adpres_gb300.feedback import _rod_tip
    L = _lib.load()
    rng = np.random.default_rng(7)
    fx = fixture()
    dk = deck_from_fixture(fx)
    cr = dk.feedback["crod"]
    cases = [([float(z) for z in dk.zdel], float(dk.coreh), float(cr["pos0"]), float(cr["ssize"]))]
    z = list(rng.uniform(2.0, 30.0, 17))
    h = 0.0
    for v in z:
        h = h + v
    cases.append((z, h, 7.3, 1.587))
    for zdel, coreh, pos0, ssize in cases:
        nstep = (coreh - pos0) / ssize
        bpos = np.concatenate([rng.uniform(-5.0, nstep + 5.0, 400), [0.0, nstep, np.floor(nstep)]])
        tip = np.zeros(len(bpos), dtype=np.int32)
        vf = np.zeros(len(bpos))
        zd = np.ascontiguousarray(zdel, dtype=np.float64)
        st = L.adp_fb_rod_tips(len(zdel), dptr(zd), coreh, pos0, ssize, len(bpos), dptr(bpos), iptr(tip), dptr(vf))
        assert st == 0
        for b, p in enumerate(bpos):
            k, w = _rod_tip(coreh - pos0 - p * ssize, zdel)
            assert tip[b] == k
            if k >= 0:
                assert vf[b] == w
