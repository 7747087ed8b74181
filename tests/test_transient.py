"""Rod ejection transient on the host side: the %EJCT / %THET / %EXTR cards
(mod_io.f90:1650-1689, 2332-2482) in the deck reader and the oracle, the
oracle's rod_eject (mod_trans.f90:17-160) on the sample deck LMW against the
committed fixture, and the bank motion of trans_calc."""
import numpy as np
import pytest

import oracle
from adpres_gb300 import deck
from adpres_gb300.transient import move_banks
from feedback_fixture import fixture


def _lmw_path():
    import os
    from conftest import REFERENCE
    p = os.path.join(REFERENCE, "smpl", "transient", "LMW")
    if not os.path.exists(p):
        pytest.skip("reference sample decks are not mounted here")
    return p


def test_deck_reader_reads_ejct_and_thet():
    dk = deck.load(_lmw_path())
    tr = dk.trans
    assert dk.mode == "RODEJECT"
    np.testing.assert_array_equal(tr["fbpos"], [60.0, 180.0])
    np.testing.assert_array_equal(tr["mdir"], [1, 2])          # bank 1 down, bank 2 up from %CROD
    assert (tr["ttot"], tr["tstep1"], tr["tdiv"], tr["tstep2"]) == (60.0, 0.25, 60.0, 1.0)
    assert tr["theta"] == 0.5 and not tr["extr"]
    assert len(tr["beta"]) == 6 and len(tr["velo"]) == dk.ng


def test_oracle_rod_eject_matches_fixture():
    fx = fixture("LMW")
    r = oracle.Oracle(_lmw_path()).rodeject()
    assert len(r) == len(fx["out_t"]) == 241
    np.testing.assert_array_equal([x[2] for x in r], fx["out_pow"])
    np.testing.assert_array_equal([x[1] for x in r], fx["out_rho"])
    assert abs(r[0][1]) < 1e-6                  # k brought to one: no reactivity at t = 0
    assert max(x[2] for x in r) == pytest.approx(1.7313, abs=1e-4)


def test_move_banks_follows_trans_calc():
    tr = dict(mdir=np.array([1, 2, 0]), tmove=np.array([1.0, 0.0, 0.0]), fbpos=np.array([60.0, 180.0, 5.0]),
              bspeed=np.array([3.0, 3.0, 3.0]))
    b = np.array([100.0, 170.0, 5.0])
    move_banks(b, tr, 0.5, 0.5)                 # bank 1 has not started
    np.testing.assert_array_equal(b, [100.0, 171.5, 5.0])
    for k in range(2, 12):
        move_banks(b, tr, 0.5, 0.5 * k)
    assert b[1] == 180.0 and b[0] == 100.0 - 1.5 * 9 and b[2] == 5.0


def _edit(text, old, new):
    assert old in text
    return text.replace(old, new, 1)


@pytest.mark.parametrize("case", ["no_ejct", "ejct_in_forward", "final_beyond_steps", "theta_small", "theta_big",
                                  "time_order"])
def test_transient_card_errors(case):
    text = open(_lmw_path()).read()
    lines = text.splitlines()
    if case == "no_ejct":
        out, skip = [], False
        for ln in lines:
            s = ln.strip()
            if s.startswith("%"):
                skip = s[1:].strip().upper() == "EJCT"
            if not skip:
                out.append(ln)
        t, msg = "\n".join(out) + "\n", "EJCT"
    elif case == "ejct_in_forward":
        t, msg = _edit(text, "RODEJECT", "FORWARD"), "not necessary"
    elif case == "final_beyond_steps":
        t, msg = _edit(text, "     60.                       7.5", "     999.                       7.5"), "final control rod"
    elif case == "theta_small":
        t, msg = _edit(text, "%THET\n0.5", "%THET\n0.0001"), "too small"
    elif case == "theta_big":
        t, msg = _edit(text, "%THET\n0.5", "%THET\n1.5"), "greater"
    else:
        t, msg = _edit(text, "60.  0.25  60.0  1.0", "60.  0.25  70.0  1.0"), "less than the total"
    with pytest.raises(deck.DeckError, match=msg):
        deck.parse(t, "/nonexistent")
    with pytest.raises(oracle.OracleError, match=msg):
        oracle.Oracle(text=t)
