"""Regenerate tests/golden/decks/LMW.npz, the rod ejection fixture, from the
ADPRES sample deck smpl/transient/LMW (a rod-movement transient: bank 2
withdrawn from t = 0, bank 1 inserted from 7.5 s, theta 0.5, 240 steps).

    python tests/golden/make_transient.py --ref <reference project root>

The fixture holds the deck's input state as the oracle reads it (as
make_golden.py), its %CROD card as adpres_gb300.deck reads it (as
make_feedback.py), the %EJCT / %THET data (tr_* keys), and the oracle's
rod_eject records (t, reactivity, relative power, nout reached, outers),
plus the same run of the oracle rebuilt with multiply-add contraction (its
rounding sensitivity).  No published output of this deck exists, so the
transient is pinned on the oracle, whose static path the IAEA3D trace pins.
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

import oracle  # noqa: E402
from adpres_gb300 import deck  # noqa: E402
from make_feedback import feedback_arrays  # noqa: E402
from make_golden import deck_inputs  # noqa: E402


def trans_arrays(dk) -> dict:
    tr = dk.trans
    out = {"tr_" + k: np.asarray(tr[k], dtype=np.float64) for k in ("fbpos", "tmove", "bspeed", "beta", "lamb", "velo")}
    out["tr_mdir"] = np.asarray(tr["mdir"], dtype=np.int32)
    out["tr_scal"] = np.array([tr["ttot"], tr["tstep1"], tr["tdiv"], tr["tstep2"], tr["theta"], float(tr["extr"])])
    return out


def records(rec, prefix) -> dict:
    a = np.array([[r[0], r[1], r[2]] for r in rec])
    return {prefix + "t": a[:, 0], prefix + "rho": a[:, 1], prefix + "pow": a[:, 2],
            prefix + "maxi": np.array([r[3] for r in rec], dtype=np.int32),
            prefix + "outers": np.array([r[4] for r in rec], dtype=np.int32)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", required=True, help="root of the reference project tree")
    args = ap.parse_args()
    path = os.path.join(args.ref, "smpl", "transient", "LMW")
    dk = deck.load(path)
    o = oracle.Oracle(path)
    fx = deck_inputs(o)
    fx.update(feedback_arrays(dk))
    fx.update(trans_arrays(dk))
    fx["mode"] = np.array("RODEJECT")
    fx.update(records(o.rodeject(), "out_"))
    fx.update(records(oracle.Oracle(path, variant="fma").rodeject(), "sens_"))
    np.savez_compressed(os.path.join(HERE, "decks", "LMW.npz"), **fx)
    d = np.abs(fx["sens_pow"] - fx["out_pow"]) / fx["out_pow"]
    print("LMW", o.geti("nnod"), "steps", len(fx["out_t"]) - 1, "peak power %.4f" % fx["out_pow"].max(),
          "multiply-add variant: max power difference %.2e, max |drho| %.2e $" %
          (d.max(), np.abs(fx["sens_rho"][1:] - fx["out_rho"][1:]).max()))


if __name__ == "__main__":
    main()
