"""Regenerate tests/golden/decks/CBCsearch.npz, the critical boron search
fixture, from the ADPRES sample deck smpl/static/CBCsearch.

Run from the repository root where the reference project is mounted
(--ref):

    python tests/golden/make_feedback.py --ref <reference project root>

The fixture holds
  * the deck's input state as the oracle reads it (as make_golden.py);
  * the feedback cards as adpres_gb300.deck reads them (fb_* keys): boron,
    fuel and moderator temperature, coolant density and control rods;
  * node cross sections from the oracle's XS_updt at three boron
    concentrations (xs_<bcon index>_<name>), after the script has checked
    that adpres_gb300.feedback.xs_update gives the same bits;
  * the oracle's critical boron search: every iterate (bcon, k, outers),
    the final nodal power and flux, and the same search with the oracle
    rebuilt with multiply-add contraction (its rounding sensitivity).
No published output of this deck exists, so the search is pinned on the
oracle, whose CMFD and nodal path the static decks' fixtures pin.
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
from adpres_gb300.feedback import xs_update  # noqa: E402
from make_golden import deck_inputs  # noqa: E402

XS_BCON = (1200.2, 1500.0, 0.0)
XS_KEYS = ("sigtr", "siga", "nuf", "sigf", "sigs")


def pack_changes(ch):
    """(nmat, ng, 4 + ng): sigtr, siga, nuf, sigf, then sigs(g -> 1..ng)."""
    return np.concatenate([np.stack([ch[k] for k in ("sigtr", "siga", "nuf", "sigf")], axis=2), ch["sigs"]], axis=2)


def feedback_arrays(dk) -> dict:
    out = {"coreh": dk.coreh, "fb_names": np.array(sorted(dk.feedback))}
    for nm, f in dk.feedback.items():
        out["fb_%s_ch" % nm] = pack_changes(f["changes"])
        if nm == "crod":
            out["fb_crod_scal"] = np.array([f["nb"], f["nstep"], f["pos0"], f["ssize"]], dtype=np.float64)
            out["fb_crod_bpos"] = np.asarray(f["bpos"], dtype=np.float64)
            out["fb_crod_fbmap"] = np.asarray(f["fbmap"], dtype=np.int32)
        else:
            out["fb_%s_scal" % nm] = np.array([f["value"], f["ref"]])
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", required=True, help="root of the reference project tree")
    args = ap.parse_args()
    path = os.path.join(args.ref, "smpl", "static", "CBCsearch")
    dk = deck.load(path)
    o = oracle.Oracle(path)
    fx = deck_inputs(o)
    fx.update(feedback_arrays(dk))
    nn, ng = o.geti("nnod"), o.geti("ng")
    fx["xs_bcon"] = np.array(XS_BCON)
    for i, b in enumerate(XS_BCON):
        o.xs_updt_at(b)
        t = xs_update(dk, b)
        for k in XS_KEYS:
            shape = (nn, ng, ng) if k == "sigs" else (nn, ng)
            a = o.fortran(k, shape)
            if not np.array_equal(a, t[k]):
                raise SystemExit("xs_update differs from the oracle: %s at bcon %g" % (k, b))
            fx["xs_%d_%s" % (i, k)] = a
    o.reset()
    it = o.cbsearch()
    fx["out_bcon"] = np.array([r[0] for r in it])
    fx["out_k"] = np.array([r[1] for r in it])
    fx["out_outers"] = np.array([r[2] for r in it], dtype=np.int32)
    fx["out_power"] = o.powdis()
    fx["out_f0"] = o.array("f0")
    q = oracle.Oracle(path, variant="fma")
    itq = q.cbsearch()
    fx["sens_bcon"] = np.array([r[0] for r in itq])
    fx["sens_k"] = np.array([r[1] for r in itq])
    fx["sens_outers"] = np.array([r[2] for r in itq], dtype=np.int32)
    pw, pq = fx["out_power"], q.powdis()
    m = pw > 0
    fx["sens_power_rel"] = float(np.max(np.abs(pq[m] - pw[m]) / pw[m]))
    np.savez_compressed(os.path.join(HERE, "decks", "CBCsearch.npz"), **fx)
    print("CBCsearch", nn, "iterates", [(round(b, 4), round(k, 7), n) for b, k, n in it])
    print("  multiply-add variant", [(round(b, 4), round(k, 7), n) for b, k, n in itq],
          "power %.1e" % fx["sens_power_rel"])


if __name__ == "__main__":
    main()
