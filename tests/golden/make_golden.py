"""Regenerate the golden fixtures under tests/golden/ from the ADPRES sources.

Run from the repository root in a container where the reference project is
mounted (--ref):

    python tests/golden/make_golden.py --ref <reference project root>

It writes
  * iaea3d_trace.json -- the reference's own printed IAEA3D convergence trace,
    parsed from docs/quick-guides.md:161-191 (outers 1-5, 15-23, 127-129, the
    nodal-update record and the final k).  This is the hard pin of the oracle.
  * decks/<name>.npz  -- for each in-scope static sample deck: the parsed
    input state (geometry, node ordering, material cross sections, ADFs,
    iteration control) as the oracle's deck reader sees it, plus the oracle's
    results (per-outer trace, k, outer count, nodal power, flux).  The GPU
    tests read these, so they never need the reference tree at run time.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402

STATIC_DECKS = ["IAEA3Ds", "adjoint", "PNM", "FDM", "FDM-1D", "DVP", "IAEA2D", "BIBLIS", "KOEBERG"]


def parse_trace(md_path: str) -> dict:
    rows, nodal = [], None
    pat = re.compile(r"^\s+(\d+)\s+(\d+\.\d+)\s+([\d.]+E[+-]\d+)\s+([\d.]+E[+-]\d+)\s*$")
    npat = re.compile(r"MAX\. CHANGE IN NODAL COUPLING COEF\.=\s*([\d.]+E[+-]\d+)\s+AT NODE I =\s*(\d+), J =\s*(\d+), K =\s*(\d+)")
    kpat = re.compile(r"MULTIPLICATION EFFECTIVE \(K-EFF\) =\s*(\d+\.\d+)")
    keff = None
    extrap_before = []
    pending_extrap = False
    with open(md_path) as f:
        lines = f.readlines()
    for ln in lines[155:205]:
        if "FISSION SOURCE EXTRAPOLATED" in ln:
            pending_extrap = True
            continue
        m = pat.match(ln)
        if m:
            p = int(m.group(1))
            rows.append({"p": p, "k": m.group(2), "ser": m.group(3), "fer": m.group(4)})
            if pending_extrap:
                extrap_before.append(p)
                pending_extrap = False
            continue
        m = npat.search(ln)
        if m:
            nodal = {"ndmax": m.group(1), "loc": [int(m.group(2)), int(m.group(3)), int(m.group(4))]}
            continue
        m = kpat.search(ln)
        if m:
            keff = m.group(1)
    return {"source": "docs/quick-guides.md:161-191", "deck": "smpl/static/IAEA3Ds",
            "rows": rows, "extrapolated_at": extrap_before, "nodal": nodal,
            "nodal_at": 22, "keff": keff, "outers": rows[-1]["p"]}


def deck_inputs(o) -> dict:
    """The parsed input state of a deck as the oracle's reader holds it."""
    nnod, ng, nmat = o.geti("nnod"), o.geti("ng"), o.geti("nmat")
    return {
        "ng": ng, "nmat": nmat, "nnod": nnod,
        "nxx": o.geti("nxx"), "nyy": o.geti("nyy"), "nzz": o.geti("nzz"),
        "ix": o.array("ix"), "iy": o.array("iy"), "iz": o.array("iz"), "mat": o.array("mat"),
        "xdel": o.array("xdel"), "ydel": o.array("ydel"), "zdel": o.array("zdel"),
        "bc": np.array([o.geti(k) for k in ("xeast", "xwest", "ynorth", "ysouth", "zbott", "ztop")], dtype=np.int32),
        "xsigtr": o.array("xsigtr"), "xsiga": o.array("xsiga"), "xnuf": o.array("xnuf"),
        "xsigf": o.array("xsigf"), "chi": o.array("chi"), "xsigs": o.array("xsigs"),
        "dc": o.array("dc"),
        "iter_int": np.array([o.geti(k) for k in ("nin", "nout", "nac", "nupd")], dtype=np.int32),
        "iter_real": np.array([o.getd("serc"), o.getd("ferc")]),
        "kern": o.geti("kern"), "adjoint": o.geti("adjoint"),
    }


def deck_fixture(path: str) -> dict:
    o = oracle.Oracle(path)
    inp = deck_inputs(o)
    o.run()
    tr = o.trace()
    out = {
        "out_k": o.getd("Ke"), "out_outers": o.geti("outers"), "out_ndmax": o.getd("ndmax"),
        "out_power": o.powdis(), "out_f0": o.array("f0"),
        "out_trace_k": np.array([r.k for r in tr]), "out_trace_ser": np.array([r.ser for r in tr]),
        "out_trace_fer": np.array([r.fer for r in tr]),
        "out_trace_flags": np.array([int(r.extrapolated) | (int(r.nodal) << 1) for r in tr], dtype=np.int32),
        "out_trace_ndmax": np.array([r.ndmax for r in tr]),
        "out_trace_loc": np.array([r.loc for r in tr], dtype=np.int32).reshape(-1, 3),
    }
    inp.update(out)
    # Rounding sensitivity of the reference algorithm on this deck: the same
    # restatement rebuilt with multiply-add contraction, and with BiCGSTAB's
    # (rs, r) formed as (rs,s) - omega (rs,t), each compared with the oracle.
    outers, trace_rel, k_pcm, pw_rel = [], 0.0, 0.0, 0.0
    pw = out["out_power"]
    m = pw > 0
    for variant in ("fma", "fma_rhost"):
        q = oracle.Oracle(path, variant=variant)
        q.run()
        kq = np.array([r.k for r in q.trace()])
        n = min(len(kq), len(out["out_trace_k"]))
        outers.append(q.geti("outers"))
        trace_rel = max(trace_rel, float(np.max(np.abs(kq[:n] - out["out_trace_k"][:n]) / out["out_trace_k"][:n])))
        k_pcm = max(k_pcm, abs(q.getd("Ke") - out["out_k"]) / out["out_k"] * 1e5)
        pw_rel = max(pw_rel, float(np.max(np.abs(q.powdis()[m] - pw[m]) / pw[m])))
    inp["sens_outers"] = np.array(outers, dtype=np.int32)
    inp["sens_trace_rel"] = trace_rel
    inp["sens_k_pcm"] = k_pcm
    inp["sens_power_rel"] = pw_rel
    return inp


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", required=True, help="root of the reference project tree")
    args = ap.parse_args()
    trace = parse_trace(os.path.join(args.ref, "docs", "quick-guides.md"))
    with open(os.path.join(HERE, "iaea3d_trace.json"), "w") as f:
        json.dump(trace, f, indent=1)
    os.makedirs(os.path.join(HERE, "decks"), exist_ok=True)
    for name in STATIC_DECKS:
        fx = deck_fixture(os.path.join(args.ref, "smpl", "static", name))
        np.savez_compressed(os.path.join(HERE, "decks", name + ".npz"), **fx)
        print(name, fx["nnod"], fx["out_k"], fx["out_outers"], "sensitivity: outers", fx["sens_outers"],
              "trace %.1e power %.1e" % (fx["sens_trace_rel"], fx["sens_power_rel"]))


if __name__ == "__main__":
    main()
