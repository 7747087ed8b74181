"""Generate tests/golden/adjoint_fd_full_core_3d.json: central differences
of the oracle's full solve (nodal update included) on the 34x34x22-node
two-group full core, the reference for dk/dSigma through the nodal update.

The oracle is converged to the nonlinear fixed point (the deck's iteration,
then criteria 1e-12, warm-started), and each difference re-converges flux,
eigenvalue and coupling coefficients from there with one cross section of
one node scaled by 1 +- rel (mod_xsec.f90:199-226 recomputes D and sigr).
Candidates are drawn by seed among fuel nodes for sigtr, siga, nuf and
sigs(1->2); one is kept when its k change at the step is above 1e-11
(1000x the oracle's convergence noise in k) and the differences at
relative steps 1e-4 and 2e-4 agree to 1e-4, the first 16 of each kind.

Run from the repository root (8 worker processes, a few minutes):
    python tests/golden/make_adjoint_fd.py
"""
from __future__ import annotations

import json
import multiprocessing as mp
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "adjoint_fd_full_core_3d.json")
COUNT = 64
SEED = 2025
REL = 1e-4


def _setup():
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))


def _candidates(nn, ng, nuf, draws):
    rng = np.random.default_rng(SEED)
    fuel = np.nonzero(nuf[:, ng - 1] > 0)[0]
    out = []
    for kind, count in draws:
        for _ in range(count):
            n = int(rng.choice(fuel))
            g = 0 if kind == "sigs" else int(rng.integers(ng))
            out.append((kind, n, g, 1 if kind == "sigs" else None))
    return out


def _work(args):
    chunk, = args
    _setup()
    import oracle
    from adpres_gb300 import synth
    from adjoint_full_ref import STATE, converge_fixed_point, full_fd
    o = oracle.Oracle(text=synth.full_core_3d(0))
    converge_fixed_point(o, tol=1e-12)
    base = {a: o.array(a).copy() for a in STATE}
    k0 = o.getd("Ke")
    nn, ng = o.geti("nnod"), o.geti("ng")
    res = []
    for idx, (kind, n, g, h) in chunk:
        if kind == "sigs":
            p = base["sigs"].reshape((nn, ng, ng), order="F")[n, g, h]
        else:
            p = base[kind].reshape((nn, ng), order="F")[n, g]
        f1 = full_fd(o, kind, n, g, REL, base, k0, h=h)
        f2 = full_fd(o, kind, n, g, 2 * REL, base, k0, h=h)
        res.append(dict(index=idx, kind=kind, n=n, g=g, h=h, p=float(p), fd=float(f1), fd2=float(f2),
                        dk=float(abs(f1 * p * 2 * REL))))
    return k0, res


def main():
    _setup()
    import oracle
    from adpres_gb300 import synth
    o = oracle.Oracle(text=synth.full_core_3d(0))
    o.xs_updt()
    nn, ng = o.geti("nnod"), o.geti("ng")
    nuf = o.fortran("nuf", (nn, ng))
    # sigtr of a random node moves k least (it acts through leakage only), so
    # it gets more draws; 16 parameters of each kind are kept
    draws = (("sigtr", 160), ("siga", 48), ("nuf", 48), ("sigs", 48))
    cands = list(enumerate(_candidates(nn, ng, nuf, draws)))
    nproc = min(8, os.cpu_count() or 1)
    chunks = [cands[i::nproc] for i in range(nproc)]
    with mp.get_context("spawn").Pool(nproc) as pool:
        parts = pool.map(_work, [(c,) for c in chunks])
    k0 = parts[0][0]
    rows = sorted((r for _, rs in parts for r in rs), key=lambda r: r["index"])
    good = [r for r in rows if r["dk"] > 1e-11 and abs(r["fd"] - r["fd2"]) <= 1e-4 * abs(r["fd"])]
    kept = []
    for kind, _ in draws:
        kept += [r for r in good if r["kind"] == kind][:COUNT // 4]
    if len(kept) < COUNT:
        raise SystemExit("only %d usable parameters" % len(kept))
    doc = {"workload": "synth.full_core_3d(0): 34x34 radial nodes x 22 planes, 2 groups, SANM",
           "fixed_point": "oracle, deck iteration then serc = ferc = 1e-12 warm-started",
           "rel_step": REL, "keff": k0, "seed": SEED, "candidates": len(rows), "params": kept}
    with open(OUT, "w") as f:
        json.dump(doc, f, indent=1)
    print("wrote %s: %d of %d candidates" % (OUT, len(kept), len(rows)))


if __name__ == "__main__":
    main()
