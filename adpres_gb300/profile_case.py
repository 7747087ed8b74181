"""Run k-eigenvalue solves of a synthetic core, for profiling a kernel of the
solver in isolation (for example under ncu):

    python -m adpres_gb300.profile_case --config core_4g --planes 40 --precision mixed --solves 1
    python -m adpres_gb300.profile_case --config batch --members 16 --precision mixed
    python -m adpres_gb300.profile_case --config batch --members 16 --shipped
    python -m adpres_gb300.profile_case --config full_core_3d --adjoint

Prints k, the outer count and the device time of each solve.  The batch
case solves the first `members` cores of the batched workload, in the
library's default schedule or, with --shipped, in the launch shape shipped
for this GPU model in batch_tuned.json (applied as a cached configuration:
three solves, each followed by a re-plan with the cores' times, so the
solve printed is the fourth launch of k_batch);
--adjoint adds the discrete adjoint and dk/dSigma after the forward solve.
"""
from __future__ import annotations

import argparse

from . import deck, synth
from .core import Core


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", default="core_4g", choices=sorted(synth.CONFIGS) + ["batch"])
    ap.add_argument("--members", type=int, default=16, help="cores of the batch case")
    ap.add_argument("--adjoint", action="store_true", help="also run adp_adjoint_sens")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--planes", type=int, default=80, help="axial planes of core_4g (20, 40 or 80)")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--solves", type=int, default=1)
    ap.add_argument("--shipped", action="store_true", help="batch case: the shipped tuned launch shape")
    a = ap.parse_args()
    if a.config == "batch":
        import json
        import os
        from .batch import Batch
        root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
        with open(os.path.join(root, "tests", "golden", "batch_members.json")) as f:
            acc = json.load(f)
        decks = [deck.parse(synth.batch_member(acc["seed"], i)) for i in acc["accepted"][:a.members]]
        b = Batch(decks, precision=a.precision)
        if a.shipped:
            from .batch import TUNED_PATH
            with open(TUNED_PATH) as f:
                shipped = json.load(f)
            cfg = next(iter(shipped.values()))["config"]
            b.apply_config(cfg)
            print("shipped shape:", b.config(), flush=True)
        for _ in range(a.solves):
            res, ms = b.solve()
            print(f"batch of {len(decks)} ({sum(len(d.ix) for d in decks)} nodes) {a.precision}: "
                  f"device_ms={ms:.2f} outers={[r['outers'] for r in res]}", flush=True)
        b.close()
        return
    if a.config == "core_4g":
        text = synth.core_4g(a.seed, planes=a.planes)
    else:
        text = synth.CONFIGS[a.config](a.seed)
    dk = deck.parse(text)
    with Core.from_deck(dk, precision=a.precision) as c:
        for _ in range(a.solves):
            c.reset()
            rep = c.outer(trace=False)
            print(f"{a.config} nodes={dk.nnod} groups={dk.ng} {a.precision}: k={rep.keff:.8f} "
                  f"outers={rep.outers} device_ms={rep.device_ms:.2f}", flush=True)
            if a.adjoint:
                _, _, arep = c.adjoint_sens()
                print(f"  adjoint: k={arep.keff:.8f} outers={arep.outers} device_ms={arep.device_ms:.2f}", flush=True)


if __name__ == "__main__":
    main()
