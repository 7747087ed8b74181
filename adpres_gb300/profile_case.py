"""Run k-eigenvalue solves of a synthetic core, for profiling a kernel of the
solver in isolation (for example under ncu):

    python -m adpres_gb300.profile_case --config core_4g --planes 40 --precision mixed --solves 1

Prints k, the outer count and the device time of each solve.
"""
from __future__ import annotations

import argparse

from . import deck, synth
from .core import Core


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", default="core_4g", choices=sorted(synth.CONFIGS))
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--planes", type=int, default=80, help="axial planes of core_4g (20, 40 or 80)")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--solves", type=int, default=1)
    a = ap.parse_args()
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


if __name__ == "__main__":
    main()
