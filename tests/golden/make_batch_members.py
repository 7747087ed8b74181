"""Select the members of the batched workload on which the reference
algorithm converges, with the oracle's k and outer count for each.

The batched workload is 256 cores drawn by adpres_gb300.synth.batch_member
(seed 0, index 0, 1, 2, ...).  On some draws the reference's outer
iteration itself diverges (the two-node update ends with ndmax > 1e3,
mod_nodal.f90:131-142), and on some it converges only marginally: a
rounding-level change (the oracle built with multiply-add contraction)
decides between convergence and divergence, or it needs over 500 outers.
No solver that follows the reference's steps with other rounding can be
expected to converge on those, so a draw is accepted only when both oracle
builds converge within MAX_OUTERS outers.  Writes batch_members.json beside
this script: {"seed", "max_outers", "accepted": [index...], "rejected":
{index: reason}, "oracle": {index: [k, outers]}}.

    python tests/golden/make_batch_members.py [count]
"""
import json
import multiprocessing as mp
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

SEED = 0
MAX_OUTERS = 500


def run(i):
    import oracle
    from adpres_gb300 import synth
    text = synth.batch_member(SEED, i)
    res = None
    for variant in ("plain", "fma"):
        o = oracle.Oracle(text=text, variant=variant)
        try:
            o.run()
        except Exception as e:   # the reference STOPs on these inputs
            return i, False, f"{variant}: {str(e)[:100]}"
        if o.geti("outers") > MAX_OUTERS:
            return i, False, f"{variant}: {o.geti('outers')} outers"
        if variant == "plain":
            res = [o.getd("Ke"), o.geti("outers")]
    return i, True, res


def main(count=256):
    import oracle
    for v in ("plain", "fma"):
        oracle.build(variant=v)
    t0 = time.time()
    accepted, rejected, ora = [], {}, {}
    ctx = mp.get_context("spawn")
    nxt = 0
    with ctx.Pool(max(1, os.cpu_count() or 1)) as pool:
        while len(accepted) < count:
            need = count - len(accepted)
            batch = list(range(nxt, nxt + need + max(4, need // 10)))
            nxt = batch[-1] + 1
            for i, ok, v in pool.imap(run, batch):
                if ok:
                    accepted.append(i)
                    ora[str(i)] = v
                else:
                    rejected[str(i)] = v
    accepted = sorted(accepted)[:count]
    ora = {k: v for k, v in ora.items() if int(k) in accepted}
    out = {"seed": SEED, "max_outers": MAX_OUTERS, "accepted": accepted, "rejected": rejected, "oracle": ora}
    with open(os.path.join(HERE, "batch_members.json"), "w") as f:
        json.dump(out, f, indent=0)
    print(f"{len(accepted)} accepted, {len(rejected)} rejected in {time.time() - t0:.0f} s")


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else 256)
