#!/usr/bin/env python
"""Benchmark of the GB300 static k-eigenvalue path.

Workload (one step = one full k-eigenvalue solve from a cold start,
f0 = 1 and k = 1, to the reference's convergence test, including the SANM
nodal updates): the 68x68x80-node, 4-group core (17x17 assemblies of 4x4
nodes, 80 planes of 5 cm, seed 0 of adpres_gb300.synth.core_4g), solved in
mixed precision (FP32 matrix copy and Krylov vectors, FP64 flux, FP64
residual per group solve, FP64 reductions and eigenvalue).  The FP64 path is
timed on the same core in the same run for the mixed-vs-FP64 comparison.

    python bench.py [--steps K] [--warmup W] [--impl ours|reference]

value: solves/s with the cross sections resident on the device (CUDA
events on the solver's stream, L2 flushed between steps).  e2e: solves/s
through the C ABI from host buffers: cross-section upload, solve, power and
flux read-back inside the timed region.  The reference arm times the CPU
restatement of the reference's loops (the oracle; no Fortran compiler is
available) on all host cores, each core running its own solve.
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "k-eig solves/s (mixed FP32/FP64, |dk| <= 1 pcm vs FP64)"
UNIT = "solves/s"
CONFIG_NAME = "core_4g"
SEED = 0
# Outers timed per process by the reference arm's bounded sample; the
# sample is scaled by the outers and nodal updates of a full solve of the
# same core that the arm times in its warm-up.
CPU_SAMPLE_OUTERS = 4


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def workload_text():
    from adpres_gb300 import synth
    return synth.core_4g(SEED)


def workload_config(dk, precision):
    return {
        "workload": "core_4g: 17x17 assemblies of 4x4 nodes, 80 planes of 5 cm (68x68x80 = 369,920 nodes), "
                    "4 groups, down-scatter only, SANM nodal update, full solve from f0=1 to serc=ferc=1e-5",
        "nodes": int(dk.nnod), "groups": int(dk.ng), "unknowns": int(dk.nnod * dk.ng), "precision": precision,
        "nin": int(dk.nin), "nupd": int(dk.nupd), "seed": SEED, "l2": "flushed between steps (256 MiB write)",
        "parallelism": "replicas only",
    }


# ---------------------------------------------------------------- clocks --
class Clocks:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.p = None
        try:
            self.p = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.QUERY, "--format=csv,noheader,nounits",
                                       "-i", str(index), "-lms", "200"], stdout=subprocess.PIPE,
                                      stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.p.terminate()
        try:
            out, _ = self.p.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
            out, _ = self.p.communicate()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


# ---------------------------------------------------------- CPU baseline --
def cpu_sample(text, outers):
    """Time the oracle on a bounded sample: its first outer call (the
    first-call start, matrix_setup and the first touch of every array, one
    outer), then the cost of one more outer iteration as the difference of
    two warm calls of 1 and 1 + `outers` outers (each call repeats
    matrix_setup, which a full solve does once), and one nodal update:
    (t_first, t_outer, t_nodal)."""
    import oracle
    o = oracle.Oracle(text=text)
    o.xs_updt()
    t0 = time.perf_counter()
    o.outer(adjoint=False, popt=1, max_outers=1)
    t_first = time.perf_counter() - t0
    t0 = time.perf_counter()
    o.outer(adjoint=False, popt=0, max_outers=1)
    t_a = time.perf_counter() - t0
    t0 = time.perf_counter()
    o.outer(adjoint=False, popt=0, max_outers=1 + outers)
    t_b = time.perf_counter() - t0
    t_outer = max(t_b - t_a, 0.0) / outers
    t0 = time.perf_counter()
    o.nodal_upd(1)
    t_nodal = time.perf_counter() - t0
    return t_first, t_outer, t_nodal


def cpu_full_solve(text):
    """One full solve of the oracle from a cold start: (seconds, outers,
    nodal updates, k)."""
    import oracle
    o = oracle.Oracle(text=text)
    t0 = time.perf_counter()
    o.run()
    t = time.perf_counter() - t0
    nodal = sum(1 for r in o.trace() if r.nodal)
    return t, o.geti("outers"), nodal, o.getd("Ke")


def _worker(args):
    text, outers = args
    return cpu_sample(text, outers)


def _full_worker(text):
    return cpu_full_solve(text)


def cpu_baseline_single(text):
    t, outers, nodal, k = cpu_full_solve(text)
    return {"value": 1.0 / t, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"oracle (CPU restatement of the reference loops, -O2, 1 core): one full solve of this core "
                      f"from a cold start, {t:.1f} s ({outers} outers, {nodal} nodal updates, k = {k:.9f})",
            "outers": outers, "nodal_updates": nodal, "seconds": t}


# ------------------------------------------------ dk/dSigma leg ----
def adjoint_leg(flush, steps=3):
    """Forward solve + adjoint + dk/dSigma on the 34x34x22-node two-group
    full core (seed 0), mixed precision and FP64, with the deck's iteration
    control: the derivative at frozen dn (adp_adjoint_sens_frozen) and the
    derivative of the fixed point through the nodal update
    (adp_adjoint_sens).  gradients/s counts D, siga, nuf per group and the
    1->2 scattering per node."""
    import torch

    from adpres_gb300 import deck, synth
    from adpres_gb300.core import Core

    dk = deck.parse(synth.full_core_3d(0))
    out = {"workload": "full_core_3d seed 0: 34x34 radial nodes x 22 planes, 2 groups, SANM, serc = ferc = 1e-5",
           "params_per_solve": int(dk.nnod * (3 * dk.ng + dk.ng * (dk.ng - 1) // 2))}
    for prec in ("mixed", "fp64"):
        c = Core.from_deck(dk, precision=prec)
        for mode in ("frozen_dn", "fixed_point"):
            def run():
                c.reset()
                r = c.outer(trace=False)
                _, _, a = c.adjoint_sens(frozen_dn=(mode == "frozen_dn"))
                return r.device_ms, c.last_adjoint_ms, a

            for _ in range(2):
                run()
            fwd, adj = [], []
            for _ in range(steps):
                flush.zero_()
                torch.cuda.synchronize()
                f, a, rep = run()
                fwd.append(f)
                adj.append(a)
            t = (sum(fwd) + sum(adj)) / steps / 1e3
            out["%s_%s" % (prec, mode)] = {
                "grads_per_s": out["params_per_solve"] / t, "ms_per_solve": t * 1e3,
                "forward_ms": sum(fwd) / steps, "adjoint_ms": sum(adj) / steps,
                "adjoint_outers": rep.outers, "rounds": rep.nodal_updates,
                "fixed_point_residual": rep.ndmax if mode == "fixed_point" else None}
        c.close()
    out["cpu_baseline"] = _adjoint_cpu_baseline(synth.full_core_3d(0), out["params_per_solve"])
    return out


def _adjoint_cpu_baseline(text, nparams):
    """The reference's only route to dk/dSigma: central differences of its
    full solve, two warm-started solves per parameter (the oracle, one host
    core, the deck's criteria).  Timed on two parameters (four solves)."""
    import numpy as np

    import oracle
    o = oracle.Oracle(text=text)
    o.run()
    state = {a: o.array(a).copy() for a in ("f0", "fs0", "dn", "D", "sigr", "siga", "sigtr", "nuf", "sigs")}
    k0 = o.getd("Ke")
    nn, ng = o.geti("nnod"), o.geti("ng")
    fuel = np.nonzero(o.fortran("nuf", (nn, ng))[:, 1] > 0)[0]
    n = int(fuel[len(fuel) // 2])
    t0 = time.perf_counter()
    for kind in ("siga", "nuf"):
        for r in (1e-4, -1e-4):
            for a, v in state.items():
                o.set_array(a, v)
            o.setd("Ke", k0)
            a = o.fortran(kind, (nn, ng)).copy()
            a[n, 1] *= 1.0 + r
            o.set_array(kind, a.reshape(-1, order="F"))
            if kind != "nuf":
                o.dsigr_updt()
            o.outer(popt=1)
    per_grad = (time.perf_counter() - t0) / 2
    return {"value": 1.0 / per_grad, "unit": "gradients/s", "cores": 1, "kind": "port",
            "sample": f"central differences of the oracle's full solve (two warm-started solves per parameter, "
                      f"the deck's criteria), timed on two parameters: {per_grad:.2f} s per gradient, "
                      f"{nparams * per_grad / 3600:.0f} h for the {nparams} parameters one adjoint solve gives"}


# ------------------------------------------- critical boron search leg ----
def _cbsearch_oracle(text):
    import oracle
    o = oracle.Oracle(text=text)
    t0 = time.perf_counter()
    it = o.cbsearch()
    return time.perf_counter() - t0, it


def cbsearch_leg(flush, steps=3):
    """th::cbsearch on the 34x34x22-node full core with boron, temperature,
    density and control-rod feedback cards (seed 0): the feedback tables go
    to the device once (adp_fb_set); each search step is the cross-section
    update at the iterate on the device (adp_fb_updt) and a warm-started
    outer on the GPU.  Timed end to end (wall clock,
    synchronised); device_ms sums the outer calls.  CPU baseline: the
    oracle's whole search on one host core."""
    import multiprocessing as mp

    import torch

    from adpres_gb300 import deck, synth
    from adpres_gb300.core import Core
    from adpres_gb300.feedback import cbsearch

    text = synth.boron_search_3d(0)
    dk = deck.parse(text)
    ctx = mp.get_context("spawn")
    with ctx.Pool(1) as pool:
        t_cpu, it_cpu = pool.apply(_cbsearch_oracle, (text,))
    out = {"workload": "boron_search_3d seed 0: 34x34 radial nodes x 22 planes, 2 groups, SANM, boron, fuel and "
                       "moderator temperature, coolant density and 2 rod banks",
           "nodes": int(dk.nnod), "oracle": {"iterates": len(it_cpu), "bcon": it_cpu[-1][0], "keff": it_cpu[-1][1],
                                             "outers": int(sum(r[2] for r in it_cpu))}}
    for prec in ("fp64", "mixed"):
        c = Core.from_deck(dk, precision=prec)
        cbsearch(c, dk)
        walls, devs = [], []
        for _ in range(steps):
            c.reset()
            flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            it = cbsearch(c, dk)
            torch.cuda.synchronize()
            walls.append(time.perf_counter() - t0)
            devs.append(c.cbsearch_device_ms)
        out[prec] = {"searches_per_s": steps / sum(walls), "ms_per_search": sum(walls) / steps * 1e3,
                     "device_ms": sum(devs) / steps, "iterates": len(it), "bcon": it[-1][0], "keff": it[-1][1],
                     "outers": int(sum(r[2] for r in it)), "dbcon_ppm_vs_oracle": abs(it[-1][0] - it_cpu[-1][0])}
        c.close()
    out["cpu_baseline"] = {"value": 1.0 / t_cpu, "unit": "searches/s", "cores": 1, "kind": "port",
                           "sample": f"the oracle's whole search on this core ({t_cpu:.2f} s)"}
    return out


# ---------------------------------------------------- transient leg ----
def _transient_oracle(text):
    import oracle
    o = oracle.Oracle(text=text)
    t0 = time.perf_counter()
    r = o.rodeject()
    return time.perf_counter() - t0, r


def transient_leg(steps=2):
    """rod_eject on the 34x34x22-node core (seed 0): steady state with k
    brought to one, adjoint weight, then 18 time steps (bank 1 ejected in
    0.05 s, theta 0.5); each step XS_updt at the new bank positions on the
    host, then removal, external source, outer_tr, precursors, power and
    reactivity on the GPU.  FP64 handle (the FP64 kernel) and mixed handle
    (the mixed kernel with the step's external source, the nodal update in
    FP64 either way), each timed end to end (wall clock); the mixed run's
    relative power and reactivity against the FP64 run's, step by step.
    The oracle's whole transient on one host core is the CPU baseline."""
    import multiprocessing as mp

    import numpy as np

    from adpres_gb300 import deck, synth
    from adpres_gb300.core import Core
    from adpres_gb300.transient import rod_eject

    text = synth.rod_ejection_3d(0)
    dk = deck.parse(text)
    ctx = mp.get_context("spawn")
    with ctx.Pool(1) as pool:
        t_cpu, ref = pool.apply(_transient_oracle, (text,))

    def run(prec):
        walls, parts, rec = [], [], None
        for i in range(steps + 1):
            core = Core.from_deck(dk, precision=prec)
            t0 = time.perf_counter()
            rec = rod_eject(core, dk)
            if i:
                walls.append(time.perf_counter() - t0)
                parts.append(core.rod_eject_wall)
            core.close()
        return sum(walls) / len(walls), parts, rec

    t, parts, rec = run("fp64")
    tm, parts_m, rec_m = run("mixed")
    pw = np.array([r[2] for r in ref])
    got = np.array([r[2] for r in rec])
    got_m = np.array([r[2] for r in rec_m])
    nsteps = len(rec) - 1
    return {"workload": "rod_ejection_3d seed 0: 34x34 radial nodes x 22 planes, 2 groups, SANM, 18 steps "
                        "(0.01 s to 0.1 s, then 0.05 s), theta 0.5",
            "nodes": int(dk.nnod), "steps": nsteps, "ms_per_transient": t * 1e3, "steps_per_s": nsteps / t,
            "outers": int(sum(r[4] for r in rec[1:])), "device_ms": float(sum(r[5] for r in rec[1:])),
            "steady_state_ms": 1e3 * sum(p[0] for p in parts) / len(parts),
            "steps_wall_ms": 1e3 * sum(p[1] for p in parts) / len(parts),
            "peak_relpow": float(got.max()), "max_relpow_diff_vs_oracle": float(np.max(np.abs(got - pw) / pw)),
            "mixed": {"ms_per_transient": tm * 1e3, "steps_per_s": nsteps / tm,
                      "outers": int(sum(r[4] for r in rec_m[1:])), "device_ms": float(sum(r[5] for r in rec_m[1:])),
                      "steady_state_ms": 1e3 * sum(p[0] for p in parts_m) / len(parts_m),
                      "steps_wall_ms": 1e3 * sum(p[1] for p in parts_m) / len(parts_m),
                      "max_relpow_diff_vs_fp64": float(np.max(np.abs(got_m - got) / got)),
                      "max_rho_diff_vs_fp64": float(np.max(np.abs(np.array([r[1] for r in rec_m])
                                                                  - np.array([r[1] for r in rec])))),
                      "steps_at_nout": int(sum(1 for r in rec_m[1:] if r[3]))},
            "cpu_baseline": {"value": nsteps / t_cpu, "unit": "time steps/s", "cores": 1, "kind": "port",
                             "sample": f"the oracle's whole transient on this core ({t_cpu:.1f} s)"}}


# ------------------------------------------------- batched solves leg ----
def _batch_oracle_member(args):
    seed, i = args
    import oracle
    from adpres_gb300 import synth
    o = oracle.Oracle(text=synth.batch_member(seed, i))
    t0 = time.perf_counter()
    o.run()
    return time.perf_counter() - t0


def batch_leg(flush, dist=None, steps=3, warmup=3, ncores=256, fp64_check=256):
    """256 independent two-group cores (radial 20..68, axial 10..40 nodes,
    config-1 cross sections with 1% lognormal perturbations) in one
    persistent launch replayed from a CUDA graph, mixed precision, schedule
    from the autotuner (cached per batch shape).  Members are those of the
    seeded draw that the reference algorithm converges on
    (tests/golden/batch_members.json).  With N > 1 ranks the members are
    split over the GPUs (adpres_gb300/partition.py: balanced by box rows x
    groups, no data-path collective, results gathered on rank 0) and the
    time of a step is the slowest rank's.  Per-instance |dk| against
    individual single-core FP64 solves; CPU baseline: the oracle on a sample
    of members, one process per host core (both with one rank only)."""
    import multiprocessing as mp

    import numpy as np
    import torch

    from adpres_gb300 import deck, synth
    from adpres_gb300.core import Core
    from adpres_gb300.partition import DistributedBatch, loads

    with open(os.path.join(ROOT, "tests", "golden", "batch_members.json")) as f:
        acc = json.load(f)
    seed, idx = acc["seed"], acc["accepted"][:ncores]
    texts = [synth.batch_member(seed, i) for i in idx]
    decks = [deck.parse(t) for t in texts]
    nodes = int(sum(len(d.ix) for d in decks))
    t0 = time.perf_counter()
    db = DistributedBatch(decks, dist=dist, precision="mixed")
    t_create = time.perf_counter() - t0
    cache = os.path.join(os.path.expanduser("~"), ".cache", "adpres_gb300", "batch_tune.json")
    t0 = time.perf_counter()
    props = torch.cuda.get_device_properties(torch.cuda.current_device())
    device_key = "sm%d%dx%d" % (props.major, props.minor, props.multi_processor_count)
    tuned = db.autotune(cache, device_key)
    cfg, tune_ms, hit = tuned if tuned else (None, 0.0, False)
    t_tune = time.perf_counter() - t0

    def one_step():
        if dist is not None:
            dist.barrier()
        return db.solve()

    for _ in range(warmup):
        one_step()
    ms = []
    for _ in range(steps):
        flush.zero_()
        torch.cuda.synchronize()
        res, _, secs = one_step()
        ms.append(secs * 1e3)
    t = sum(ms) / len(ms) / 1e3
    part = {"ranks": db.world, "members_per_rank": [len(p) for p in db.parts],
            "load_max_over_mean": max(loads(db.weights, db.parts)) / (sum(db.weights) / db.world)}
    db.close()
    if db.rank != 0:
        return None
    if db.world > 1:
        return {"workload": f"{len(decks)} two-group cores, {nodes} nodes in all, split over {db.world} GPUs",
                "value": len(decks) / t, "unit": "solves/s", "ms_per_batch": t * 1e3, "steps": steps,
                "warmup": warmup, "scaling": "strong", "partition": part,
                "converged": sum(r["converged"] for r in res), "config_rank0": cfg}
    conv = sum(r["converged"] for r in res)
    # individual FP64 single-core solves
    dks, outs64, k64 = [], [], []
    t0 = time.perf_counter()
    for i in range(min(fp64_check, len(decks))):
        c = Core.from_deck(decks[i], precision="fp64")
        r = c.outer(trace=False)
        dks.append(abs(res[i]["keff"] - r.keff) / r.keff * 1e5)
        outs64.append(r.outers)
        k64.append(r.keff)
        c.close()
    t_fp64 = time.perf_counter() - t0
    # the worst member against its fixed point: a tight FP64 solve (criteria
    # 1e-10) tells how far the loosely converged end points (ser, fer < 1e-5,
    # ndmax < 1e-2) of the batch and of the single solve each sit from it
    wi = int(np.argmax(dks))
    c = Core.from_deck(decks[wi], precision="fp64", serc=1e-10, ferc=1e-10)
    rt = c.outer(trace=False)
    c.close()
    worst_tight = {"k_tight": rt.keff, "outers_tight": rt.outers,
                   "batch_pcm_from_tight": abs(res[wi]["keff"] - rt.keff) / rt.keff * 1e5}
    # CPU baseline: the oracle on a sample, all host cores
    nproc = os.cpu_count() or 1
    sample = [(seed, i) for i in idx[:nproc]]
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(nproc) as pool:
        tcpu = pool.map(_batch_oracle_member, sample)
    wall = time.perf_counter() - t0
    cpu_rate = len(sample) / wall
    return {
        "workload": f"{len(decks)} two-group cores, radial 20..68, axial 10..40 nodes, {nodes} nodes in all "
                    "(seeded draw, members the reference converges on), SANM, mixed precision",
        "value": len(decks) / t, "unit": "solves/s", "ms_per_batch": t * 1e3, "steps": steps, "warmup": warmup,
        "converged": conv, "config": cfg, "tuned_from_cache": hit, "tune_s": t_tune, "create_s": t_create,
        "device_key": device_key,
        "outers_mean": float(np.mean([r["outers"] for r in res])),
        "teams": sorted({r["team"] for r in res}),
        # share of the launch's block-time spent inside some core's solve
        # (each core's start-to-end time x its team size over blocks x the
        # batch time): what the schedule leaves idle at the tail
        "block_time_used": (sum(r["device_ms"] * r["team"] for r in res)
                            / (props.multi_processor_count * int((cfg or {}).get("blocks_per_sm", 1)) * ms[-1])),
        "dk_pcm_vs_fp64_single": {"max": float(max(dks)), "rms": float(np.sqrt(np.mean(np.square(dks)))),
                                  "checked": len(dks), "fp64_single_s": t_fp64,
                                  "above_1pcm": int(sum(d > 1.0 for d in dks)),
                                  "worst": {"member": wi, "outers_mixed": int(res[wi]["outers"]),
                                            "outers_fp64": int(outs64[wi]), "fp64_single_pcm_from_tight":
                                                abs(k64[wi] - worst_tight["k_tight"]) / worst_tight["k_tight"] * 1e5,
                                            **worst_tight},
                                  "same_outers": int(sum(res[i]["outers"] == outs64[i] for i in range(len(dks))))},
        "cpu_baseline": {"value": cpu_rate, "unit": "solves/s", "cores": nproc, "kind": "port",
                         "sample": f"oracle full solves of the first {len(sample)} members, one process per host core, "
                                   f"wall {wall:.1f} s (mean {np.mean(tcpu):.1f} s per member)"},
        "l2_flush": "256 MiB written between steps", "partition": part,
    }


def batch_stated_leg(flush, cfg, steps=2, warmup=1, ncores=256):
    """The batched workload as stated for it, unfiltered: 256 draws of
    synth.batch_member_stated (config-1 cross-section sets including the
    rodded region, 1% lognormal factors, the default nodal-update interval),
    solved in one launch with the first leg's tuned configuration (applied
    as a cached one: three timed solves, each followed by a re-plan), mixed
    precision.  Counts the members whose two-node iteration diverges (in the
    batch and in single FP64 solves) and those more than 1 pcm from their
    single FP64 solve."""
    import numpy as np
    import torch

    from adpres_gb300 import _lib, deck, synth
    from adpres_gb300._lib import AdpError
    from adpres_gb300.batch import Batch
    from adpres_gb300.core import Core

    decks = [deck.parse(synth.batch_member_stated(0, i)) for i in range(ncores)]
    nodes = int(sum(len(d.ix) for d in decks))
    b = Batch(decks, precision="mixed")
    if cfg:
        # as a cached configuration: timed solves and re-plans first
        b.apply_config(cfg)
    for _ in range(warmup):
        b.solve(check=False)
    ms = []
    for _ in range(steps):
        flush.zero_()
        torch.cuda.synchronize()
        res, m = b.solve(check=False)
        ms.append(m)
    b.close()
    t = sum(ms) / len(ms) / 1e3
    single = []
    for dk in decks:
        c = Core.from_deck(dk, precision="fp64")
        try:
            r = c.outer(trace=False)
            single.append((0, r.keff, r.outers))
        except AdpError as e:
            single.append((e.status, None, None))
        c.close()
    div_b = [i for i, r in enumerate(res) if r["status"] == _lib.ADP_ERR_DIVERGED]
    div_s = [i for i, r in enumerate(single) if r[0] == _lib.ADP_ERR_DIVERGED]
    both = [i for i in range(ncores) if res[i]["status"] == 0 and res[i]["converged"] and single[i][0] == 0]
    dpcm = np.array([abs(res[i]["keff"] - single[i][1]) / single[i][1] * 1e5 for i in both])
    return {"workload": f"{ncores} unfiltered draws of synth.batch_member_stated, {nodes} nodes in all, "
                        "config-1 sets with the rodded region, default nupd, mixed precision",
            "value": ncores / t, "unit": "solves/s (every member, diverged ones included)", "ms_per_batch": t * 1e3,
            "steps": steps, "warmup": warmup, "config": cfg,
            "converged": int(sum(1 for r in res if r["status"] == 0 and r["converged"])),
            "diverged_batch": len(div_b), "diverged_fp64_single": len(div_s),
            "diverged_both": len(set(div_b) & set(div_s)),
            "other_status": sorted({int(r["status"]) for r in res if r["status"] not in (0, _lib.ADP_ERR_DIVERGED)}),
            "dk_pcm_vs_fp64_single": {"compared": len(both), "max": float(dpcm.max()) if len(dpcm) else None,
                                      "rms": float(np.sqrt(np.mean(dpcm ** 2))) if len(dpcm) else None,
                                      "above_1pcm": int(np.sum(dpcm > 1.0))},
            "outers_mean": float(np.mean([r["outers"] for r in res]))}


# ------------------------------------------------------------ our arm ----
def run_ours(args):
    import numpy as np
    import torch

    from adpres_gb300 import _lib, deck, perfmodel
    from adpres_gb300.core import Core

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    if not os.path.exists(_lib.LIB_PATH):
        from adpres_gb300 import build as libbuild
        libbuild.build()

    text = workload_text()
    dk = deck.parse(text)
    prec = args.precision
    core = Core.from_deck(dk, precision=prec)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")

    def step(c):
        c.reset()
        return c.outer(adjoint=False, popt=1, trace=False)

    for _ in range(args.warmup):
        step(core)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    t_before = core.timers()
    clocks = Clocks(local)
    dev_ms, outers, nodal = [], [], []
    torch.cuda.synchronize()
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        rep = step(core)
        dev_ms.append(rep.device_ms)
        outers.append(rep.outers)
        nodal.append(rep.nodal_updates)
    torch.cuda.synchronize()
    ck = clocks.stop()
    t_after = core.timers()
    total_s = max_over_ranks(dist, sum(dev_ms) / 1e3)
    value = world * args.steps / total_s
    keff_mixed = rep.keff
    p_mixed = core.power()

    # dominant kernel: the persistent outer-iteration kernel
    launches = t_after["outer_kernel_launches"] - t_before["outer_kernel_launches"]
    kms = t_after["outer_kernel_ms"] - t_before["outer_kernel_ms"]
    n_outers = sum(outers)
    NB = dk.nxx * dk.nyy * dk.nzz
    # canonical algorithmic bytes (w = 4 for the FP32-storage form, 8 FP64)
    w = 4 if prec == "mixed" else 8
    canon_per_outer = dk.nnod * perfmodel.canonical_bytes_per_node_outer(dk.ng, dk.nin, w)
    bytes_per_launch = canon_per_outer * n_outers / launches
    avg_launch_s = kms / 1e3 / launches
    achieved = bytes_per_launch / avg_launch_s / 1e9
    # the kernel's own count: the words it moves at their stored widths (the
    # FP64 / double-float P0 operands at 8 bytes)
    kernel_bytes_per_launch = NB * perfmodel.bytes_per_row_outer(dk.ng, dk.nin, dk.nac, prec) * n_outers / launches
    # the all-zero source planes P0 leaves out (counted by the canonical figure)
    skipped_per_launch = NB * perfmodel.p0_skipped_bytes_per_row_outer(dk.xsigs, dk.chi, dk.mat) * n_outers / launches
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(peaks_path):
        with open(peaks_path) as f:
            peak = float(json.load(f)["hbm_gbs"])
        peak_src = "measured"
    else:
        peak, peak_src = 6800.0, "fallback"
    # DRAM traffic of one launch: the ncu capture of the 68x68x40 core's first
    # launch gives the bytes per box row and outer; scaled to this launch by
    # box rows x outers per launch (the same kernel on twice the planes)
    traffic, traffic_src = None, None
    prof = os.path.join(ROOT, "profiles", "k_outer_mixed_core_4g_planes80_dram.json")
    if os.path.exists(prof) and prec == "mixed":
        with open(prof) as f:
            pj = json.load(f)
        traffic = pj["dram_bytes_per_outer"] * n_outers / launches
        traffic_src = pj["capture"]
    gpu_launches = int(sum(2 + 0 for _ in outers) + launches + 5 * sum(nodal))

    # FP64 path on the same core: solves/s and the mixed-precision error
    core64 = Core.from_deck(dk, precision="fp64")
    for _ in range(args.warmup):
        step(core64)
    d64 = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        r64 = step(core64)
        d64.append(r64.device_ms)
    p64 = core64.power()
    fp64_value = args.steps / (sum(d64) / 1e3)
    dk_pcm = abs(keff_mixed - r64.keff) / r64.keff * 1e5
    m = p64 > 0
    perr = np.abs(p_mixed[m] - p64[m]) / p64[m]
    core64.close()

    # single-GPU legs reported by rank 0 only; with N ranks the others go
    # straight to the batched leg's first barrier
    adjoint = adjoint_leg(flush) if rank == 0 else None
    boron = cbsearch_leg(flush) if rank == 0 else None
    transient = transient_leg() if rank == 0 else None
    batched = batch_leg(flush, dist) if not args.no_batch else None
    batched_stated = (batch_stated_leg(flush, batched.get("config")) if batched and world == 1 else None)

    # e2e through the C ABI from host buffers: the inputs sit in pinned host
    # memory in the reference's column-major layouts (set up before timing)
    e2e_steps = max(2, min(args.steps, 5))
    keep = []

    def pinned(a, dt=np.float64):
        flat = np.asfortranarray(a, dtype=dt).reshape(-1, order="F")
        t = torch.empty(flat.size, dtype=torch.float64 if dt == np.float64 else torch.int32, pin_memory=True)
        v = t.numpy()
        v[:] = flat
        keep.append(t)
        return v.reshape(np.shape(a), order="F")

    xin = [pinned(a) for a in (dk.xsigtr, dk.xsiga, dk.xnuf, dk.xsigf, dk.chi)]
    mat_p, sigs_p, dc_p = pinned(dk.mat, np.int32), pinned(dk.xsigs), pinned(dk.dc)
    h2d = sum(a.nbytes for a in xin) + mat_p.nbytes + sigs_p.nbytes + dc_p.nbytes
    d2h = dk.nnod * 8 + dk.nnod * dk.ng * 8
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        core.xs_updt(*xin, mat_p, sigs_p, dc_p)
        core.reset()
        core.outer(adjoint=False, popt=1, trace=False)
        core.power()
        core.flux()
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(dist, time.perf_counter() - t0)
    e2e_value = world * e2e_steps / e2e_s

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    cpu = cpu_baseline_single(text) if world == 1 else None
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_s * 1e3 / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 Krylov steps / double-float (f32 pair) residual and reductions" if prec == "mixed" else "f64",
        "data": "synthetic (seeded core, reference deck format)", "config": workload_config(dk, prec),
        "outers_per_solve": statistics.mean(outers), "nodal_updates_per_solve": statistics.mean(nodal),
        "keff": keff_mixed,
        "fp64": {"value": fp64_value, "unit": UNIT, "keff": r64.keff, "outers": r64.outers,
                 "steps": args.steps, "mixed_speedup": value / fp64_value},
        "accuracy_vs_fp64": {"dk_pcm": dk_pcm, "power_max_rel": float(perr.max()),
                             "power_rms_rel": float(np.sqrt(np.mean(perr ** 2)))},
        "roofline": {"kernel": "k_outer<mixed>" if prec == "mixed" else "k_outer<fp64>", "bound": "hbm",
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_src, "traffic": traffic, "traffic_source": traffic_src,
                     "bytes": "canonical: nodes x %d B per outer (w = %d)" % (
                         perfmodel.canonical_bytes_per_node_outer(dk.ng, dk.nin, w), w),
                     "algorithmic_bytes_per_launch": bytes_per_launch, "avg_launch_ms": avg_launch_s * 1e3,
                     "launches": launches, "outers_per_launch": n_outers / launches,
                     "kernel_count_bytes_per_launch": kernel_bytes_per_launch,
                     "kernel_count_achieved": kernel_bytes_per_launch / avg_launch_s / 1e9,
                     "kernel_count_frac": kernel_bytes_per_launch / avg_launch_s / 1e9 / peak,
                     "p0_zero_plane_bytes_skipped_per_launch": skipped_per_launch},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
        "adjoint": adjoint,
        "cbsearch": boron,
        "transient": transient,
        "batched": batched,
        "batched_stated": batched_stated,
        "gpu_launches": gpu_launches,
        "clocks": ck,
        "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


# ---------------------------------------------------- replicas (N > 1) ----
def max_over_ranks(dist, x):
    """The largest of every rank's x (the slowest replica's time); x itself
    when there is one rank.  NCCL reduces a device tensor, gloo a host one."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(x)
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------------ reference arm ----
def run_reference(args):
    """The reference arm: the oracle (CPU restatement of the reference's
    loops; no Fortran compiler exists here) on all host cores, one process
    per core.  Warm-up: every process times one full solve of the workload
    from a cold start, which gives the solve's outers and nodal updates.
    Each timed step: every process times a bounded sample (the first outer
    call with its start, the cost of an outer from two warm calls, one nodal
    update: cpu_sample), whose model time t_first + (outers - 1) x t_outer
    + nodal x t_nodal is scaled by the ratio of the warm-up's measured full
    solves to the same model on the warm-up's samples (the model alone
    misses per-outer work that the short calls do not show, on both sides
    of 1 by machine); solves/s = processes / that time.  The line reports
    the warm-up's measured full solves/s and the calibration."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import oracle
    from adpres_gb300 import deck
    oracle.build()
    text = workload_text()
    dk = deck.parse(text)
    cores = os.cpu_count() or 1
    outers = CPU_SAMPLE_OUTERS
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        t0 = time.perf_counter()
        full = pool.map(_full_worker, [text] * cores)
        full_wall = time.perf_counter() - t0
        warm = []
        for _ in range(max(1, args.warmup - 1)):
            warm.extend(pool.map(_worker, [(text, outers)] * cores))
        times = []
        per = []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            res = pool.map(_worker, [(text, outers)] * cores)
            times.append(time.perf_counter() - t0)
            per.extend(res)
    n_out, n_nod = full[0][1], full[0][2]
    def model(rs):
        return (statistics.mean(r[0] for r in rs) + (n_out - 1) * statistics.mean(r[1] for r in rs)
                + n_nod * statistics.mean(r[2] for r in rs))

    calib = statistics.mean(f[0] for f in full) / model(warm)
    est = model(per) * calib
    value = cores / est
    measured = cores / full_wall
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": statistics.mean(times) * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded core, reference deck format)",
        "config": workload_config(dk, "fp64"), "impl": "reference",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"each step: {cores} independent processes, each timing the oracle's (CPU "
                                   f"restatement of the reference loops) first outer call with its start, "
                                   f"{outers} more outers (the difference of two warm calls) and one nodal update on "
                                   f"this core; solves/s = processes / (t_first + {n_out - 1} x t_outer + {n_nod} x "
                                   f"t_nodal), times {calib:.3f} (the warm-up's full solves over the same model on "
                                   f"its samples) = {cores} / {est:.1f} s, with {n_out} outers and {n_nod} nodal "
                                   f"updates from the warm-up's full solves"},
        "full_solves_in_warmup": {"value": measured, "unit": UNIT, "processes": cores, "wall_s": full_wall,
                                  "per_process_s": [round(f[0], 2) for f in full], "outers": n_out,
                                  "nodal_updates": n_nod, "sample_over_measured": value / measured,
                                  "calibration": calib},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--precision", choices=["mixed", "fp64"], default="mixed")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-solves leg")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        log("warm-up raised to 3 steps")
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
