"""Batched solves split over ranks (adpres_gb300/partition.py) on the CPU:
the assignment is balanced by box rows x groups and the same on every
rank; two gloo ranks each solve their share (here with the oracle as the
solver, one process per rank) and rank 0 gathers every member's k and
power in the batch's order, equal to solving the whole batch in one
process."""
import os
import socket
import sys

import numpy as np
import torch.multiprocessing as tmp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from adpres_gb300 import deck, synth  # noqa: E402
from adpres_gb300.partition import loads, member_weight, partition  # noqa: E402


def test_partition_is_balanced_and_complete():
    rng = np.random.default_rng(0)
    w = rng.integers(1, 100, 257).astype(float)
    for n in (1, 2, 3, 4, 8):
        parts = partition(w, n)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(w)))
        L = loads(w, parts)
        # longest-processing-time bound: max load <= mean + largest item
        assert max(L) <= sum(w) / n + max(w)
        assert partition(w, n) == parts          # deterministic: every rank computes the same
    assert partition([5.0, 5.0], 4) == [[0], [1], [], []]


def _decks():
    texts = [synth.small_core(seed=s, ng=2, nx=3 + (s % 3), ny=3 + (s % 2), nz=2 + (s % 2)) for s in range(7)]
    return texts, [deck.parse(t) for t in texts]


def _oracle_solver(dks):
    """The rank's share solved by the oracle, one member after another."""
    import oracle
    res, pw = [], []
    for dk in dks:
        o = oracle.Oracle(text=dk.text)
        o.run()
        res.append({"keff": o.getd("Ke"), "outers": o.geti("outers"), "converged": 1})
        pw.append(o.powdis())
    return res, pw


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    from adpres_gb300.partition import DistributedBatch
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        texts, dks = _decks()
        for t, dk in zip(texts, dks):
            dk.text = t
        db = DistributedBatch(dks, dist=dist, solver=_oracle_solver)
        res, pw, secs = db.solve()
        out.put((rank, db.mine, None if res is None else [r["keff"] for r in res],
                 None if pw is None else [p.tolist() for p in pw], secs))
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_gather_every_member():
    import oracle
    world = 2
    ctx = tmp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in ps:
        p.start()
    got = sorted(q.get(timeout=300) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    texts, dks = _decks()
    parts = partition([member_weight(d) for d in dks], world)
    assert [g[1] for g in got] == parts
    assert got[1][2] is None and got[1][3] is None
    k0, p0 = got[0][2], got[0][3]
    assert len(k0) == len(dks)
    for i, t in enumerate(texts):
        o = oracle.Oracle(text=t)
        o.run()
        assert k0[i] == o.getd("Ke")
        np.testing.assert_array_equal(np.array(p0[i]), o.powdis())
    assert got[0][4] == got[1][4]             # both ranks see the slowest rank's time
