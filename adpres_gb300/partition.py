"""Batched solves partitioned over GPUs, one process per GPU.

The members of a batch are independent cores, so a batch splits across
GPUs with no exchange on the data path: each rank solves its share with its
own ``Batch`` on its own GPU, and the per-member results (k, outers, flags,
nodal power) are gathered on rank 0 over the host (``torch.distributed``
object collectives, NCCL or gloo).  The reference solves one core per
process (mod_control.f90:11-47); this has no counterpart there.

Shares are balanced by each member's work estimate, box rows x groups
(the same weight the single-GPU schedule starts from): longest first, each
member to the least-loaded rank, ties to the lower rank, so every rank
computes the same assignment without communicating.
"""
from __future__ import annotations

import heapq


def member_weight(dk) -> float:
    """Work estimate of one member: box rows x groups."""
    return float(int(dk.nxx) * int(dk.nyy) * int(dk.nzz) * int(dk.ng))


def partition(weights, nranks):
    """Member indices of each rank, longest-processing-time first; each list
    is in ascending member order."""
    if nranks < 1:
        raise ValueError("nranks must be at least 1")
    order = sorted(range(len(weights)), key=lambda i: (-float(weights[i]), i))
    heap = [(0.0, r) for r in range(nranks)]
    out = [[] for _ in range(nranks)]
    for i in order:
        load, r = heapq.heappop(heap)
        out[r].append(i)
        heapq.heappush(heap, (load + float(weights[i]), r))
    return [sorted(x) for x in out]


def loads(weights, parts):
    return [sum(float(weights[i]) for i in p) for p in parts]


class DistributedBatch:
    """A batch of decks split over the ranks of a process group.

    solver: a callable taking the rank's decks and returning, per deck, a
    dict of results (it must include "keff") and the nodal power; by default
    a ``Batch`` on the rank's current GPU.  ``solve`` returns
    (results, powers, seconds) on rank 0 -- results and powers in the
    batch's member order, seconds the slowest rank's solve time (the
    batch's device time on a GPU, wall time for a given solver) -- and
    (None, None, seconds) elsewhere.
    """

    def __init__(self, decks, dist=None, precision="mixed", solver=None, **over):
        self.decks = list(decks)
        self.dist = dist if (dist is not None and dist.is_initialized()) else None
        self.rank = self.dist.get_rank() if self.dist else 0
        self.world = self.dist.get_world_size() if self.dist else 1
        self.weights = [member_weight(dk) for dk in self.decks]
        self.parts = partition(self.weights, self.world)
        self.mine = self.parts[self.rank]
        self._solver = solver
        self._batch = None
        if solver is None and self.mine:
            from .batch import Batch
            self._batch = Batch([self.decks[i] for i in self.mine], precision=precision, **over)

    def close(self):
        if self._batch is not None:
            self._batch.close()
            self._batch = None

    def autotune(self, cache=None, device=None):
        if self._batch is not None:
            return self._batch.autotune(cache, device)
        return None

    def _local(self):
        import time
        t0 = time.perf_counter()
        if self._solver is not None:
            res, pw = self._solver([self.decks[i] for i in self.mine])
        elif self._batch is not None:
            res, ms = self._batch.solve()
            pw = [self._batch.power(j) for j in range(len(self.mine))]
            return res, pw, ms / 1e3
        else:
            res, pw = [], []
        return res, pw, time.perf_counter() - t0

    def solve(self):
        res, pw, secs = self._local()
        if self.dist is None:
            return res, pw, secs
        mine = list(zip(self.mine, res, pw))
        got = [None] * self.world
        self.dist.all_gather_object(got, (self.rank, mine, secs))
        slowest = max(g[2] for g in got)
        if self.rank != 0:
            return None, None, slowest
        results = [None] * len(self.decks)
        powers = [None] * len(self.decks)
        for _, items, _ in got:
            for i, r, p in items:
                results[i] = r
                powers[i] = p
        return results, powers, slowest
