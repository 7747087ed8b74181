"""The batch planner on the host (adp_batch_plan_preview, no GPU): the
schedule k_batch runs, from box-row weights (before any solve is timed)
and from measured per-core times (the target-end plan).

Properties checked on seeded workloads shaped like the batched workload
(256 cores of 20..68 x 20..68 x 10..40 nodes on 152 or 304 blocks) and on
more cores than blocks:
  * every core runs on exactly team[i] distinct blocks, ranks 0..team-1,
    team within [1, max_team];
  * the block lists are subsequences of one global order of the cores, so
    no cycle of teams waiting on each other can form (the kernel's
    deadlock-freedom argument);
  * the timed plan's predicted end is within 10% of its lower bound (the
    least block-time of all cores spread over the blocks, or the longest
    core at max_team) and no later than the untimed plan's under the same
    durations;
  * bad arguments are refused.
"""
import ctypes

import numpy as np
import pytest

from adpres_gb300 import _lib

KAPPA = 0.03   # the preview's duration model t(s) = A (1/s + KAPPA)


def _lib_loaded():
    try:
        return _lib.load()
    except Exception as e:   # the library is built by build(); skip where it is absent
        pytest.skip("library not built: %s" % e)


def preview(rows, blocks, max_team, grain=1.0, t=None, tteam=None):
    L = _lib_loaded()
    n = len(rows)
    rows = np.ascontiguousarray(rows, dtype=np.float64)
    cap = n * max_team
    team = np.zeros(n, np.int32)
    begin = np.zeros(blocks + 1, np.int32)
    core = np.zeros(cap, np.int32)
    rank = np.zeros(cap, np.int32)
    mk = ctypes.c_double()
    cfg = _lib.AdpBatchConfig(256, max_team, grain, 1, 1)
    tp = tt = None
    if t is not None:
        t = np.ascontiguousarray(t, dtype=np.float64)
        tteam = np.ascontiguousarray(tteam, dtype=np.int32)
        tp, tt = _lib.dptr(t), _lib.iptr(tteam)
    st = L.adp_batch_plan_preview(n, _lib.dptr(rows), tp, tt, blocks, ctypes.byref(cfg), cap, _lib.iptr(team),
                                  _lib.iptr(begin), _lib.iptr(core), _lib.iptr(rank), ctypes.byref(mk))
    return st, team, begin, core[:begin[-1]], rank[:begin[-1]], mk.value


def workload(seed, n=256):
    rng = np.random.default_rng(seed)
    nxy = rng.integers(20, 69, n)
    nz = rng.integers(10, 41, n)
    rows = (nxy * nxy * nz * 2).astype(np.float64)
    # measured-like times: work ~ rows x outers on one block, outers 69..414
    outers = rng.integers(69, 415, n)
    t1 = rows * outers * 1e-3
    return rows, t1


def dur(t1, s):
    # the preview's model from a time on one block
    return t1 * (1.0 / s + KAPPA) / (1.0 + KAPPA)


def check_structure(n, blocks, max_team, team, begin, core, rank):
    assert team.min() >= 1 and team.max() <= max_team
    assert len(core) == int(team.sum())
    where = {}
    for b in range(blocks):
        for k in range(begin[b], begin[b + 1]):
            where.setdefault(int(core[k]), []).append((b, int(rank[k])))
    assert sorted(where) == list(range(n))
    for i, places in where.items():
        assert len(places) == team[i]
        assert len({b for b, _ in places}) == team[i]          # distinct blocks
        assert sorted(r for _, r in places) == list(range(team[i]))
    # one global order: position of each core in the order of first appearance
    # over a topological merge must agree with every block's list
    pos = {}
    lists = [list(core[begin[b]:begin[b + 1]]) for b in range(blocks)]
    before = {}
    for lst in lists:
        for a, c in zip(lst, lst[1:]):
            before.setdefault(int(a), set()).add(int(c))
    # the relation "a before c in some list" must be acyclic
    state = {}

    def visit(u):
        state[u] = 1
        for v in before.get(u, ()):
            if state.get(v) == 1:
                return False
            if state.get(v) is None and not visit(v):
                return False
        state[u] = 2
        return True

    import sys
    sys.setrecursionlimit(10000)
    for u in range(n):
        if state.get(u) is None:
            assert visit(u), "block lists order two cores both ways: teams could wait on each other"


@pytest.mark.parametrize("seed,blocks,max_team", [(0, 304, 32), (1, 152, 8), (2, 304, 4)])
def test_untimed_plan_structure(seed, blocks, max_team):
    rows, _ = workload(seed)
    st, team, begin, core, rank, mk = preview(rows, blocks, max_team, grain=4.0)
    assert st == 0 and mk > 0
    check_structure(len(rows), blocks, max_team, team, begin, core, rank)


@pytest.mark.parametrize("seed,blocks,max_team", [(0, 304, 32), (1, 304, 8), (2, 152, 16), (3, 304, 2)])
def test_timed_plan_structure_and_end(seed, blocks, max_team):
    rows, t1 = workload(seed)
    n = len(rows)
    st, team, begin, core, rank, mk = preview(rows, blocks, max_team, t=t1, tteam=np.ones(n, np.int32))
    assert st == 0
    check_structure(n, blocks, max_team, team, begin, core, rank)
    work = sum(min(s * dur(t1[i], s) for s in range(1, max_team + 1)) for i in range(n)) / blocks
    longest = max(dur(t1[i], max_team) for i in range(n))
    lb = max(work, longest)
    assert lb <= mk <= 1.10 * lb, (mk / lb)
    # the untimed plan, replayed with the same durations, ends no earlier
    st2, team2, begin2, core2, rank2, _ = preview(rows, blocks, max_team, grain=1.0)
    assert st2 == 0
    load = np.zeros(blocks)
    seen = set()
    lists = [list(core2[begin2[b]:begin2[b + 1]]) for b in range(blocks)]
    cores_of = {}
    for b, lst in enumerate(lists):
        for c in lst:
            cores_of.setdefault(int(c), []).append(b)
    # replay in the global order (first appearance across lists is consistent)
    order = []
    ptr = [0] * blocks
    while len(order) < n:
        progressed = False
        for b in range(blocks):
            if ptr[b] < len(lists[b]):
                c = int(lists[b][ptr[b]])
                if c in seen:
                    continue
                if all(lists[bb][ptr[bb]] == c for bb in cores_of[c] if ptr[bb] < len(lists[bb])):
                    bs = cores_of[c]
                    t0 = max(load[bb] for bb in bs)
                    for bb in bs:
                        load[bb] = t0 + dur(t1[c], team2[c])
                        ptr[bb] += 1
                    seen.add(c)
                    order.append(c)
                    progressed = True
        assert progressed
    assert mk <= load.max() * 1.0001


def test_more_cores_than_blocks():
    rng = np.random.default_rng(7)
    n, blocks = 1000, 304
    rows = rng.uniform(100, 5000, n)
    t1 = rows * rng.uniform(0.5, 2.0, n)
    st, team, begin, core, rank, mk = preview(rows, blocks, 8, t=t1, tteam=np.ones(n, np.int32))
    assert st == 0
    check_structure(n, blocks, 8, team, begin, core, rank)
    lb = max(sum(dur(t1[i], 1) for i in range(n)) / blocks, max(dur(t1[i], 8) for i in range(n)))
    assert mk <= 1.10 * lb


def test_bad_arguments_are_refused():
    rows = np.ones(4)
    assert preview(rows, 0, 4)[0] == _lib.ADP_ERR_INPUT
    assert preview(np.array([1.0, -1.0]), 8, 4)[0] == _lib.ADP_ERR_INPUT
    assert preview(rows, 8, 4, t=np.array([1.0, 1.0, 0.0, 1.0]), tteam=np.ones(4, np.int32))[0] == _lib.ADP_ERR_INPUT
