"""The batch tuning cache on the host (no GPU): ranks that share the cache
path never read a partial file, and a damaged or foreign file reads as an
empty cache instead of failing the solve."""
import json
import multiprocessing as mp
import os


def _writer(args):
    path, rank, rounds = args
    from adpres_gb300.batch import _read_cache, _write_cache
    for i in range(rounds):
        db = _read_cache(path)   # must never raise, even mid-write of another rank
        db["rank%d-%d" % (rank, i)] = {"config": {"threads": 256}, "ms": float(i)}
        _write_cache(path, db)
    return True


def test_concurrent_writers_never_leave_a_partial_file(tmp_path):
    path = str(tmp_path / "cache" / "batch_tune.json")
    with mp.get_context("spawn").Pool(4) as pool:
        assert all(pool.map(_writer, [(path, r, 25) for r in range(4)]))
    with open(path) as f:
        db = json.load(f)
    assert isinstance(db, dict) and len(db) >= 25
    assert not [n for n in os.listdir(os.path.dirname(path)) if n.endswith(".tmp")]


def test_damaged_or_foreign_cache_reads_as_empty(tmp_path):
    from adpres_gb300.batch import _read_cache
    p = tmp_path / "c.json"
    assert _read_cache(str(p)) == {}
    p.write_text('{"half": ')
    assert _read_cache(str(p)) == {}
    p.write_text("[1, 2]")
    assert _read_cache(str(p)) == {}
