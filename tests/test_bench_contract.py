"""The bench line's contract on the CPU: the reference arm (the oracle on
the host cores) prints one JSON line with the keys the measurement needs,
and the byte model counts the source planes the outer kernel leaves out."""
import json
import os
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_json_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "0"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["value"] > 0 and d["higher_is_better"] is True
    assert d["config"]["workload"].startswith("core_4g")
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    # the warm-up's measured full solves calibrate the sampled figure
    fw = d["full_solves_in_warmup"]
    assert fw["outers"] > 0 and fw["nodal_updates"] > 0 and fw["value"] > 0
    assert 0.5 < fw["sample_over_measured"] < 2.0


def test_canonical_bytes():
    from adpres_gb300 import perfmodel
    # 4 groups, nin = 2: 339 words per node and outer
    assert perfmodel.canonical_bytes_per_node_outer(4, 2, 8) == 8 * 339
    assert perfmodel.canonical_bytes_per_node_outer(2, 2, 8) == 8 * 163


def test_skipped_source_planes_in_the_byte_model():
    from adpres_gb300 import deck, perfmodel, synth
    # 4 groups, down-scatter only, chi = 0 in groups 3 and 4: 6 + 2 planes
    dk = deck.parse(synth.core_4g(0, planes=20))
    assert perfmodel.p0_skipped_bytes_per_row_outer(dk.xsigs, dk.chi, dk.mat) == 16.0 * 8
    # a plane nonzero in one material in use is kept
    xs = np.array(dk.xsigs, copy=True)
    xs[int(np.asarray(dk.mat)[0]) - 1, 3, 0] = 1e-3
    assert perfmodel.p0_skipped_bytes_per_row_outer(xs, dk.chi, dk.mat) == 16.0 * 7
    # a material not in use does not count
    unused = np.setdiff1d(np.arange(xs.shape[0]), np.unique(dk.mat) - 1)
    if len(unused):
        xs2 = np.array(dk.xsigs, copy=True)
        xs2[unused[0], 3, 0] = 1e-3
        assert perfmodel.p0_skipped_bytes_per_row_outer(xs2, dk.chi, dk.mat) == 16.0 * 8
