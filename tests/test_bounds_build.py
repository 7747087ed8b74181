"""The range-checked build (-DADP_BOUNDS): every node index and every
neighbour index the nodal, nodal-adjoint and matrix-assembly stages form is
checked against the box and the active-node mask, a bad one is reported as
ADP_ERR_BOUNDS and its item skipped (nothing traps).  The per-stage tiny-grid
tests, the failure-path tests, the small-core parity tests and batches of
many small ragged cores (teams of one to sixteen blocks) run against that
build, in a child process (one library per process), and pass: no index
leaves its range on any boundary combination."""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_stage_and_failure_tests_pass_under_the_bounds_build():
    sys.path.insert(0, ROOT)
    from adpres_gb300 import build
    lib = build.build(variant="bounds")
    env = dict(os.environ, ADPRES_LIB=lib)
    cmd = [sys.executable, "-m", "pytest", "-q", "-x", "-p", "no:cacheprovider",
           os.path.join(ROOT, "tests", "test_stages_gpu.py"), os.path.join(ROOT, "tests", "test_failures_gpu.py"),
           os.path.join(ROOT, "tests", "test_gpu_parity.py") + "::test_small_cores_match_oracle",
           os.path.join(ROOT, "tests", "test_adjoint_full.py") + "::test_nodal_vjp_matches_autograd",
           os.path.join(ROOT, "tests", "test_batch.py") + "::test_many_small_cores_more_cores_than_blocks",
           os.path.join(ROOT, "tests", "test_batch.py") + "::test_team_sizes_give_the_same_answer"]
    r = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=3000)
    print(r.stdout[-3000:])
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-2000:]
    assert "ADP_ERR_BOUNDS" not in r.stdout
