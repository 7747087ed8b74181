import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

# The reference project's tree (its sample decks): ADPRES_REFERENCE, else a
# checkout named "reference" beside this repository; tests that need it
# skip where neither exists (the GPU machines have no copy).
REFERENCE = os.environ.get("ADPRES_REFERENCE") or os.path.join(os.path.dirname(ROOT), "reference")
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built extension")


def reference_deck(name):
    """Path of a sample deck of the reference project, or skip when absent."""
    p = os.path.join(REFERENCE, "smpl", "static", name)
    if not os.path.exists(p):
        pytest.skip("reference sample decks are not mounted here")
    return p
