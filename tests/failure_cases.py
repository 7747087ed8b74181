"""Inputs that drive the path into each STOP of the reference (or into the
NaN it produces silently), shared by the oracle's CPU test and the GPU
tests.  Every case is made on the host: cross sections, ADFs or a state
set through the public API; none needs a fault on the GPU."""
from __future__ import annotations

import numpy as np

from adpres_gb300 import synth

TEXT = synth.small_core(seed=2, ng=2, kern="SANM", adf=True, bc=(0, 0, 0, 0, 0, 0))
TINY_ADF_MAT = 2         # material whose ADFs are set to 1e-6
TINY_ADF = 1e-6
DN_BIG = 2.0e3           # coupling coefficients that the next nodal update moves by more than 1e3
NAN_NODE, NAN_GROUP = 3, 1


def tiny_adf(dc, mat):
    """dc (nnod, ng, 6) with every ADF of one material at 1e-6: the no-pivot
    LU of the two-node problems meets an input diagonal below 1e-4
    (LU_solve, mod_nodal.f90:851-872)."""
    dc = np.array(dc, dtype=np.float64, copy=True)
    dc[np.asarray(mat) == TINY_ADF_MAT] = TINY_ADF
    return dc


def nan_siga(siga):
    a = np.array(siga, dtype=np.float64, copy=True)
    a[NAN_NODE, NAN_GROUP] = np.nan
    return a
