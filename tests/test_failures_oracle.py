"""The reference's behaviour on the failure cases of tests/failure_cases.py,
through the oracle (CPU): the two-node LU's pivot STOP and the divergence
STOP (mod_nodal.f90:851-872, :131-142) become error codes; a zero flux and
fission source, or a NaN cross section, make the reference produce k = NaN
without stopping (bicg has no breakdown guard, mod_cmfd.f90:1203-1243, and
check_xs's comparisons are false for NaN, mod_xsec.f90:90-168) -- the C ABI
turns those into ADP_ERR_BREAKDOWN and ADP_ERR_NAN."""
import numpy as np
import pytest

import oracle
from failure_cases import DN_BIG, TEXT, nan_siga, tiny_adf


def test_oracle_pivot_stop():
    o = oracle.Oracle(text=TEXT)
    o.xs_updt()
    nn, ng = o.geti("nnod"), o.geti("ng")
    o.set_array("dc", tiny_adf(o.fortran("dc", (nn, ng, 6)), o.array("mat")).reshape(-1, order="F"))
    with pytest.raises(oracle.OracleError) as e:
        o.outer(popt=1)
    assert e.value.code == oracle.ORA_ERR_PIVOT


def test_oracle_divergence_stop():
    o = oracle.Oracle(text=TEXT)
    o.run()
    o.seti("nupd", 1)
    o.set_array("dn", np.full(o.geti("nnod") * o.geti("ng") * 6, DN_BIG))
    with pytest.raises(oracle.OracleError) as e:
        o.outer(popt=1)
    assert e.value.code == oracle.ORA_ERR_DIVERGED


def test_oracle_zero_start_and_nan_give_nan_k():
    o = oracle.Oracle(text=TEXT)
    o.run()
    nn, ng = o.geti("nnod"), o.geti("ng")
    o.set_array("f0", np.zeros(nn * ng))
    o.set_array("fs0", np.zeros(nn))
    o.outer(popt=1)
    assert np.isnan(o.getd("Ke"))
    o = oracle.Oracle(text=TEXT)
    o.xs_updt()
    o.set_array("siga", nan_siga(o.fortran("siga", (nn, ng))).reshape(-1, order="F"))
    o.dsigr_updt()
    o.outer(popt=1)
    assert np.isnan(o.getd("Ke"))
