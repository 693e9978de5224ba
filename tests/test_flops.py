"""The analytic FP64 work model (pfgpu/flops.py, the numerator of the bench's
roofline) against the reference algorithm's arithmetic counted op by op:
the oracle's RStep compiled with a counting scalar (oracle/flop_real.hpp,
oracle/oracle_count.cpp) on the parity cells.  The model may understate the
counted work by a few per cent (it leaves out per-cell-solve overheads such
as the final RTAuxVarCompute and the kinetic-state update) but must never
overstate it, so the reported roofline fraction is conservative."""
import numpy as np
import pytest

import cases
from pfgpu import flops


@pytest.mark.parametrize("name,lo", [("random12", 0.97), ("calcite", 0.93)])
def test_flop_model_matches_counted_reference(oracle, name, lo):
    net, st = cases.case(oracle, name)
    st = st.subset(np.arange(300))
    fl, tr, its = oracle.count_rstep(net, st, cases.CASE_DT[name])
    f_it, t_it = flops.per_iteration(net)
    ratio = f_it * its.sum() / fl.sum()
    assert lo <= ratio <= 1.0, ratio
    tratio = t_it * its.sum() / tr.sum()
    assert 0.85 <= tratio <= 1.0, tratio


def test_counting_build_gives_the_oracle_results(oracle):
    """Counting does not change the arithmetic: the counted RStep leaves the
    same state as the plain oracle."""
    net, st = cases.case(oracle, "random12")
    st = st.subset(np.arange(64))
    a, b = st.copy(), st.copy()
    oracle.rstep(net, a, cases.CASE_DT["random12"])
    oracle.count_rstep(net, b, cases.CASE_DT["random12"])
    for k in ("pri_molal", "total", "sec_molal", "mnrl_rate", "mnrl_volfrac"):
        np.testing.assert_array_equal(a.a[k], b.a[k], err_msg=k)
