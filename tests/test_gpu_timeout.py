"""The tensor-core kernel's bounded waits, made to run out on purpose.

Every wait in tc_gemm_kernel has a budget; when one runs out the kernel
raises its abort flag, lets the matrix products already issued finish (under
the fixed default budget), frees its tensor memory and sets the operator's
error flag.  Here the budget is cut to one cycle, so the first wait that is
not satisfied at once gives up: the apply must report TBEM_ERR_TIMEOUT, keep
reporting it, and leave the device usable for other work.  Nothing faults:
the waits end by themselves and return a status.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TIMEOUT = -5


def _sphere_op(precision="mixed"):
    from tbempy import ThreeD, meshes
    locs, nrm, w = meshes.sphere_points(3)  # 3,840 points
    op = ThreeD.FMMOperator(ThreeD.LaplaceSingle(), locs, nrm, locs, nrm, w,
                            ThreeD.FMMConfig(0.3, 152, 50, 0.05, False), precision=precision)
    return op, locs, nrm, w


def test_tensor_core_wait_budget_exhausted_reports_timeout_and_device_stays_usable():
    torch = pytest.importorskip("torch")
    from tbempy import ThreeD
    from tbempy._lib import TbemError
    op, locs, nrm, w = _sphere_op()
    assert op.tc_tile() > 0, "the operator must run its M2L on the tensor cores"
    x = np.random.default_rng(0).uniform(-1, 1, op.n_cols())
    y_ok = op.apply(x)  # the default budget: a normal apply
    op.set_wait_cycles(1)
    with pytest.raises(TbemError) as e:
        op.apply(x)  # host output: the timeout is reported by this call
    assert e.value.code == TIMEOUT
    op.set_wait_cycles(0)
    with pytest.raises(TbemError) as e:
        op.apply(x)  # the failure is latched
    assert e.value.code == TIMEOUT
    with pytest.raises(TbemError) as e:
        op.sync()
    assert e.value.code == TIMEOUT

    # device output: the apply itself is asynchronous and returns; sync()
    # reports the timeout before the caller uses the result
    op2, *_ = _sphere_op()
    op2.set_wait_cycles(1)
    xd = torch.tensor(x, device="cuda")
    op2.apply(xd)
    with pytest.raises(TbemError) as e:
        op2.sync()
    assert e.value.code == TIMEOUT

    # the device is still usable: a fresh operator and plain torch work run
    op3, *_ = _sphere_op()
    y3 = op3.apply(x)
    assert np.linalg.norm(y3 - y_ok) <= 1e-6 * np.linalg.norm(y_ok)
    op3.sync()
    t = torch.arange(1000, device="cuda", dtype=torch.float64)
    assert float(t.sum().item()) == 499500.0
    exact = ThreeD.DirectOperator(ThreeD.LaplaceSingle(), locs, nrm, locs, nrm, w).apply(x)
    assert np.linalg.norm(y3 - exact) <= 1e-5 * np.linalg.norm(exact)
