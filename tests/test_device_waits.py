"""Failure detection of the MIC sweeps' bounded device waits, and the per-stage
device times of a step.

The sweeps of FLUID_3D_MIC::applyMICPreconditioner (FLUID_3D_MIC.cpp:864-899)
run here as persistent wavefront kernels whose CTAs wait on one another; every
such wait is bounded, and an expired wait must come back to the host as
PLUME_ERR_TIMEOUT with the handle still usable.  The test makes a wait expire
without faulting anything: plume_set_wait_gate makes each sweep CTA first
poll a device flag that nothing sets, before it issues any copy, so the wait
runs out, the kernel records it and returns with nothing in flight.
"""
import os

import numpy as np
import pytest

from cfs_plume_gb300 import _abi
from cfs_plume_gb300.plume import Plume, PlumeError

pytestmark = pytest.mark.gpu

WEIGHTS = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "cfs_plume_gb300",
                       "weights", "unet_warmstart.bin")


def _rhs(n, seed=5):
    return np.random.default_rng(seed).standard_normal(n)


@pytest.mark.parametrize("precision", [_abi.PREC_FP64, _abi.PREC_FP32])
def test_expired_sweep_wait_reports_timeout_and_handle_recovers(precision):
    # open top and bottom: the Poisson matrix is non-singular for any b
    if precision == _abi.PREC_FP64:
        p = _abi.default_params(res=(24, 32, 24))
    else:
        p = _abi.default_params(res=(24, 32, 24), precision=_abi.PREC_FP32, criterion=_abi.CRIT_REL2,
                                tol=1e-6)
    h = Plume(p)
    b = _rhs(h.N)
    x_ref, st_ref = h.solve_poisson(b)  # (FP32: builds the CG-loop graph)
    assert st_ref.converged == 1
    h.set_wait_gate(True, 1000)
    with pytest.raises(PlumeError) as e:
        h.solve_poisson(b)
    assert e.value.status == _abi.ERR_TIMEOUT
    assert "wait expired" in str(e.value)
    h.set_wait_gate(False)
    x, st = h.solve_poisson(b)
    # the same kernels in the same order: the solve after the expired one
    # gives the first solve's result bit for bit
    assert st.iterations == st_ref.iterations
    np.testing.assert_array_equal(x, x_ref)
    # and so does a fresh handle
    x_new, _ = Plume(p).solve_poisson(b)
    np.testing.assert_array_equal(x, x_new)
    h.close()


def test_gate_poll_limit_must_be_positive():
    h = Plume(_abi.default_params(res=(16, 20, 12)))
    with pytest.raises(PlumeError) as e:
        h.set_wait_gate(True, 0)
    assert e.value.status == _abi.ERR_INVALID
    h.close()


@pytest.mark.parametrize("learned", [False, True])
def test_stage_times_add_up_to_the_step(learned):
    """plume_step_stats' per-stage device times (the reference's TIMER
    buckets, src/util/TIMER.cpp:33-149, measured with CUDA events) cover the
    step: they and ms_solve add up to ms_total."""
    kw = dict(warm_start=_abi.WARM_LEARNED) if learned else {}
    p = _abi.plume_config((48, 64, 48), **kw)
    h = Plume(p)
    if learned:
        from cfs_plume_gb300.net import PlumeNet
        net = PlumeNet(path=WEIGHTS)
        net.attach(h)
    for s in range(3):
        h.add_source(s)
        st = h.step()
        stages = [getattr(st, "ms_" + k) for k in _abi.STAGES]
        assert all(v >= 0.0 for v in stages), stages
        assert st.ms_solve > 0 and st.ms_advection > 0 and st.ms_vorticity > 0
        assert sum(stages) == pytest.approx(st.ms_total, abs=0.02), (stages, st.ms_total)
        if learned:
            assert st.ms_guess > 0
        else:
            assert st.ms_guess < 0.01
    h.close()
