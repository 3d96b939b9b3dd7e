"""Host logic of the Newton driver that needs no GPU: the adaptive increment generator reproduces the
increments the reference tried in every Newton fixture, given the reference's iteration counts."""

import numpy as np
import pytest

import newton_cases as nc


@pytest.mark.parametrize("name", nc.names())
def test_adaptive_stepper_replays_reference_increments(name):
    case = nc.load(name)
    stepper, _, _, _, ctl = nc.step_inputs(case)
    rec = case["increments"]
    errs = case["increment_errors"]
    gen = stepper.generateTimeStep()
    for k in range(len(rec)):
        ts = next(gen)
        assert ts.number == int(rec[k, 0])
        assert np.isclose(ts.stepProgressIncrement, rec[k, 1], rtol=0, atol=1e-15)
        assert np.isclose(ts.stepProgress, rec[k, 2], rtol=0, atol=1e-15)
        assert np.isclose(ts.totalTime, rec[k, 5], rtol=1e-15, atol=1e-15)
        if errs[k]:
            stepper.discardAndChangeIncrement(ctl["cutbackFactor"])
        elif int(rec[k, 6]) >= ctl["criticalIter"]:
            stepper.preventIncrementIncrease()
    with pytest.raises(StopIteration):
        next(gen)


def test_dirichlet_and_loads_follow_the_step_amplitude():
    from edelweissfe_gb300.solver import Dirichlet, NodeForces, TimeStep

    ts = TimeStep(3, 0.25, 0.75, 0.25, 0.75, 0.75)
    d = Dirichlet([1, 4], [0.01, -0.02])
    assert np.allclose(d.getDelta(ts), [0.0025, -0.005])
    f = NodeForces([2], [100.0])
    assert np.allclose(f.getCurrentLoad(ts), [75.0])
