"""Dormand-Prince (SolverMode.DormandPrince, junction.hpp:866-1002 and
1982-2045).  The bit-for-bit pins against the reference's own logs are the
dp_* cases of test_oracle_pin.py (oracle) and test_gpu_fp64_parity.py (FP64
plain GPU form).  Here: the behaviour around them."""
import pytest

import cases
import cmtj_gb300 as cm
import oracle_harness


def _bilayer(mod, total):
    j, runs = cases.mtj_rh_point(mod, total=total)
    r = dict(runs[0])
    r["solverMode"] = mod.SolverMode.DormandPrince
    return j, r


def test_multilayer_rejection_stops_with_error():
    """With several layers a rejected step makes the reference use hopt = -1
    as the step and never finish; the GPU solver (and the oracle) stop with
    an error instead."""
    j, r = _bilayer(oracle_harness.oracle_module(), 1e-10)
    with pytest.raises(RuntimeError, match="hopt"):
        j.runSimulation(**r)


def test_adaptive_log_stays_within_capacity():
    from cmtj_gb300.engine import plan_run
    p = plan_run(2e-9, 1e-13, 1e-12, solver=cm.SolverMode.DormandPrince)
    assert p.adaptive and p.n_log == 2002
    j, runs = cases.DETERMINISTIC["dp_vsd_sine"](oracle_harness.oracle_module())
    for rr in runs:
        j.runSimulation(**rr)
    t = j.getLog()["time"]
    assert 0 < len(t) <= p.n_log
    assert all(b > a for a, b in zip(t, t[1:]))


def test_custom_driver_rejected():
    j, runs = cases.DETERMINISTIC["custom_driver"](oracle_harness.oracle_module())
    r = dict(runs[0])
    r["solverMode"] = cm.SolverMode.DormandPrince
    with pytest.raises(RuntimeError, match="Dormand"):
        j.runSimulation(**r)


def _pid_params():
    # The default gains (kp = +0.2) scale the step by ratio^0.2, which shrinks
    # it as the error falls and never ends; a negative kp is the working sign.
    p = cm.AdaptiveIntegrationParams()
    p.use_pid_control = True
    p.kp, p.ki, p.kd = -0.2, -0.01, 0.0
    return p


def test_pid_default_gains_hit_the_attempt_limit():
    j, runs = cases.sto(oracle_harness.oracle_module(), total=2e-10)
    p = cm.AdaptiveIntegrationParams()
    p.use_pid_control = True
    j.layers[0].setAdaptiveParams(p)
    r = dict(runs[0])
    r["solverMode"] = cm.SolverMode.DormandPrince
    with pytest.raises(RuntimeError, match="step attempts"):
        j.runSimulation(**r)


def test_pid_state_persists_across_runs():
    """The PID controller's state lives on the layer (junction.hpp:955-961)
    and carries over to the next runSimulation call."""
    j, runs = cases.sto(oracle_harness.oracle_module(), total=2e-10)
    j.layers[0].setAdaptiveParams(_pid_params())
    r = dict(runs[0])
    r["solverMode"] = cm.SolverMode.DormandPrince
    j.runSimulation(**r)
    ap = j.layers[0].adaptiveParams
    assert ap.integral_error != 0.0 and ap.prev_error_ratio != 1.0


@pytest.mark.gpu
def test_gpu_multilayer_rejection_stops_with_error(gpu_lib):
    j, r = _bilayer(cm, 1e-10)
    with pytest.raises(RuntimeError, match="hopt"):
        j.runSimulation(**r)


@pytest.mark.gpu
def test_gpu_pid_matches_oracle(gpu_lib):
    """PID step control (not reachable from the reference's Python API, whose
    binding has no setAdaptiveParams): GPU against the oracle."""
    import numpy as np
    logs = []
    for mod in (cm, oracle_harness.oracle_module()):
        j, runs = cases.sto(mod, total=5e-10)
        j.layers[0].setAdaptiveParams(_pid_params())
        r = dict(runs[0])
        r["solverMode"] = cm.SolverMode.DormandPrince
        j.runSimulation(**r)
        logs.append({k: np.asarray(v) for k, v in j.getLog().items()})
    a, b = logs
    assert a["time"].shape == b["time"].shape
    for k in b:
        assert np.max(np.abs(a[k] - b[k])) <= 1e-9 * max(1.0, np.max(np.abs(b[k]))), k
