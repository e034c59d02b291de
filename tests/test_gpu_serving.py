"""Continuous batching (cmtj_gb300.serving): requests of mixed kinds
(2-layer RK4, 1-layer thermal Euler-Heun, uneven 1-4-layer spin-diode with
on-device <I R>) arrive while others run; each request's results are the
same alone and in the mix, at any tick length (the FP32 form's tolerance
is 1e-4; the bits agree)."""
import numpy as np
import pytest

from cmtj_gb300 import serving


def _trace():
    return serving.make_trace(8, rate_hz=400.0, seed=11, min_solves=64, max_solves=512, t_min=2e-10, t_max=8e-10)


@pytest.mark.gpu
def test_serving_results_same_alone_and_in_mix(gpu_lib):
    mix = _trace()
    eng = serving.ServingEngine(hbm_budget_bytes=256 << 20, chunk_steps=500)
    done = eng.run(mix)
    assert all(r.done_at is not None for r in done)
    assert all(np.all(r.state["status"] == 0) for r in done)
    for k in (0, 3, 6):
        alone = _trace()[k]
        alone.arrival = 0.0
        e2 = serving.ServingEngine(hbm_budget_bytes=64 << 20, chunk_steps=700)  # other tick length
        e2.run([alone])
        a, b = done[k].state, alone.state
        assert np.array_equal(a["step"], b["step"])
        assert float(np.max(np.abs(a["m"] - b["m"]))) <= 1e-4
        assert np.array_equal(a["m"], b["m"]), k
        if done[k].red_every:
            assert np.array_equal(a["r_sum"], b["r_sum"]) and np.array_equal(a["v_sum"], b["v_sum"])


@pytest.mark.gpu
def test_serving_admission_waits_for_hbm_budget(gpu_lib):
    """A pool smaller than the sum of the requests: later requests wait for
    slots and still complete."""
    reqs = serving.make_trace(6, rate_hz=1e6, seed=5, min_solves=200, max_solves=300, t_min=2e-10, t_max=3e-10)
    per = serving.SlotPool.BYTES_PER_SLOT
    eng = serving.ServingEngine(hbm_budget_bytes=per * 700, chunk_steps=1000)
    assert eng.pool.capacity < sum(r.spec.n for r in reqs)
    done = eng.run(reqs)
    assert all(r.done_at is not None for r in done)
    assert eng.pool.free == [(0, eng.pool.capacity)]


@pytest.mark.gpu
def test_serving_policy_changes_order_not_results(gpu_lib):
    """Shortest-job-first and FIFO admission give the same bits per request."""
    states = []
    for policy in ("fifo", "sjf"):
        eng = serving.ServingEngine(hbm_budget_bytes=64 << 20, chunk_steps=500, policy=policy)
        done = eng.run(_trace())
        states.append({r.tag + str(r.arrival): r.state for r in done})
    assert states[0].keys() == states[1].keys()
    for k in states[0]:
        assert np.array_equal(states[0][k]["m"], states[1][k]["m"]), k


@pytest.mark.gpu
def test_serving_fp64_requests_same_alone_and_in_mix(gpu_lib):
    """FP64 plain requests run on their own stream beside the FP32 ticks;
    each one's junctions end in the same bits as the same junctions run
    alone through engine.run_junctions."""
    from cmtj_gb300 import engine

    def trace():
        return serving.make_trace(6, rate_hz=400.0, seed=21, min_solves=64, max_solves=256, t_min=2e-10,
                                  t_max=4e-10, f64_fraction=0.5)

    mix = trace()
    assert {r.precision for r in mix} == {"f32", "f64"}
    done = serving.ServingEngine(hbm_budget_bytes=64 << 20, chunk_steps=500).run(mix)
    assert all(r.done_at is not None for r in done)
    checked = 0
    for a, b in zip(sorted(done, key=lambda r: r.arrival), trace()):
        if a.precision != "f64":
            continue
        plan = engine.plan_run(b.total_time, b.time_step, b.total_time)
        engine.run_junctions(b.junctions, plan, b.solver)
        for x, y in zip(a.junctions, b.junctions):
            for lx, ly in zip(x.layers, y.layers):
                assert (lx.mag.x, lx.mag.y, lx.mag.z) == (ly.mag.x, ly.mag.y, ly.mag.z)
        checked += 1
    assert checked >= 1
