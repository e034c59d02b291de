"""The run-time launch tuner on the GPU: its trials leave the batch
untouched, and every choice it can make (log tile, resident-CTA bound,
FP64 lanes per layer) gives the same bits as the fixed defaults."""
import ctypes

import numpy as np
import pytest

import cmtj_gb300 as cm
from cmtj_gb300 import _abi, autotune, batch, engine, sweeps

DT = 1e-13


@pytest.fixture
def fresh_table(tmp_path, monkeypatch):
    monkeypatch.setattr(autotune, "PATH", str(tmp_path / "autotune.json"))
    monkeypatch.setattr(autotune, "_table", None)
    monkeypatch.setenv("CMTJ_AUTOTUNE", "1")


def _pimm(n=4096, steps=3000):
    spec, _ = sweeps.pimm_config(n_h=64, n_draw=n // 64, dt=DT, total=steps * DT)
    return batch.lower(spec, DT, steps)


@pytest.mark.gpu
def test_tuned_fp32_batch_equals_defaults(gpu_lib, fresh_table, monkeypatch):
    """A logged PIMM batch and an uneven spin-diode batch with weighted
    reductions: tuned (trials first) and untuned runs give identical
    states and logs."""
    cases = [(_pimm(), cm.SolverMode.RK4, dict(log_mode=batch.LOG_MIX, log_every=10)),
             (None, cm.SolverMode.RK4, dict(red_every=1))]
    spec, n_steps = sweeps.vsd_config(n_f=8, n_h=64, dt=DT, t_min=2e-10, t_max=4e-10)
    cases[1] = (batch.lower(spec, DT, n_steps), cm.SolverMode.RK4,
                dict(red_every=1, red_weights=batch.lowpass_step_response(int(n_steps.max()), 1 / DT)))
    for low, solver, kw in cases:
        monkeypatch.setenv("CMTJ_AUTOTUNE", "1")
        tuned = batch.BatchRun(low, DT, solver, **kw)
        tuned.launch()
        assert any(t is not None for t in tuned.tuning)
        monkeypatch.setenv("CMTJ_AUTOTUNE", "0")
        plain = batch.BatchRun(low, DT, solver, **kw)
        plain.launch()
        a, b = tuned.state(), plain.state()
        assert np.all(a["status"] == 0)
        assert a.tobytes() == b.tobytes()
        assert np.array_equal(tuned.d_log.cpu().numpy(), plain.d_log.cpu().numpy())


@pytest.mark.gpu
@pytest.mark.parametrize("solver,layers", [("RK4", 2), ("EulerHeun", 1), ("RK4", 4)])
def test_every_bound_and_tile_gives_the_same_bits(gpu_lib, solver, layers):
    """Each compiled resident-CTA bound of a variant, and log tiles of 4
    and 16, run the same junctions to the same bits: final states and
    every logged sample (the padding after a row's last sample is not a
    result)."""
    mode = getattr(cm.SolverMode, solver)
    if layers == 1:
        spec, ns, _ = sweeps.pbit_config(n_j=4, n_per=256, dt=DT, t_min=1e-10, t_max=2e-10)
    elif layers == 2:
        spec, ns = sweeps.pimm_config(n_h=32, n_draw=16, dt=DT, total=1600 * DT)
        ns = np.full(spec.n, 1600)
    else:
        spec, ns = sweeps.vsd_config(n_f=4, n_h=128, dt=DT, t_min=1e-10, t_max=2e-10)
        keep = np.nonzero(spec.n_layers == 4)[0]
        spec, ns = spec.take(keep), ns[keep]
        # the rows of one kernel variant (one partition)
        first = batch.BatchRun(batch.lower(spec, DT, ns), DT, mode)
        rows = first.part_rows[0]
        spec, ns = spec.take(rows), ns[rows]
    low = batch.lower(spec, DT, ns)
    lib = _abi.load()
    log_mode = batch.LOG_M if layers < 4 else batch.LOG_MIX
    probe = batch.BatchRun(low, DT, mode, log_mode, 20)
    assert len(probe.parts) == 1
    nl, _, _, code = probe.parts[0]
    arr = (ctypes.c_int32 * 4)()
    assert lib.cmtj_batch_bounds_f32(nl, int(mode), code & 0xffffff, ctypes.cast(arr, ctypes.c_void_p), 4) == 2
    results = []
    for bound in (arr[0], arr[1]):
        for tile in (4, 16):
            run = batch.BatchRun(low, DT, mode, log_mode, 20)
            run._launch_part(0, None, engine.torch().cuda.current_stream(), tile, (code & 0xffffff) | (bound << 24))
            st = run.state()
            assert np.all(st["status"] == 0)
            log = run.d_log.cpu().numpy()
            samples = np.concatenate([run.log_of(k, log).ravel() for k in range(run.n)])
            results.append((st.tobytes(), samples.tobytes(), bound, tile))
    same_state = len({r[0] for r in results}) == 1
    same_log = len({r[1] for r in results}) == 1
    assert same_state and same_log, (same_state, same_log, [r[2:] for r in results])


@pytest.mark.gpu
def test_tuned_fp64_lanes_equal_defaults(gpu_lib, fresh_table, monkeypatch):
    """The FP64 plain form on 4096 R(H) MTJs for 3000 steps: with the lane
    layout the tuner picks and with the library's pick, the same bits."""
    from cmtj_gb300 import tune
    out = []
    for flag in ("1", "0"):
        monkeypatch.setenv("CMTJ_AUTOTUNE", flag)
        js = tune.rh_junctions(4096, 3000 * DT)
        engine.run_junctions(js, engine.plan_run(3000 * DT, DT, 100 * DT), cm.SolverMode.RK4)
        out.append(np.array([[l.mag.x, l.mag.y, l.mag.z] for j in js for l in j.layers]))
    assert autotune.lookup(autotune.f64_key(2, 1, 4096)) is not None
    assert np.array_equal(out[0], out[1])
