"""Batched launches replayed through CUDA graphs (BatchRun.graph): a
replay gives the direct launch's bits, for one partition and for several
forked onto their own streams, and replays of a chunked launch resume the
state exactly as chunked direct launches do."""
import numpy as np
import pytest

import cmtj_gb300 as cm
from cmtj_gb300 import batch, engine, sweeps

DT = 1e-13


def _uneven():
    spec, n_steps = sweeps.vsd_config(n_f=4, n_h=64, dt=DT, t_min=1e-10, t_max=3e-10)
    return batch.lower(spec, DT, n_steps)


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["pimm", "uneven"])
def test_graph_replay_equals_direct_launch(gpu_lib, kind):
    t = engine.torch()
    if kind == "pimm":
        spec, _ = sweeps.pimm_config(n_h=32, n_draw=32, dt=DT, total=2000 * DT)
        low, kw = batch.lower(spec, DT, 2000), dict(log_mode=batch.LOG_MIX, log_every=10)
    else:
        low, kw = _uneven(), dict(red_every=1)
    direct = batch.BatchRun(low, DT, cm.SolverMode.RK4, **kw)
    direct.launch()
    want_s, want_log = direct.state().copy(), direct.d_log.cpu().numpy().copy()
    run = batch.BatchRun(low, DT, cm.SolverMode.RK4, **kw)
    if kind == "uneven":
        assert len(run.parts) > 1
    zero = t.zeros_like(run.d_s)
    g = run.graph()
    for _ in range(2):
        run.d_s.copy_(zero)
        run.d_log.zero_()
        g.replay()
        t.cuda.synchronize()
        assert run.state().tobytes() == want_s.tobytes()
        assert np.array_equal(run.d_log.cpu().numpy(), want_log)


@pytest.mark.gpu
def test_graph_replays_resume_chunks(gpu_lib):
    """Replaying a 500-step chunk graph until every junction is done gives
    the bits of one full launch."""
    t = engine.torch()
    low = _uneven()
    full = batch.BatchRun(low, DT, cm.SolverMode.RK4, red_every=1)
    full.launch()
    run = batch.BatchRun(low, DT, cm.SolverMode.RK4, red_every=1)
    g = run.graph(chunk_steps=500)
    t.cuda.synchronize()
    run.d_s.zero_()
    for _ in range(int(np.ceil(low.n_steps.max() / 500))):
        g.replay()
    t.cuda.synchronize()
    assert np.all(run.state()["step"] == low.n_steps)
    assert run.state().tobytes() == full.state().tobytes()
