"""cmtj_batch_run_f32_noalloc: the allocation-free form of the FP32 batched
solver, for callers that cannot call cudaMalloc (a stream being captured
into a CUDA graph, real-time threads, hosts that give a plugin a fixed
memory arena).  It keeps its work-stealing ticket in a static device array
inside the library instead of a caller buffer.

The test calls it through the C ABI, twice in a row on the same buffers,
and checks both results against cmtj_batch_run_f32's within the FP32 form's
tolerance (max|dm| <= 1e-4; the same kernel runs, so the bits agree too).
This file is collected last so that a run stopping at the first failure has
run every other test before it."""
import ctypes

import numpy as np
import pytest

import cases
import cmtj_gb300
from cmtj_gb300 import _abi, batch, engine

TOL_M_F32 = 1e-4


def _mixed_batch():
    js = []
    for k in range(40):
        name = ["mtj_rh_point", "sto", "tri_layer", "vsd_sine", "sot_strip"][k % 5]
        js.append(cases.DETERMINISTIC[name](cmtj_gb300)[0])
    spec = batch.BatchSpec.from_junctions(js)
    low = batch.lower(spec, 1e-13, 2000)
    return low


def _run_noalloc(run, lib, slot):
    p = run.params
    p["chunk_steps"] = 2 ** 32 - 1
    for nl, d_order, cnt, code in run.parts:
        p["log_tile"] = batch.default_tile(batch.log_channels(run.log_mode, nl))
        rc = lib.cmtj_batch_run_f32_noalloc(engine.ptr(run.d_j), engine.ptr(run.d_l), engine.ptr(run.d_s),
                                            engine.ptr(d_order), cnt, nl, code, p.ctypes.data,
                                            engine.ptr(run.d_log), slot, 0, engine.stream_ptr())
        _abi.check(rc, lib)


@pytest.mark.gpu
def test_noalloc_matches_allocating_entry_point(gpu_lib):
    torch = engine.torch()
    lib = _abi.load()
    run = batch.BatchRun(_mixed_batch(), 1e-13, cmtj_gb300.SolverMode.RK4, batch.LOG_M, 10)
    zero_state = torch.zeros_like(run.d_s)

    run.d_s.copy_(zero_state)
    run.launch()
    ref_state = run.state().copy()
    ref_log = run.d_log.cpu().numpy().copy()
    assert np.all(ref_state["status"] == 0) and np.all(ref_state["step"] == 2000)

    for call in range(2):  # two calls in a row on the same slot: the second re-zeroes the used ticket
        run.d_s.copy_(zero_state)
        run.d_log.zero_()
        _run_noalloc(run, lib, slot=3)
        torch.cuda.synchronize()
        st = run.state()
        log = run.d_log.cpu().numpy()
        assert np.all(st["status"] == 0) and np.all(st["step"] == 2000), call
        assert np.all(st["n_logged"] == ref_state["n_logged"]), call
        assert float(np.max(np.abs(st["m"] - ref_state["m"]))) <= TOL_M_F32, call
        assert float(np.max(np.abs(log - ref_log))) <= TOL_M_F32, call


@pytest.mark.gpu
def test_noalloc_rejects_slot_beyond_static_array(gpu_lib):
    lib = _abi.load()
    p = np.zeros(1, dtype=batch.F32_PARAMS_DTYPE)
    p["solver"] = int(cmtj_gb300.SolverMode.RK4)
    dummy = ctypes.c_void_p(1)
    rc = lib.cmtj_batch_run_f32_noalloc(dummy, dummy, dummy, dummy, 1, 1, 0, p.ctypes.data, None, 64, 0, None)
    assert rc == _abi.CMTJ_ERR_LIMIT
    assert "outside [0, 64)" in _abi.last_error(lib)


@pytest.mark.gpu
def test_noalloc_launch_replays_from_a_cuda_graph(gpu_lib):
    """Captured into a CUDA graph (no allocation may happen while a stream
    is being captured) and replayed twice: each replay gives the direct
    launch's bits."""
    torch = engine.torch()
    lib = _abi.load()
    run = batch.BatchRun(_mixed_batch(), 1e-13, cmtj_gb300.SolverMode.RK4, batch.LOG_M, 10)
    zero_state = torch.zeros_like(run.d_s)
    run.d_s.copy_(zero_state)
    _run_noalloc(run, lib, slot=5)  # direct launch; also resolves the static ticket's address
    torch.cuda.synchronize()
    want_state = run.state().copy()
    want_log = run.d_log.cpu().numpy().copy()
    graph = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream()
    with torch.cuda.stream(side):
        with torch.cuda.graph(graph, stream=side):
            run.d_s.copy_(zero_state)
            _run_noalloc(run, lib, slot=5)
    for _ in range(2):
        run.d_log.zero_()
        graph.replay()
        torch.cuda.synchronize()
        st = run.state()
        assert np.all(st["status"] == 0) and np.all(st["step"] == 2000)
        assert np.array_equal(st["m"], want_state["m"])
        assert np.array_equal(run.d_log.cpu().numpy(), want_log)
