"""SeriesStack / ParallelStack on the GPU against the reference's own stack
and junction logs (tests/golden/stack_*.npz): KCL and non-KCL, delayed and
non-delayed coupling, 1- and 2-layer STT junctions, constant / sine / step
coupled currents.  Tolerances as for the FP64 plain form: max|dm| <= 1e-9,
relative 1e-9 on resistance, currents and couplings."""
import numpy as np
import pytest

import cases
import cmtj_gb300


def _load(name):
    g = np.load("%s/golden/%s.npz" % (cases.__file__.rsplit("/", 1)[0], name))
    stack = {k[7:]: g[k] for k in g.files if k.startswith("stack__")}
    js = {}
    for k in g.files:
        if k.startswith("j"):
            q, key = k.split("__", 1)
            js.setdefault(int(q[1:]), {})[key] = g[k]
    return stack, [js[q] for q in sorted(js)]


def _close(a, b, key):
    assert a.shape == b.shape, (key, a.shape, b.shape)
    if key == "time":
        assert np.array_equal(a, b)
    elif key.endswith(("_mx", "_my", "_mz")):
        assert np.max(np.abs(a - b)) <= 1e-9, (key, np.max(np.abs(a - b)))
    else:
        scale = max(np.max(np.abs(b)), 1e-300)
        assert np.max(np.abs(a - b)) <= 1e-9 * scale, (key, np.max(np.abs(a - b)) / scale)


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(cases.STACKS))
def test_stack_matches_reference(gpu_lib, name):
    gs, gj = _load(name)
    slog, jlogs = cases.run_stack_case(cmtj_gb300, name)
    assert set(slog) == set(gs)
    for k in gs:
        _close(slog[k], gs[k], k)
    assert len(jlogs) == len(gj)
    for a, b in zip(jlogs, gj):
        assert set(a) == set(b)
        for k in b:
            _close(a[k], b[k], k)


def _force_params(monkeypatch, **fields):
    """Lower with the given cmtj_sim_params_t fields overridden."""
    from cmtj_gb300 import _lower
    orig = _lower.make_params

    def make_params(*a, **k):
        p = orig(*a, **k)
        for f, v in fields.items():
            p[f] = v
        return p

    monkeypatch.setattr(_lower, "make_params", make_params)


@pytest.mark.gpu
@pytest.mark.parametrize("lanes", [1, 4])
@pytest.mark.parametrize("name", sorted(cases.STACKS))
def test_stack_both_layouts_match_reference(gpu_lib, monkeypatch, name, lanes):
    """The stack kernel with a layer per lane and with a layer's x, y, z on
    a quad of lanes, against the reference's logs."""
    _force_params(monkeypatch, lanes_per_layer=lanes)
    gs, gj = _load(name)
    slog, jlogs = cases.run_stack_case(cmtj_gb300, name)
    for k in gs:
        _close(slog[k], gs[k], k)
    for a, b in zip(jlogs, gj):
        for k in b:
            _close(a[k], b[k], k)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["kcl", "delayed", "nondelayed", "kcl_thermal"])
def test_wide_stack_thread_per_junction_equals_lanes(gpu_lib, monkeypatch, mode):
    """40 bilayer junctions in one stack.  Told that a junction may hold 8
    layers, the stack no longer fits a CTA of lanes and runs one thread per
    junction (k_stack_f64); otherwise its layers run on lanes
    (k_stack_lanes).  Both give the same bits in every log."""
    def build():
        js = [cases._stt_bilayer(cmtj_gb300, 1.0 + 0.01 * k, 1e3 + 40 * k, (0.1 + 0.005 * k, 0.2, 1))
              for k in range(40)]
        if mode == "kcl_thermal":
            for q, j in enumerate(js):
                j.setLayerTemperatureDriver("all", cmtj_gb300.constantDriver(300.0))
                for l, layer in enumerate(j.layers):
                    layer.noise_seed = 9000 + 10 * q + l
        s = cmtj_gb300.stack.SeriesStack(js, useKCL=mode.startswith("kcl"), phaseOffset=0.1)
        if mode == "nondelayed":
            s.setDelayed(False)
        s.setCouplingStrength(0.05)
        s.setCoupledCurrentDriver(cmtj_gb300.sineDriver(1e10, 4e10, 3e9, 0))
        s.runSimulation(5e-11, 1e-13, 1e-12)
        return s

    on_lanes = build()
    _force_params(monkeypatch, max_layers=8, lanes_per_layer=1)
    per_thread = build()
    a, b = on_lanes.getLog(), per_thread.getLog()
    assert a.keys() == b.keys()
    for k in a:
        assert np.array_equal(np.asarray(a[k]), np.asarray(b[k])), k
    for q in range(40):
        la, lb = on_lanes.getLog(q), per_thread.getLog(q)
        for k in la:
            assert np.array_equal(np.asarray(la[k]), np.asarray(lb[k])), (q, k)
