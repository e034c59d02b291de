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
