"""FP64 plain GPU form against the reference's own logs.

Tolerances (deterministic, T = 0): max|dm| <= 1e-9 on every logged
magnetisation component, relative 1e-9 on resistances and on the other
logged fields, time stamps identical (Dormand-Prince: relative 1e-9)."""
import numpy as np
import pytest

import cases
import cmtj_gb300
from test_oracle_pin import load_golden

TOL_M = 1e-9
TOL_REL = 1e-9


def _check(name, log, golden):
    assert set(log) == set(golden), set(log) ^ set(golden)
    for k, g in golden.items():
        a = log[k]
        assert a.shape == g.shape, (k, a.shape, g.shape)
        if k == "time" and not name.startswith("dp_"):
            assert np.array_equal(a, g)
        elif k == "time":
            # Dormand-Prince times are sums of adaptive steps whose factor
            # comes from pow(), which may differ from glibc's by an ulp
            assert np.max(np.abs(a - g)) <= TOL_REL * np.max(np.abs(g)), (name, k)
        elif k.endswith(("_mx", "_my", "_mz")):
            assert np.max(np.abs(a - g)) <= TOL_M, (name, k, np.max(np.abs(a - g)))
        else:
            scale = max(np.max(np.abs(g)), 1e-300)
            assert np.max(np.abs(a - g)) <= TOL_REL * scale, (name, k, np.max(np.abs(a - g)) / scale)


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(cases.DETERMINISTIC))
def test_fp64_plain_matches_reference(gpu_lib, name):
    golden, gmags = load_golden(name)
    _, log, mags = cases.run_case(cmtj_gb300, name)
    _check(name, log, golden)
    for lid, gm in gmags.items():
        assert np.max(np.abs(np.asarray(mags[lid]) - gm)) <= TOL_M


@pytest.mark.gpu
def test_fp64_plain_batch_equals_single(gpu_lib):
    """A junction gives the same log alone and inside a batch of others."""
    from cmtj_gb300 import engine
    js = [cases.mtj_rh_point(cmtj_gb300, hx=h, total=2e-10)[0] for h in (-5e5, -1e5, 2e5, 6e5)]
    solo = cases.mtj_rh_point(cmtj_gb300, hx=2e5, total=2e-10)[0]
    plan = engine.plan_run(2e-10, 1e-13, 1e-12)
    engine.run_junctions(js, plan, cmtj_gb300.SolverMode.RK4)
    engine.run_junctions([solo], plan, cmtj_gb300.SolverMode.RK4)
    a, b = js[2].getLog(), solo.getLog()
    for k in b:
        assert a[k] == b[k], k
