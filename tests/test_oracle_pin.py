"""The oracle (oracle/cmtj_oracle.cpp) against the reference's own outputs.

tests/golden/<case>.npz holds logs produced by the reference extension built
from its sources (tests/golden/make_golden.py).  The oracle must reproduce
every logged value bit for bit: it restates the reference's arithmetic in
the same order with no FMA contraction, and runs on the same libm."""
import numpy as np
import pytest

import cases
import oracle_harness


def load_golden(name):
    g = np.load("%s/golden/%s.npz" % (cases.__file__.rsplit("/", 1)[0], name))
    log = {k[5:]: g[k] for k in g.files if k.startswith("log__")}
    mags = {k[5:]: g[k] for k in g.files if k.startswith("mag__")}
    return log, mags


@pytest.mark.parametrize("name", sorted(cases.DETERMINISTIC))
def test_oracle_matches_reference_bitwise(name):
    golden, gmags = load_golden(name)
    _, log, mags = cases.run_case(oracle_harness.oracle_module(), name)
    assert set(log) == set(golden), set(log) ^ set(golden)
    for k in golden:
        assert log[k].shape == golden[k].shape, k
        # identical bits, not merely close
        assert np.array_equal(log[k], golden[k]), (k, np.max(np.abs(log[k] - golden[k])))
    for lid in gmags:
        assert np.array_equal(np.asarray(mags[lid]), gmags[lid]), lid


def test_log_length_law():
    """len(time) = ceil(T/dt / writeEvery) (tests/test_layer.cpp:42-47 in
    the reference asserts T/dt rows at writeEvery 1)."""
    j, _ = cases.mtj_rh_point(oracle_harness.oracle_module())
    j.runSimulation(1e-10, 1e-13, 1e-13)
    assert len(j.getLog()["time"]) == int(1e-10 / 1e-13)
    assert j.getLog()["time"][:3] == [0.0, 1e-13, 2e-13]
