"""div_by (cmtj_gb300/csrc/recip.cuh), the FP64 plain form's division by a
per-run constant (Ms, Ms*t, 6), against the IEEE quotient a / b on the GPU,
bit for bit: random dividends over the whole exponent range, +-0,
subnormals, quotients at and next to powers of two and at the edges of the
normal range, and the divisors the physics uses."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _lib(tmp_path_factory):
    from cmtj_gb300 import build as B
    out = tmp_path_factory.mktemp("divcheck") / "libdivcheck.so"
    subprocess.check_call([B._nvcc(), *B.ARCH, "-O3", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC", "-shared",
                           "-I", os.path.join(ROOT, "cmtj_gb300", "csrc"), os.path.join(HERE, "div_by_check.cu"),
                           "-o", str(out)])
    lib = ctypes.CDLL(str(out))
    P = ctypes.c_void_p
    lib.run_div_check.argtypes = [P, P, ctypes.c_int, P, P]
    lib.run_div_check.restype = ctypes.c_int
    return lib


def _cases(rng):
    with np.errstate(over="ignore"):
        return _cases_raw(rng)


def _cases_raw(rng):
    divisors = np.array([1.0, 1.2, 1.5, 6.0, 0.8, 1.6, 1.2 * 1.5e-9, 1.5 * 2e-9, 1.0 * 1.2e-9, 3.0, 7.0, 1e-300,
                         1e300, 2.0 ** -1000, np.nextafter(1.0, 2.0), np.nextafter(2.0, 1.0)])
    divisors = np.concatenate([divisors, rng.uniform(0.05, 5.0, 200), np.exp(rng.uniform(-600, 600, 200))])
    a_list, b_list = [], []
    for b in divisors:
        m = 4000
        x = np.concatenate([
            rng.standard_normal(m) * np.exp(rng.uniform(-50, 50, m)),           # typical fields and moments
            np.exp(rng.uniform(-700, 700, m // 4)) * rng.choice([-1, 1], m // 4),  # the exponent range
            np.ldexp(1.0, rng.integers(-1070, 1020, m // 8)) * b,                 # quotients at powers of two
        ])
        k = np.ldexp(1.0, rng.integers(-900, 900, m // 8))
        near = np.concatenate([np.nextafter(k * b, np.inf), np.nextafter(k * b, -np.inf)])  # next to them
        edge = np.array([0.0, -0.0, 5e-324, -5e-324, 2.2250738585072014e-308, 1.7976931348623157e308,
                         1e-310, b, -b, 2 * b, b / 3])
        a = np.concatenate([x, near, edge])
        a = a[np.isfinite(a)]
        a_list.append(a)
        b_list.append(np.full(a.shape, b))
    return np.concatenate(a_list), np.concatenate(b_list)


@pytest.mark.gpu
def test_div_by_equals_ieee_quotient(gpu_lib, tmp_path_factory):
    lib = _lib(tmp_path_factory)
    rng = np.random.default_rng(20261204)
    a, b = _cases(rng)
    a, b = np.ascontiguousarray(a), np.ascontiguousarray(b)
    n = a.size
    assert n > 2_000_000
    fast = np.zeros(n, dtype=np.uint64)
    ieee = np.zeros(n, dtype=np.uint64)
    rc = lib.run_div_check(a.ctypes.data, b.ctypes.data, n, fast.ctypes.data, ieee.ctypes.data)
    assert rc == 0
    bad = np.flatnonzero(fast != ieee)
    assert bad.size == 0, [(float(a[i]), float(b[i]), hex(int(fast[i])), hex(int(ieee[i]))) for i in bad[:5]]
