"""The C-ABI library loads (no GPU needed) and exports every symbol that
include/*.h declares, with struct layouts matching the Python mirror."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if not fn.endswith(".h"):
            continue
        src = open(os.path.join(ROOT, "include", fn)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\*?\s*(cmtj_[A-Za-z0-9_]+)\s*\(", src, re.M):
            names.add(m.group(1))
    return names


@pytest.fixture(scope="module")
def lib():
    from cmtj_gb300 import _abi, build
    build.build()
    return _abi.load()


def test_library_exports_header_symbols(lib):
    names = declared_functions()
    assert "cmtj_run_simulation_f64" in names
    for n in sorted(names):
        assert hasattr(lib, n), n


def test_python_prototypes_cover_header(lib):
    from cmtj_gb300 import _abi
    assert declared_functions() <= set(_abi.PROTOTYPES), declared_functions() - set(_abi.PROTOTYPES)


def test_struct_layout_and_version(lib):
    from cmtj_gb300 import _abi
    _abi.check_layout(lib)
    assert lib.cmtj_log_width(2, 0) == _abi.log_width(2, False) == 10
    assert lib.cmtj_log_width(3, 1) == 3 * 29 + 4


def test_feature_constants_mirror_header():
    """The Python mirrors of the header's FP32 feature flags."""
    src = open(os.path.join(ROOT, "include", "cmtj_gpu.h")).read()
    defs = {k: int(v, 0) for k, v in re.findall(r"#define (CMTJ_\w+)\s+(0x[0-9a-fA-F]+|\d+)", src)}
    from cmtj_gb300 import batch
    for name in ("FULL_DEMAG", "DIPOLE", "IDMI", "K2", "STT", "SOT", "WAVES", "SCALAR_WAVES", "IEC2", "OFFAXIS",
                 "ALL"):
        assert defs["CMTJ_FEAT_" + name] == getattr(batch, "FEAT_" + name), name


def test_f32_batch_rejects_chunk_inside_a_log_tile(lib):
    """A chunk that ends inside a log tile would leave the next chunk's bulk
    log stores off a 16-byte boundary: the entry point refuses it before it
    touches the device (no GPU needed)."""
    import ctypes
    import numpy as np
    from cmtj_gb300 import _abi, batch
    p = np.zeros(1, dtype=batch.F32_PARAMS_DTYPE)
    p["solver"] = 0  # RK4
    p["log_mode"] = batch.LOG_M
    p["log_every"] = 10
    p["log_tile"] = 4
    dummy = ctypes.c_void_p(16)
    for chunk in (41, 60, 4):  # none a multiple of 10 * 4 steps
        p["chunk_steps"] = chunk
        rc = lib.cmtj_batch_run_f32(dummy, dummy, dummy, dummy, 1, 1, 0, p.ctypes.data, dummy, dummy, 0, None)
        assert rc == _abi.CMTJ_ERR_ARG, chunk
        assert "not a multiple of log_every * log_tile = 40" in _abi.last_error(lib)


def test_f64_rejects_unknown_arithmetic(lib):
    """cmtj_sim_params_t.arithmetic outside enum cmtj_arithmetic is refused
    before any device work (no GPU needed), and the Python lowering refuses
    an unknown name."""
    import ctypes
    import numpy as np
    import pytest
    from cmtj_gb300 import _abi, _lower
    p = np.zeros(1, dtype=_abi.SIM_PARAMS_DTYPE)
    p["solver"] = 0  # RK4
    p["write_every"] = 1
    p["arithmetic"] = 7
    dummy = ctypes.c_void_p(16)
    rc = lib.cmtj_run_simulation_f64(dummy, 1, dummy, None, p.ctypes.data, dummy, dummy, None)
    assert rc == _abi.CMTJ_ERR_ARG
    assert "unknown arithmetic 7" in _abi.last_error(lib)
    plan = _lower.plan_run(1e-12, 1e-13, 1e-13)
    with pytest.raises(ValueError, match="arithmetic"):
        _lower.make_params(plan, 0, False, 10, 2, "fast")
    assert int(_lower.make_params(plan, 0, False, 10, 2, "fused")["arithmetic"][0]) == _abi.ARITH_FUSED


def test_empty_inputs_return_ok_before_touching_buffers(lib):
    """Zero junctions, stacks, groups, rows or buffers: each entry point
    checks its arguments and returns CMTJ_OK before it reads a pointer (no
    GPU needed)."""
    import numpy as np
    from cmtj_gb300 import _abi, batch
    p = np.zeros(1, dtype=_abi.SIM_PARAMS_DTYPE)
    p["solver"] = 1  # RK4
    p["write_every"] = 1
    P = p.ctypes.data
    assert lib.cmtj_run_simulation_f64(None, 0, None, None, P, None, None, None) == _abi.CMTJ_OK
    assert lib.cmtj_run_stack_f64(None, 0, None, None, None, None, None, P, None, None, 5, 2, None, None) == \
        _abi.CMTJ_OK
    assert lib.cmtj_run_group_f64(None, 0, None, None, None, None, None, P, None, 1, None, None) == _abi.CMTJ_OK
    fp = np.zeros(1, dtype=batch.F32_PARAMS_DTYPE)
    assert lib.cmtj_batch_run_f32(None, None, None, None, 0, 2, 0, fp.ctypes.data, None, None, 0, None) == \
        _abi.CMTJ_OK
    assert lib.cmtj_spectrum_f32(None, 4096, 0, 4096, 4096, 1, 100, None, None) == _abi.CMTJ_OK
    assert lib.cmtj_alpha_noise_f32(None, 0, 1000, None, None, None, 0, None) == _abi.CMTJ_OK
    # limits: an FFT above 8192 points and a layer count above the FP32 form's
    assert lib.cmtj_spectrum_f32(None, 16384, 1, 16384, 16384, 1, 100, None, None) == _abi.CMTJ_ERR_ARG
    assert lib.cmtj_batch_run_f32(None, None, None, None, 1, 5, 0, fp.ctypes.data, None, None, 0, None) == \
        _abi.CMTJ_ERR_ARG
