"""PIMM and spin-diode procedures (cmtj_gb300.procedures) against the
reference's own procedures (cmtj/utils/procedures.py:42-331), whose outputs
on the cases of procedure_cases.py are in tests/golden/procedures.npz
(tests/golden/make_procedures.py).

On CPU the FP64 runs go through the oracle (bit-identical to the
reference), so every output must match bit for bit, the seeded disturbance
included.  On the GPU: the FP64 plain form within 1e-9 (relative to each
output's scale), the FP32 form within its accuracy bound, and a list of
junctions advanced together equal to each junction run alone."""
import os

import numpy as np
import pytest

import cmtj_gb300 as cm
import oracle_harness
import procedure_cases as pc
from cmtj_gb300 import procedures

GOLDEN = np.load(os.path.join(os.path.dirname(__file__), "golden", "procedures.npz"))


def _run(name, precision="f64", module=cm):
    j, kw = pc.CASES[name](module, procedures.ResistanceParameters)
    kind = kw.pop("kind")
    np.random.seed(pc.SEED)
    if kind == "pimm":
        spec, freqs, out = procedures.PIMM_procedure(j, precision=precision, **kw)
        return {"spectrum": np.asarray(spec), "freqs": np.asarray(freqs), "Rx": np.asarray(out["Rx"]),
                "Ry": np.asarray(out["Ry"]), "m_avg": np.asarray(out["m_avg"])}
    return {"vsd": np.asarray(procedures.VSD_procedure(j, precision=precision, **kw))}


def _oracle_f64(junctions, duration, int_step):
    oracle_harness.run_oracle(junctions, duration, int_step, int_step)


@pytest.mark.parametrize("name", sorted(pc.CASES))
def test_procedure_matches_reference_bitwise_on_oracle(name, monkeypatch):
    monkeypatch.setattr(procedures, "_run_f64", _oracle_f64)
    got = _run(name)
    for k, v in got.items():
        g = GOLDEN[name + "__" + k]
        assert v.shape == g.shape, (name, k, v.shape, g.shape)
        assert np.array_equal(v, g), (name, k, np.max(np.abs(v - g)))


def test_procedure_helpers():
    Hspan, H = procedures.FieldScan.amplitude_scan(-1.0, 1.0, 3, 90, 0)
    assert np.allclose(H[:, 0], [-1, 0, 1]) and np.allclose(H[:, 1:], 0)
    Hs, Hb = procedures.FieldScan.amplitude_scan(-1.0, 1.0, 3, 90, 0, back=True)
    assert len(Hs) == 5 and np.allclose(Hb[:, 0], [-1, 0, 1, 0, -1])
    m = np.zeros((2, 3, 4))
    m[:, 0] = 1.0
    rs = procedures.calculate_resistance_series([1, 2], [1, 1], [0.5, 0.5], [0, 0], [0, 0], m, [1, 1], [1, 1])[0]
    rp = procedures.calculate_resistance_parallel([1, 2], [1, 1], [0.5, 0.5], [0, 0], [0, 0], m, [1, 1], [1, 1])[0]
    assert np.allclose(rs, 4.0) and np.allclose(rp, 1.0 / (1 / 1.5 + 1 / 2.5))
    with pytest.raises(ValueError):
        j, kw = pc.pimm_bilayer(cm, procedures.ResistanceParameters)
        kw.pop("kind")
        kw["resistance_params"] = kw["resistance_params"][:1]
        procedures.PIMM_procedure(j, **kw)


def _scale(g):
    return max(float(np.max(np.abs(g))), 1e-30)


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(pc.CASES))
def test_procedure_fp64_gpu_matches_reference(gpu_lib, name):
    """The FP64 plain form keeps max|dm| <= 1e-9 against the reference, so:
    spectra of N samples within 1e-9 N, resistances within 1e-9 of their
    scale, and the spin-diode voltage (a mean of I R that cancels down to
    ~1e-5 ohm) within 1e-9 x the magnetoresistance scale (100 ohm)."""
    got = _run(name, "f64")
    for k, v in got.items():
        g = GOLDEN[name + "__" + k]
        assert v.shape == g.shape
        if k == "freqs":
            tol = 0.0
        elif k == "spectrum":
            tol = 1e-9 * 2000
        elif k == "vsd":
            tol = 1e-9 * 100.0
        elif k == "m_avg":
            tol = 1e-9
        else:
            tol = 1e-9 * _scale(g)
        assert np.max(np.abs(v - g)) <= tol, (name, k, np.max(np.abs(v - g)))


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["pimm_bilayer_saturated", "vsd_bilayer", "vsd_bilayer_rx"])
def test_procedure_fp32_gpu_within_bound(gpu_lib, name):
    """The FP32 form: m within 1e-4 of FP64 per sample, so the spectrum of
    N samples within 1e-4 N, resistances within 1e-4 of their
    magnetoresistance scale, and the spin-diode voltage within 1e-4 x the MR
    scale (it is a mean of I R).  Only well-conditioned chains qualify: the
    pimm_bilayer chain (from +z through H = 0) turns a 1e-7 nudge of m0 into
    4e-5 of m_avg in FP64 itself, so FP32 rounding lands near 1e-4 there."""
    got = _run(name, "f32")
    for k, v in got.items():
        g = GOLDEN[name + "__" + k]
        assert v.shape == g.shape
        if k == "freqs":
            assert np.array_equal(v, g)
        elif k == "spectrum":
            n = 2000
            assert np.max(np.abs(v - g)) <= 1e-4 * n
        elif k in ("Rx", "Ry"):
            assert np.max(np.abs(v - g)) <= 1e-4 * 2 * (0.24 + 0.46 + 0.3) * 10
        elif k == "m_avg":
            assert np.max(np.abs(v - g)) <= 1e-4
        else:
            assert np.max(np.abs(v - g)) <= 1e-4 * 100.0, (name, k, v, g)


@pytest.mark.gpu
def test_procedure_chains_together_equal_alone(gpu_lib):
    outs = []
    for mode in ("together", "alone"):
        js, kws = [], []
        for hx in (0.0, 5e4):
            j, kw = pc.pimm_bilayer(cm, procedures.ResistanceParameters)
            j.setLayerMagnetisation("free", cm.CVector(0.1, 0.0, 1.0) if hx else cm.CVector(0, 0, 1))
            kw.pop("kind")
            js.append(j)
            kws.append(kw)
        if mode == "together":
            outs.append(procedures.PIMM_procedure(js, **kws[0]))
        else:
            outs.append([procedures.PIMM_procedure(j, **kw) for j, kw in zip(js, kws)])
    for (sa, fa, oa), (sb, fb, ob) in zip(*outs):
        assert np.array_equal(sa, sb) and np.array_equal(fa, fb)
        assert np.array_equal(np.asarray(oa["Rx"]), np.asarray(ob["Rx"]))
