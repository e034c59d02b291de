"""cmtj.utils helpers around the time loop (cmtj/utils/linear.py,
filters.py, parallel.py): FieldScan's constructors, the Butterworth
filters and distribute."""
import numpy as np
from scipy.signal import butter, lfilter

from cmtj_gb300.utils import Filters, FieldScan
from cmtj_gb300.utils.linear import FieldScan as LinearFieldScan
from cmtj_gb300.utils.parallel import distribute


def test_fieldscan_constructors():
    assert LinearFieldScan is FieldScan
    span, H = FieldScan.theta_scan(0, 90, 4, 1e5, 30)
    th = np.deg2rad(span)
    ph = np.deg2rad(30)
    assert np.allclose(H, np.stack([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)], 1) * 1e5)
    span, H = FieldScan.phi_scan(0, 180, 5, 2e5, 60)
    ph = np.deg2rad(span)
    th = np.deg2rad(60)
    assert np.allclose(H, np.stack([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph),
                                    np.cos(th) * np.ones_like(ph)], 1) * 2e5)
    theta, phi, r = FieldScan.vector2angle(1.0, 1.0, np.sqrt(2.0))
    assert np.isclose(theta, 45.0) and np.isclose(phi, 45.0) and np.isclose(r, 2.0)
    v = FieldScan.angle2vector(30, 40, 3.0)
    back = FieldScan.cvector2angle(v)
    assert np.allclose(back, (30, 40, 3.0))


def test_filters_are_scipy_butterworth():
    x = np.random.default_rng(0).normal(size=2000)
    fs = 1e12
    b, a = butter(5, 1e10 / (0.5 * fs), btype="low", analog=False)
    assert np.array_equal(Filters.butter_lowpass_filter(x, 1e10, fs), lfilter(b, a, x))
    b, a = butter(5, [0.1, 0.3], btype="bandpass", analog=False)
    assert np.array_equal(Filters.butter_bandpass_filter(x, (0.1, 0.3), fs), lfilter(b, a, x))
    b, a = butter(5, [0.9 * 2e11 / (0.5 * fs), 2e11 / (0.5 * fs)], btype="bandpass", analog=False)
    assert np.array_equal(Filters.butter_bandpass_filter(x, 2e11, fs), lfilter(b, a, x))
    arr = np.arange(12.0).reshape(3, 4)
    assert np.array_equal(Filters.detrend_axis(arr, 0), arr - np.median(arr, axis=0))
    assert np.array_equal(Filters.detrend_axis(arr, 1), (arr.T - np.median(arr, axis=1)).T)


def test_distribute_yields_every_combination_with_its_indices():
    spaces = [[1.0, 2.0, 3.0], [10.0, 20.0]]
    got = list(distribute(lambda a, b: a * b, spaces, n_cores=3, shuffle=True))
    assert len(got) == 6
    for idx, out in got:
        assert out == spaces[0][idx[0]] * spaces[1][idx[1]]
    assert sorted(tuple(i) for i, _ in got) == [(i, j) for i in range(3) for j in range(2)]
