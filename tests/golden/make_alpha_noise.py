"""Reference buffers of the buffered 1/f^alpha noise.

Runs the reference's own BufferedAlphaNoise::fillBuffer (core/noise.hpp,
through oracle/_ref/libalpha_ref.so, built from the reference sources by
oracle/build_ref.sh) on seeded cases and records each case's white draws
and coloured buffer.  The map from white draws to buffer is deterministic,
so the restatements (the oracle and cmtj_alpha_noise_f32, given the same
white draws) must reproduce the buffers to float rounding.
Output: tests/golden/alpha_noise.npz.

    CMTJ_REF=<reference checkout> python tests/golden/make_alpha_noise.py
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

# (buffer length, alpha, standard deviation, mt19937 seed)
CASES = [(1, 1.0, 1.0, 11), (2, 0.5, 1.0, 12), (7, 1.5, 1.0, 13),
         (1000, 0.0, 1.0, 21), (1000, 0.5, 1.0, 22), (1000, 1.0, 1.0, 23), (1000, 1.5, 1.0, 24),
         (1000, 2.0, 1.0, 25), (1537, 0.3, 0.25, 31), (1537, 1.0, 0.25, 32), (1537, 1.9, 0.25, 33)]


def main():
    from oracle.build import build_reference
    ref = build_reference()
    if ref is None:
        raise SystemExit("reference sources not available (set CMTJ_REF)")
    lib = ctypes.CDLL(os.path.join(ref, "libalpha_ref.so"))
    lib.alpha_ref_fill.restype = ctypes.c_int
    lib.alpha_ref_fill.argtypes = [ctypes.c_uint32, ctypes.c_double, ctypes.c_double, ctypes.c_uint32,
                                   ctypes.c_void_p, ctypes.c_void_p]
    out = {"cases": np.array([c[:3] for c in CASES], dtype=np.float64)}
    for k, (n, alpha, std, seed) in enumerate(CASES):
        white = np.zeros(n, dtype=np.float32)
        buf = np.zeros(n, dtype=np.float32)
        rc = lib.alpha_ref_fill(n, alpha, std, seed, white.ctypes.data, buf.ctypes.data)
        assert rc == 0
        out["white_%d" % k] = white
        out["out_%d" % k] = buf
        print("n=%d alpha=%.2f std=%.2f: buffer std %.4g" % (n, alpha, std, float(np.std(buf))))
    np.savez_compressed(os.path.join(HERE, "alpha_noise.npz"), **out)


if __name__ == "__main__":
    main()
