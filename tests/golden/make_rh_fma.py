"""How far the reference's own last bits move the R(H) sweep when it is
compiled with FMA contraction.

The reference's setup.py passes no -ffp-contract flag, so GCC contracts
a*b + c into FMAs wherever the target has them (aarch64, or x86-64 with
-mfma); the x86-64 baseline build has no FMA.  Both are the reference.
This script runs the R(H) sweep of the FP64 plain form in full (the 2-layer
MTJ of tune.rh_junctions: 64 fields over +-800 kA/m, 10 ns at dt = 1e-13,
every step logged) on both builds of oracle/_ref (oracle/build_ref.sh) and
records, per field, the largest |dm| over both layers' logged m and the
largest relative difference of R between them.

Output: tests/golden/rh_fma_spread.npz (fields, max_abs_dm, max_rel_dR).

    CMTJ_REF=<reference checkout> bash oracle/build_ref.sh
    python tests/golden/make_rh_fma.py
"""
import multiprocessing as mp
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
PLAIN = os.path.join(ROOT, "oracle", "_ref")
FMA = os.path.join(ROOT, "oracle", "_ref", "fma")
FIELDS = np.linspace(-800e3, 800e3, 64)
KEYS = ("free_mx", "free_my", "free_mz", "ref_mx", "ref_my", "ref_mz", "R_free_ref")


def _run(ref_path, h):
    """m and R logs of one field point on the build at ref_path."""
    sys.path.insert(0, ref_path)
    import cmtj
    assert os.path.dirname(cmtj._cmtj.__file__) == ref_path, cmtj._cmtj.__file__
    V = cmtj.CVector
    demag = [V(0.0024, 0, 0), V(0, 0.0024, 0), V(0, 0, 0.9952)]
    free = cmtj.Layer("free", mag=V(0, 0, 1), anis=V(0, 0, 1), Ms=1.2, thickness=1.5e-9, cellSurface=1e-16,
                      demagTensor=demag, damping=0.01)
    ref = cmtj.Layer("ref", mag=V(0, 0, 1), anis=V(0, 0, 1), Ms=1.5, thickness=2e-9, cellSurface=1e-16,
                     demagTensor=demag, damping=0.01)
    j = cmtj.Junction([free, ref], 100, 200)
    j.setLayerAnisotropyDriver("free", cmtj.constantDriver(3e5))
    j.setLayerAnisotropyDriver("ref", cmtj.constantDriver(1e6))
    j.setIECDriver("free", "ref", cmtj.constantDriver(-5e-5))
    j.setLayerExternalFieldDriver("all", cmtj.AxialDriver(float(h), 0, 0))
    j.runSimulation(1e-8, 1e-13, 1e-13)
    log = j.getLog()
    return np.stack([np.asarray(log[k], dtype=np.float64) for k in KEYS], 1)


def _plain(args):
    k, tmp = args
    np.save(os.path.join(tmp, "%d.npy" % k), _run(PLAIN, FIELDS[k]))
    return k


def _compare(args):
    k, tmp = args
    a = np.load(os.path.join(tmp, "%d.npy" % k))
    b = _run(FMA, FIELDS[k])
    assert a.shape == b.shape, (a.shape, b.shape)
    dm = float(np.max(np.abs(b[:, :6] - a[:, :6])))
    dr = float(np.max(np.abs(b[:, 6] - a[:, 6]) / np.abs(a[:, 6])))
    return k, dm, dr


def main():
    for d in (PLAIN, FMA):
        if not any(f.startswith("_cmtj") for f in os.listdir(d) if os.path.isdir(d)):
            raise SystemExit("build oracle/_ref first (CMTJ_REF=... bash oracle/build_ref.sh)")
    ctx = mp.get_context("spawn")
    dm = np.zeros(len(FIELDS))
    dr = np.zeros(len(FIELDS))
    # one pool per build: a worker keeps the first `cmtj` it imported
    with tempfile.TemporaryDirectory() as tmp:
        with ctx.Pool(os.cpu_count() or 1) as pool:
            list(pool.imap_unordered(_plain, [(k, tmp) for k in range(len(FIELDS))]))
        with ctx.Pool(os.cpu_count() or 1) as pool:
            for k, a, b in pool.imap_unordered(_compare, [(k, tmp) for k in range(len(FIELDS))]):
                dm[k], dr[k] = a, b
    out = os.path.join(HERE, "rh_fma_spread.npz")
    np.savez(out, fields=FIELDS, max_abs_dm=dm, max_rel_dR=dr)
    print("wrote", out)
    for k in np.argsort(-dm)[:8]:
        print("field %2d  H = %9.0f A/m  max|dm| %.3g  max rel dR %.3g" % (k, FIELDS[k], dm[k], dr[k]))


if __name__ == "__main__":
    main()
