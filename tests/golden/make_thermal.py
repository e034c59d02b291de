"""Reference switching statistics for the stochastic (sLLGS) parity test.

The reference draws its thermal field from an unseeded std::mt19937
(junction.hpp:174-175), so thermal runs can only be compared in statistics.
This script runs the reference extension (oracle/_ref, built from the
reference sources) on the p-bit case of tests/thermal_cases.py: n runs per
current density, Euler-Heun, T = 300 K, and records how many ended with
m_z < 0.  Output: tests/golden/pbit_switching.npz.

With --alpha it runs the p-bit layer with buffered 1/f^alpha noise
(thermal_cases.ALPHA_CASES, 2 ns each, the reference's BufferedAlphaNoise,
whose FFT comes from the stand-in header under oracle/stubs/) and writes
tests/golden/alpha_switching.npz.

With --sweep it runs the p-bit sweep at its full parameters instead
(thermal_cases.pbit_sweep_junction: Ku 2.5e5 J/m^3, 17 of the sweep's 64
current densities over [0, 5e11] A/m^2, each run's duration drawn from
U[5, 20] ns) and writes tests/golden/pbit_sweep.npz.

    CMTJ_REF=<reference checkout> python tests/golden/make_thermal.py [--sweep | --alpha] [runs]
"""
import multiprocessing as mp
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "tests"))
sys.path.insert(0, ROOT)


def _worker(args):
    ref_path, j_density, n = args
    sys.path.insert(0, ref_path)
    import cmtj
    import thermal_cases
    switched = 0
    for _ in range(n):
        junc, run = thermal_cases.pbit_junction(cmtj, j_density)
        junc.runSimulation(**run)
        if junc.getLayerMagnetisation("free").z < 0:
            switched += 1
    return switched


def _sweep_worker(args):
    ref_path, j_density, n, seed = args
    sys.path.insert(0, ref_path)
    import cmtj
    import thermal_cases
    switched = 0
    for d in thermal_cases.sweep_durations(n, seed):
        junc, run = thermal_cases.pbit_sweep_junction(cmtj, j_density, d)
        junc.runSimulation(**run)
        if junc.getLayerMagnetisation("free").z < 0:
            switched += 1
    return switched


def main_sweep(argv):
    from oracle.build import build_reference
    import thermal_cases
    ref = build_reference()
    if ref is None:
        raise SystemExit("reference sources not available (set CMTJ_REF)")
    n = int(argv[0]) if argv else 1024
    currents = thermal_cases.SWEEP_CURRENTS
    chunks = 16
    tasks = [(ref, float(j), n // chunks, 7000 + 100 * q + c)
             for q, j in enumerate(currents) for c in range(chunks)]
    with mp.get_context("spawn").Pool(os.cpu_count()) as pool:
        res = pool.map(_sweep_worker, tasks, chunksize=1)
    counts = np.array(res).reshape(len(currents), chunks).sum(axis=1)
    runs = (n // chunks) * chunks
    np.savez_compressed(os.path.join(HERE, "pbit_sweep.npz"), currents=np.asarray(currents),
                        switched=counts, runs=np.full(len(currents), runs),
                        t_min=thermal_cases.SWEEP_T_MIN, t_max=thermal_cases.SWEEP_T_MAX,
                        Ku=thermal_cases.SWEEP_KU)
    for j, c in zip(currents, counts):
        print("j=%.3g  P=%.3f" % (j, c / runs))


def _alpha_worker(args):
    ref_path, case, n = args
    sys.path.insert(0, ref_path)
    import cmtj
    import thermal_cases
    switched = 0
    for _ in range(n):
        junc, run = thermal_cases.alpha_pbit_junction(cmtj, *case)
        junc.runSimulation(**run)
        if junc.getLayerMagnetisation("free").z < 0:
            switched += 1
    return switched


def main_alpha(argv):
    from oracle.build import build_reference
    import thermal_cases
    ref = build_reference()
    if ref is None:
        raise SystemExit("reference sources not available (set CMTJ_REF)")
    n = int(argv[0]) if argv else 1024
    cases = thermal_cases.ALPHA_CASES
    chunks = 16
    tasks = [(ref, case, n // chunks) for case in cases for _ in range(chunks)]
    with mp.get_context("spawn").Pool(os.cpu_count()) as pool:
        res = pool.map(_alpha_worker, tasks, chunksize=1)
    counts = np.array(res).reshape(len(cases), chunks).sum(axis=1)
    runs = (n // chunks) * chunks
    np.savez_compressed(os.path.join(HERE, "alpha_switching.npz"), cases=np.asarray(cases, dtype=np.float64),
                        switched=counts, runs=np.full(len(cases), runs))
    for c, k in zip(cases, counts):
        print(c, "P=%.3f" % (k / runs))


def main(argv):
    if argv and argv[0] == "--sweep":
        return main_sweep(argv[1:])
    if argv and argv[0] == "--alpha":
        return main_alpha(argv[1:])
    from oracle.build import build_reference
    import thermal_cases
    ref = build_reference()
    if ref is None:
        raise SystemExit("reference sources not available (set CMTJ_REF)")
    n = int(argv[0]) if argv else 512
    currents = thermal_cases.PBIT_CURRENTS
    chunks = 8
    tasks = [(ref, float(j), n // chunks) for j in currents for _ in range(chunks)]
    with mp.get_context("spawn").Pool(os.cpu_count()) as pool:
        res = pool.map(_worker, tasks)
    counts = np.array(res).reshape(len(currents), chunks).sum(axis=1)
    np.savez_compressed(os.path.join(HERE, "pbit_switching.npz"), currents=np.asarray(currents),
                        switched=counts, runs=np.full(len(currents), (n // chunks) * chunks))
    for j, c in zip(currents, counts):
        print("j=%.3g  P=%.3f" % (j, c / ((n // chunks) * chunks)))


if __name__ == "__main__":
    main(sys.argv[1:])
