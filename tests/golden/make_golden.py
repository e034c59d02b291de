"""Generate the golden fixtures in tests/golden/ from the reference itself.

Runs every case of tests/cases.py with the reference's `_cmtj` extension
(built from the reference sources by oracle/build_ref.sh into oracle/_ref/)
and stores the full-precision logs and final magnetisations as
<case>.npz.  Needs the reference sources, so it runs in the development
container only; the fixtures are committed and travel with the tests.

    CMTJ_REF=<reference checkout> python tests/golden/make_golden.py [case ...]
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "tests"))
sys.path.insert(0, ROOT)


def reference_module():
    from oracle.build import build_reference
    ref = build_reference()
    if ref is None:
        raise SystemExit("reference sources not available (set CMTJ_REF); cannot regenerate fixtures")
    sys.path.insert(0, ref)
    import cmtj  # the shim package of oracle/_ref
    import cmtj.stack  # noqa: F401
    return cmtj


def save_case(cm, name):
    import cases
    _, log, mags = cases.run_case(cm, name)
    out = {"log__" + k: v for k, v in log.items()}
    for lid, m in mags.items():
        out["mag__" + lid] = np.asarray(m, dtype=np.float64)
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **out)
    return path, sum(v.size for v in log.values())


def save_stack_case(cm, name):
    import cases
    slog, jlogs = cases.run_stack_case(cm, name)
    out = {"stack__" + k: v for k, v in slog.items()}
    for q, lg in enumerate(jlogs):
        out.update({"j%d__%s" % (q, k): v for k, v in lg.items()})
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **out)
    return path, sum(v.size for v in out.values())


def main(argv):
    import cases
    cm = reference_module()
    names = argv or (list(cases.DETERMINISTIC) + list(cases.STACKS))
    for name in names:
        if name in cases.STACKS:
            path, n = save_stack_case(cm, name)
        else:
            path, n = save_case(cm, name)
        print("%-28s %8d values  %7.1f KB" % (name, n, os.path.getsize(path) / 1024))


if __name__ == "__main__":
    main(sys.argv[1:])
