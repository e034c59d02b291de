"""Reference logs of the GroupInteraction cases in tests/group_cases.py,
run with the reference extension built from its sources (oracle/_ref).
Output: tests/golden/groups.npz (key "<case>__<junction>__<log key>").

    CMTJ_REF=<reference checkout> python tests/golden/make_groups.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "tests"))
sys.path.insert(0, ROOT)


def main():
    from make_golden import reference_module
    cm = reference_module()
    import cmtj.reservoir  # noqa: F401
    import group_cases
    out = {}
    for name in group_cases.CASES:
        logs = group_cases.run_case(cm, name)
        for k, lg in logs.items():
            for key, v in lg.items():
                out["%s__%d__%s" % (name, k, key)] = v
        print(name, len(logs), "junctions", {k: len(v["time"]) for k, v in logs.items()})
    np.savez_compressed(os.path.join(HERE, "groups.npz"), **out)


if __name__ == "__main__":
    main()
