"""Reference outputs of the PIMM and spin-diode procedures
(cmtj/utils/procedures.py:42-331), run with the reference extension built
from its sources (oracle/_ref) on small sweeps.  Output:
tests/golden/procedures.npz.

    CMTJ_REF=<reference checkout> python tests/golden/make_procedures.py
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
    import procedure_cases as pc
    from cmtj.utils.procedures import PIMM_procedure, ResistanceParameters, VSD_procedure
    out = {}
    for name, case in pc.CASES.items():
        j, kw = case(cm, ResistanceParameters)
        np.random.seed(pc.SEED)
        if kw.pop("kind") == "pimm":
            spec, freqs, o = PIMM_procedure(j, **kw)
            out[name + "__spectrum"] = np.asarray(spec)
            out[name + "__freqs"] = np.asarray(freqs)
            for k in ("Rx", "Ry", "m_avg"):
                out[name + "__" + k] = np.asarray(o[k])
        else:
            out[name + "__vsd"] = np.asarray(VSD_procedure(j, **kw))
        print(name, {k: v.shape for k, v in out.items() if k.startswith(name)})
    np.savez_compressed(os.path.join(HERE, "procedures.npz"), **out)


if __name__ == "__main__":
    main()
