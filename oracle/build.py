"""Build recipe for the oracle (test infrastructure, never shipped).

Compiles oracle/cmtj_oracle.cpp into oracle/_build/libcmtj_oracle.so with
-ffp-contract=off so that a*b+c is never fused (the reference's x86-64
build has no FMA; on aarch64 GCC would otherwise contract), and, when the
reference checkout is named by $CMTJ_REF, runs oracle/build_ref.sh to build the real
reference extension into oracle/_ref/.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libcmtj_oracle.so")
SRC = os.path.join(HERE, "cmtj_oracle.cpp")
HDR = os.path.join(os.path.dirname(HERE), "include", "cmtj_gpu.h")
FLAGS = ["-O2", "-std=c++17", "-fPIC", "-shared", "-pthread", "-ffp-contract=off", "-fno-fast-math"]


def _stale(target, *deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build_oracle(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    if _stale(LIB, SRC, HDR, __file__):
        cmd = ["g++", *FLAGS, SRC, "-o", LIB + ".tmp"]
        if verbose:
            print(" ".join(cmd))
        subprocess.check_call(cmd)
        os.replace(LIB + ".tmp", LIB)
    return LIB


def build_reference(verbose=False):
    """Build oracle/_ref from the reference checkout named by $CMTJ_REF;
    None when it is unset or holds no python/cmtj.cpp."""
    ref = os.environ.get("CMTJ_REF")
    if not ref or not os.path.isfile(os.path.join(ref, "python", "cmtj.cpp")):
        return None
    subprocess.check_call(["bash", os.path.join(HERE, "build_ref.sh")],
                          stdout=None if verbose else subprocess.DEVNULL)
    return os.path.join(HERE, "_ref")


if __name__ == "__main__":
    print(build_oracle(verbose=True))
    print(build_reference(verbose=True))
    sys.exit(0)
