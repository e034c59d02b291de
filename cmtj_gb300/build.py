"""Build recipe of libcmtj_gpu.so (sm_103a only).

Each translation unit under csrc/ is compiled by nvcc in parallel and the
objects are linked into cmtj_gb300/_build/libcmtj_gpu.so (CUDA runtime
linked statically, so the library does not depend on which libcudart the
host process loaded).  The FP64 plain-form units are compiled with
--fmad=false: its arithmetic must round exactly like the reference's.
"""
import concurrent.futures
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(BUILD, "libcmtj_gpu.so")
INCLUDE = os.path.join(os.path.dirname(PKG), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I" + INCLUDE]
# per-unit extra flags
UNITS = {
    "abi.cu": [],
    "plain_f64.cu": ["--fmad=false"],
    "plain_lanes_f64.cu": ["--fmad=false"],
    "dp_quads_f64.cu": ["--fmad=false"],
    "stack_f64.cu": ["--fmad=false"],
    "stack_lanes_f64.cu": ["--fmad=false"],
    "group_f64.cu": ["--fmad=false"],
    "group_lanes_f64.cu": ["--fmad=false"],
    "batch_f32.cu": [],
    "batch_f32_l1.cu": [],
    "batch_f32_l2.cu": [],
    "batch_f32_l3.cu": [],
    "batch_f32_l4.cu": [],
    "reduce.cu": [],
    "alpha_noise.cu": [],
}


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs.append(os.path.join(INCLUDE, "cmtj_gpu.h"))
    return hs


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, extra_flags=(), units=None, lib=None):
    units = UNITS if units is None else units
    lib = LIB if lib is None else lib
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    hdrs = _headers() + [os.path.abspath(__file__)]
    objs = []
    jobs = []
    for unit, flags in units.items():
        src = os.path.join(CSRC, unit)
        obj = os.path.join(BUILD, unit.replace(".cu", ".o"))
        objs.append(obj)
        if _stale(obj, [src] + hdrs):
            cmd = [nvcc, *ARCH, *COMMON, *flags, *extra_flags, "-c", src, "-o", obj]
            jobs.append(cmd)

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
        if verbose and r.stderr.strip():
            print(r.stderr, flush=True)

    with concurrent.futures.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(run, jobs))
    if jobs or _stale(lib, objs):
        cmd = [nvcc, *ARCH, "-shared", "-o", lib + ".tmp", *objs]
        run(cmd)
        os.replace(lib + ".tmp", lib)
    return lib


if __name__ == "__main__":
    extra = sys.argv[1:]
    print(build(verbose=True, extra_flags=extra))
