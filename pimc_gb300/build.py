"""Build the GB300 hot-path library (libpimc_gb300.so) with nvcc for sm_103a.

Every translation unit is compiled in parallel into pimc_gb300/_build/ and
linked in-tree next to this file.  fp64_kernels.cu is compiled with
-fmad=false so that the plain FP64 form rounds each product and sum once, in
the reference's order; the FP32 kernels with -ftz=true.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libpimc_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
          "-I", os.path.join(ROOT, "include"), "-I", CSRC]
PER_FILE = {
    "fp64_kernels.cu": ["-fmad=false"],
    # FP32 pair and phase kernels: subnormal FP32 values flush to zero, which
    # drops the subnormal handling around rsqrt/ex2/sin/cos (about 6 % of the
    # canonical walker sweep, 7 % of the worm walkers' step); FP64 arithmetic
    # is unaffected
    "walkers.cu": ["-ftz=true"],
    "mixed_kernels.cu": ["-ftz=true"],
    "scatter.cu": ["-ftz=true"],
    "isf_static.cu": ["-ftz=true"],
    "worm_walkers.cu": ["-ftz=true"],
    "path_estimators.cu": ["-fmad=false"],
    "gp.cu": ["-fmad=false"],
}
SOURCES = ["api.cu", "fp64_kernels.cu", "mixed_kernels.cu", "scatter.cu",
           "isf_tc.cu", "walkers.cu", "plain_moves.cu", "isf_static.cu", "path_estimators.cu", "gp.cu", "worm_walkers.cu"]


def nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _compile(src, extra_flags):
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    path = os.path.join(CSRC, src)
    deps = [path] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    deps.append(os.path.join(ROOT, "include", "pimc_gb300.h"))
    deps.append(os.path.abspath(__file__))          # flags live here
    if os.path.exists(obj) and all(os.path.getmtime(obj) >= os.path.getmtime(d) for d in deps):
        return obj, ""
    cmd = [nvcc()] + ARCH + COMMON + PER_FILE.get(src, []) + extra_flags + ["-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
    return obj, r.stderr


def build(verbose=False, extra_flags=()):
    os.makedirs(BUILD, exist_ok=True)
    srcs = [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        results = list(ex.map(lambda s: _compile(s, list(extra_flags)), srcs))
    objs = [o for o, _ in results]
    if verbose:
        for _, log in results:
            if log.strip():
                print(log)
    if not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcuda"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
