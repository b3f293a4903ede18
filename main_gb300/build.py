"""Build the mpcmd CUDA library for sm_103a (in-tree, main_gb300/_build/)."""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libmpcmd.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
                 "-I", os.path.join(ROOT, "include")]
# (source, extra flags): the FP64 kernels are compiled without FMA contraction so
# their arithmetic is the operation sequence the FP64 oracle performs.
UNITS = [
    ("mpcmd_kernels_f32.cu", []),
    ("mpcmd_kernels_f64.cu", ["--fmad=false"]),
    ("mpcmd_scan.cu", []),
    ("mpcmd_engine.cu", []),
    ("mpcmd_static.cu", ["--fmad=false"]),
    ("mpcmd_ensemble_f32.cu", []),
    ("mpcmd_ensemble_f64.cu", ["--fmad=false"]),
    ("mpcmd_ensemble.cu", []),
    ("mpcmd_mlp.cu", []),
]
HEADERS = ["mpcmd_device.cuh", "mpcmd_engine.cuh", "mpcmd_kernels.cuh", "mpcmd_ensemble.cuh",
           "mpcmd_ensemble_impl.cuh", "mpcmd_ensemble_base.h"]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.sep not in c or os.path.exists(c)):
            return c
    return "nvcc"


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, u) for u, _ in UNITS] + [os.path.join(CSRC, h) for h in HEADERS]
    deps += [os.path.join(ROOT, "include", "mpcmd.h"), os.path.abspath(__file__)]
    return any(os.path.getmtime(p) > t for p in deps)


def build(force=False, verbose=False, checked=False):
    """Compile every CUDA unit (in parallel) and link libmpcmd.so; return its path.

    checked=True builds libmpcmd_checked.so with bounds checks that record and
    skip a bad index and a synchronisation after every launch."""
    lib = LIB if not checked else os.path.join(OUT, "libmpcmd_checked.so")
    if not checked and not force and not _stale():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    tag = "_checked" if checked else ""
    flags = ["-DMPCMD_CHECKED"] if checked else []

    def compile_unit(unit):
        src, extra = unit
        obj = os.path.join(OUT, src.replace(".cu", tag + ".o"))
        cmd = [nvcc] + COMMON + flags + extra + ["-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        subprocess.run(cmd, check=True)
        return obj

    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(compile_unit, UNITS))
    tmp = lib + ".tmp.%d" % os.getpid()
    subprocess.run([nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"], check=True)
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv, checked="--checked" in sys.argv))
