"""Build libpsy_gpu.so (the C ABI of include/psy_gpu.h) with nvcc for sm_103a.

Each translation unit compiles in its own nvcc process (in parallel), then
one nvcc link step makes the shared library in psychopath_gb300/_lib/.
Floating point: --fmad=false on the device and -ffp-contract=off on the host
so every operation rounds as written (parity with the reference's CPU
arithmetic); precise division and square root stay on (nvcc defaults).  The
one exception is wave_f32.cu, the f32 camera and hit-shading kernels of the
optimized form, compiled with FMA contraction (its error against the FP64
oracle is measured).
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB_PATH = os.path.join(OUT_DIR, "libpsy_gpu.so")
SOURCES = ["kernels.cu", "trace_kernels.cu", "scene_build.cu", "capi.cu", "server.cu", "bvh_build.cu",
           "radix_sort.cu", "halton.cu", "wave_f32.cu", "compact.cu"]
FMAD = {"wave_f32.cu": "--fmad=true"}  # per-source override of --fmad=false
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cuh", ".h", ".inc"))]
    files.append(os.path.join(HERE, "..", "include", "psy_gpu.h"))
    return files


def build(force=False, verbose=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB_PATH):
        t = os.path.getmtime(LIB_PATH)
        if all(os.path.getmtime(d) <= t for d in _deps()):
            return LIB_PATH
    common = ARCH + ["-O3", "-lineinfo", "-std=c++17", "--fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off",
                     "-I", os.path.join(HERE, "..", "include")]
    # extra nvcc flags (e.g. -DPSY_SSTACK=8 for another shared-memory stack
    # depth); pass force=True when changing them
    common += os.environ.get("PSY_NVCC_EXTRA", "").split()
    objs = []

    def compile_one(src):
        obj = os.path.join(OUT_DIR, src.replace(".cu", ".o"))
        cmd = [nvcc(), "-c", os.path.join(CSRC, src), "-o", obj] + [FMAD.get(src, f) if f == "--fmad=false" else f
                                                                   for f in common]
        if verbose:
            cmd += ["-Xptxas", "-v"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
        if verbose:
            sys.stderr.write(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB_PATH + ".tmp"
    cmd = [nvcc(), "-shared", "-o", tmp] + objs + ARCH + ["-lcudart", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc link failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB_PATH)
