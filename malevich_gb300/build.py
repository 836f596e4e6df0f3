"""Build the CUDA library in-tree: malevich_gb300/libmalevich_gb300.so (sm_103a only).

The translation units are compiled in parallel with nvcc and linked into one shared library
that exports the C ABI declared in include/malevich.h. --fmad=false keeps every float
multiply and add separately rounded, as the reference's AVX code computes them.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libmalevich_gb300.so")
SOURCES = ["kernels.cu", "api.cu", "noalloc.cu", "adjoint.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "--fmad=false", "-prec-div=true", "-prec-sqrt=true", "-std=c++17",
         "-Xcompiler", "-fPIC,-fvisibility=hidden", "-I", CSRC, "-I", os.path.join(ROOT, "include")]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def _stale(outputs, inputs):
    if not all(os.path.exists(o) for o in outputs):
        return True
    t = min(os.path.getmtime(o) for o in outputs)
    return any(os.path.getmtime(i) > t for i in inputs)


def build(force=False, verbose=False, extra=()):
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(ROOT, "include", "malevich.h")]
    if not force and not _stale([LIB], deps + [__file__]):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()

    def compile_one(src):
        obj = os.path.join(BUILD, src + ".o")
        cmd = [nvcc] + ARCH + FLAGS + list(extra) + ["-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
        if verbose and r.stderr:
            print(r.stderr, file=sys.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s" % r.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    v = "-v" in sys.argv
    extra = ["-Xptxas", "-v"] if v else []
    print(build(force=True, verbose=v, extra=extra))
