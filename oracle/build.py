"""Compile the oracle restatement (oracle.c) into oracle/_build/liboracle.so.

Test infrastructure only. Plain gcc, no x86 intrinsics, so it builds on x86-64 and on aarch64.
-ffp-contract=off keeps the reference's unfused float operations; -fwrapv its wrapping int32.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
SOURCES = ["oracle.c", "oracle_adjoint.c"]


def build_oracle(force=False, openmp=True):
    srcs = [os.path.join(HERE, s) for s in SOURCES if os.path.exists(os.path.join(HERE, s))]
    hdrs = [os.path.join(HERE, "oracle.h")]
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(f) <= t for f in srcs + hdrs):
            return LIB
    os.makedirs(BUILD, exist_ok=True)
    flags = ["-O2", "-std=gnu11", "-fPIC", "-shared", "-ffp-contract=off", "-fwrapv", "-fno-fast-math"]
    cmd = ["gcc"] + flags + (["-fopenmp"] if openmp else []) + ["-o", LIB + ".tmp"] + srcs + ["-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0 and openmp:
        # a host without libgomp: build single-threaded
        cmd = ["gcc"] + flags + ["-o", LIB + ".tmp"] + srcs + ["-lm"]
        r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stderr)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
