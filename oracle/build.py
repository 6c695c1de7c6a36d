"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/odometry_oracle.c three times (shared integer kernels, FP32
and FP64 twins) and oracle/cnn_oracle.c (the warm-start network) into
oracle/_build/liboracle.so with gcc.  The oracle is
built with -ffp-contract=off so that x86-64 and aarch64 hosts round the same
way; the explicit fma() calls in the source model nvcc's fused
multiply-adds where the reference accumulates ``acc += a * b``.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")
SRC = os.path.join(HERE, "odometry_oracle.c")
CNN_SRC = os.path.join(HERE, "cnn_oracle.c")

CFLAGS = ["-O2", "-fPIC", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-std=gnu11",
          "-Wall", "-Wno-unused-function", "-Wno-unknown-pragmas"]


def build_oracle(force=False, verbose=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(
            os.path.getmtime(SRC), os.path.getmtime(os.path.join(HERE, "odometry_oracle.h")),
            os.path.getmtime(CNN_SRC), os.path.getmtime(__file__)):
        return LIB
    objs = []
    procs = []
    for tag, define in (("shared", "ORC_SHARED"), ("f32", "ORC_REAL_F32"), ("f64", "ORC_REAL_F64")):
        obj = os.path.join(OUT_DIR, f"oracle_{tag}.o")
        cmd = ["gcc", *CFLAGS, f"-D{define}", "-c", SRC, "-o", obj]
        if verbose:
            print(" ".join(cmd))
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
        objs.append(obj)
    obj = os.path.join(OUT_DIR, "cnn_oracle.o")
    cmd = ["gcc", *CFLAGS, "-c", CNN_SRC, "-o", obj]
    procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    objs.append(obj)
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("oracle build failed: %s\n%s" % (" ".join(cmd), out.decode()))
    cmd = ["gcc", "-shared", "-fopenmp", "-o", LIB, *objs, "-lm"]
    subprocess.check_call(cmd)
    return LIB


if __name__ == "__main__":
    print(build_oracle(force=True, verbose="-v" in sys.argv))
