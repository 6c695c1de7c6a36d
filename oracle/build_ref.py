"""Build recipe for oracle/_ref/ref_kernels.cubin (test infrastructure only).

Compiles the reference's own kernels (src/odom/reduce.cu and src/odom/utils.cu
from the reference checkout at /root/reference, read in place, never copied)
through oracle/ref_shim.cu into a device-only cubin for sm_103a, with the
reference's numeric flags (src/CMakeLists.txt:116).  The reference's build
system (catkin/cmake with Eigen, Pangolin, OpenCV, GL) is not used and could
not run here; these two translation units need none of it.

The cubin holds no host code, so the same file runs on any host CPU.  When the
reference checkout is absent (as on a machine that only runs the tests), the
previously built cubin is used as is.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_SRC = "/root/reference/src"
OUT_DIR = os.path.join(HERE, "_ref")
CUBIN = os.path.join(OUT_DIR, "ref_kernels.cubin")
SHIM = os.path.join(HERE, "ref_shim.cu")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
FLAGS = ["-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++14", "--ftz=true",
         "--prec-div=false", "--prec-sqrt=false", "-diag-suppress", "2361,2464,20208,177,550,1215"]


def build_ref(force=False, verbose=False):
    """Returns the cubin path, or None when it cannot be built or found."""
    srcs = [os.path.join(REF_SRC, "odom", "reduce.cu"), os.path.join(REF_SRC, "odom", "utils.cu")]
    if not all(os.path.exists(s) for s in srcs):
        return CUBIN if os.path.exists(CUBIN) else None
    os.makedirs(OUT_DIR, exist_ok=True)
    deps = srcs + [SHIM, __file__]
    if not force and os.path.exists(CUBIN) and os.path.getmtime(CUBIN) >= max(os.path.getmtime(d) for d in deps):
        return CUBIN
    cmd = [NVCC, *FLAGS, "-I" + REF_SRC, SHIM, "-o", CUBIN]
    if verbose:
        print(" ".join(cmd))
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if p.returncode != 0:
        sys.stderr.write("reference cubin build failed:\n" + p.stdout.decode(errors="replace")[-4000:])
        return None
    return CUBIN


if __name__ == "__main__":
    print(build_ref(force=True, verbose=True))
