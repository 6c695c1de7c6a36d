"""Build recipe for oracle/_ref/ref_kernels.cubin (test infrastructure only).

Compiles the reference's own kernels (src/odom/reduce.cu and src/odom/utils.cu
of a reference checkout, read in place, never copied)
through oracle/ref_shim.cu into a device-only cubin for sm_103a, with the
reference's numeric flags (src/CMakeLists.txt:116).  The reference's build
system (catkin/cmake with Eigen, Pangolin, OpenCV, GL) is not used and could
not run here; these two translation units need none of it.

The checkout is named by the `ref_root` argument or the SLAM_REFERENCE
environment variable (its top directory, the one holding src/).  The cubin
holds no host code, so the same file runs on any host CPU.  When no checkout
is named or present (as on a machine that only runs the tests), the
previously built cubin is used as is.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_ref")
CUBIN = os.path.join(OUT_DIR, "ref_kernels.cubin")
SHIM = os.path.join(HERE, "ref_shim.cu")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
FLAGS = ["-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++14", "--ftz=true",
         "--prec-div=false", "--prec-sqrt=false", "-diag-suppress", "2361,2464,20208,177,550,1215"]


def build_ref(ref_root=None, force=False, verbose=False):
    """Returns the cubin path, or None when it cannot be built or found."""
    ref_root = ref_root or os.environ.get("SLAM_REFERENCE", "")
    ref_src = os.path.join(ref_root, "src") if ref_root else ""
    srcs = [os.path.join(ref_src, "odom", "reduce.cu"), os.path.join(ref_src, "odom", "utils.cu")]
    if not ref_src or not all(os.path.exists(s) for s in srcs):
        return CUBIN if os.path.exists(CUBIN) else None
    os.makedirs(OUT_DIR, exist_ok=True)
    deps = srcs + [SHIM, __file__]
    if not force and os.path.exists(CUBIN) and os.path.getmtime(CUBIN) >= max(os.path.getmtime(d) for d in deps):
        return CUBIN
    cmd = [NVCC, *FLAGS, "-I" + ref_src, SHIM, "-o", CUBIN]
    if verbose:
        print(" ".join(cmd))
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if p.returncode != 0:
        sys.stderr.write("reference cubin build failed:\n" + p.stdout.decode(errors="replace")[-4000:])
        return None
    return CUBIN


if __name__ == "__main__":
    # usage: python -m oracle.build_ref <reference checkout>
    print(build_ref(sys.argv[1] if len(sys.argv) > 1 else None, force=True, verbose=True))
