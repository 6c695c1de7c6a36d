"""In-tree build of the native libraries (no cmake).

  slam_gb300/_lib/libslam_gb300.so  -- the tracker: CUDA kernels for sm_103a
                                       + C++ host driver + C ABI
  slam_gb300/_lib/libslam_synth.so  -- synthetic RGB-D scene generator (host)

The odometry kernels (odo_*.cu) are compiled with the reference's numeric flags
(--ftz=true --prec-div=false --prec-sqrt=false, src/CMakeLists.txt:116) so
that projective association decisions round exactly as the reference's do.
Translation units compile in parallel; a rebuild only happens when a source
is newer than the library.
"""
import glob
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "_lib")
OBJDIR = os.path.join(LIBDIR, "obj")
LIB = os.path.join(LIBDIR, "libslam_gb300.so")
SYNTH_LIB = os.path.join(LIBDIR, "libslam_synth.so")

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NUMERIC = ["--ftz=true", "--prec-div=false", "--prec-sqrt=false"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I" + os.path.join(ROOT, "include")]

# translation units of the tracker library
CU_SOURCES = ["odo_maps.cu", "odo_track.cu", "depth_filter.cu", "model_predict.cu", "cnn.cu", "synth_gpu.cu",
              "transfer.cu"]
CPP_SOURCES = ["odo_host.cpp", "batch_host.cpp", "cnn_host.cpp", "inputs_host.cpp"]


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if p.returncode != 0:
        raise RuntimeError("build failed: %s\n%s" % (" ".join(cmd), p.stdout.decode(errors="replace")))
    return p.stdout.decode(errors="replace")


def build(force=False, verbose=False, extra_nvcc=()):
    os.makedirs(OBJDIR, exist_ok=True)
    headers = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(ROOT, "include", "*.h"))
    jobs = []
    objs = []
    for src in CU_SOURCES + CPP_SOURCES:
        path = os.path.join(CSRC, src)
        if not os.path.exists(path):
            continue
        obj = os.path.join(OBJDIR, src + ".o")
        objs.append(obj)
        if force or _newer(obj, [path, __file__] + headers):
            if src.endswith(".cu"):
                # the reference's numeric flags for the tracking kernels only
                numeric = NUMERIC if src.startswith("odo_") else []
                cmd = [NVCC, *ARCH, *COMMON, *numeric, "-Xcompiler", "-ffp-contract=off", *extra_nvcc, "-c", path,
                       "-o", obj]
            else:
                cmd = [NVCC, *COMMON, "-Xcompiler", "-ffp-contract=off", "-c", path, "-o", obj]
            jobs.append(cmd)
    with ThreadPoolExecutor(max_workers=max(1, min(8, os.cpu_count() or 1))) as ex:
        for f in [ex.submit(_run, j, verbose) for j in jobs]:
            f.result()
    if force or jobs or _newer(LIB, objs):
        _run([NVCC, *ARCH, "-shared", "-cudart", "static", "-o", LIB, *objs], verbose)
    synth_src = os.path.join(CSRC, "synth.cpp")
    if force or _newer(SYNTH_LIB, [synth_src, os.path.join(CSRC, "synth_common.h"), __file__]):
        _run(["g++", "-O2", "-fPIC", "-shared", "-fopenmp", "-std=c++17", "-ffp-contract=off",
              synth_src, "-o", SYNTH_LIB], verbose)
    return LIB


if __name__ == "__main__":
    build(force="-f" in sys.argv, verbose=True)
    print(LIB)
