"""Entry points of the drop-in boundary beside the depth-input path:

* initICP(verts, norms) (src/odom/RGBDOdometryef.cpp:144-167) bit for bit
  against the reference's own copyMaps / resizeVMap / resizeNMap kernels, with
  row pitches larger than the row;
* the loop-closure caller shapes of the reference -- Ferns::findFrame's
  80x60 ICP-only check (src/lc/Ferns.cpp:253-270: initICPModel +
  initICP(maps) + getIncrementalTransformation(false, 100, false, false,
  false)) and the model-to-model check with covariance gating
  (src/apps/elastic_fusion_file.cpp:450-485) -- against the oracle's host
  loop;
* getCovariance (src/odom/RGBDOdometryef.cpp:597-600) against the oracle's
  LU inverse;
* one whole tracking call through the C++ shim (include/RGBDOdometryGB.hpp)
  from a C++ program with pitched device allocations."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT
from gpu_helpers import (OracleRuns, check_pose, dev, frame_runs, gpu_images, new_gpu_odo, pair_images, rel_close,
                         report, set_images, track)

pytestmark = pytest.mark.gpu


def pitched(a, extra_cols):
    """A CUDA tensor view of `a` ([rows][cols][4] or [rows][cols]) whose rows
    are `extra_cols` elements longer than the image (a non-tight pitch)."""
    import torch
    a = np.ascontiguousarray(a)
    shape = (a.shape[0], a.shape[1] + extra_cols) + a.shape[2:]
    buf = torch.zeros(shape, dtype={np.float32: torch.float32, np.uint8: torch.uint8}[a.dtype.type], device="cuda")
    buf[:, :a.shape[1]] = torch.from_numpy(a).cuda()
    return buf[:, :a.shape[1]]


@pytest.fixture(scope="module")
def ref(gpu):
    from oracle import ref_runner
    if not ref_runner.available():
        pytest.skip("reference cubin not built (needs the reference checkout at build time)")
    return ref_runner.RefKernels()


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def same_map(ours, theirs):
    o = ours.reshape(3, -1)
    t = theirs.reshape(3, -1)
    if not np.array_equal(np.isnan(o[0]), np.isnan(t[0])):
        return False
    ok = ~np.isnan(t[0])
    return np.array_equal(bits(o[:, ok]), bits(t[:, ok]))


def live_maps(pair, scene_seed):
    """Camera-frame RGBA32F vertex/normal maps of the live view (what
    Ferns/FillIn hand to initICP(verts, norms)), rendered noise-free at T2."""
    from slam_gb300 import synth
    scene = synth.make_room(scene_seed)
    m = synth.render(scene, pair["T2"], pair["cam"], depth=False, rgba=True, model=True)
    return m["vert"], m["norm"], m["rgba"]


@pytest.mark.parametrize("extra", [0, 7], ids=["tight", "pitched"])
def test_init_icp_maps_matches_reference(ref, extra):
    from slam_gb300 import synth
    pair = synth.make_pair(12)
    v4, n4, _ = live_maps(pair, 12)
    odo = new_gpu_odo(pair["cam"])
    odo.initICP(pitched(v4, extra), pitched(n4, extra), 20.0)
    vm, nm = ref.copy_maps(dev(v4), dev(n4))
    raw = [(vm, nm)]
    for l in (1, 2):
        raw.append((ref.resize(raw[-1][0], False), ref.resize(raw[-1][1], True)))
    for l in range(3):
        assert same_map(odo.download(1, l), raw[l][0].cpu().numpy()), ("vmap_curr", l)
        assert same_map(odo.download(2, l), raw[l][1].cpu().numpy()), ("nmap_curr", l)
    # quirk kept (src/odom/RGBDOdometryef.cpp:245): initRGB's depth comes
    # from the maps of the last initICP(verts, norms)
    odo.initRGB(pitched(pair["rgba"], extra))
    d0 = ref.verts_to_depth(dev(v4)).cpu().numpy()
    got = odo.download(6, 0)
    ok = ~np.isnan(d0)
    assert np.array_equal(np.isnan(got), ~ok) and np.array_equal(bits(got[ok]), bits(d0[ok]))


def _ferns_pair(seed):
    """A relocalisation candidate at the Ferns resolution (640x480 / 8):
    the stored fern's maps at T1, the current frame's maps at T2."""
    from slam_gb300 import synth
    cam = synth.Camera().scaled(80, 60)
    pair = synth.make_pair(seed, cam=cam, max_deg=4.0, max_m=0.05)
    pair["live_vert"], pair["live_norm"], pair["live_rgba"] = live_maps(pair, seed)
    return pair


FERNS_FLAGS = dict(rgbOnly=False, icpWeight=100.0, pyramid=False, fastOdom=False, so3=False)


def _load_maps(odo, pair, rgb):
    is_gpu = hasattr(odo, "handle")
    cv = dev if is_gpu else (lambda a: a)
    odo.initICPModel(cv(pair["model_vert"]), cv(pair["model_norm"]), 20.0, pair["T1"].astype(np.float32))
    if rgb:
        odo.initRGBModel(cv(pair["model_rgba"]))
    odo.initICP(cv(pair["live_vert"]), cv(pair["live_norm"]), 20.0)
    if rgb:
        odo.initRGB(cv(pair["live_rgba"]))


@pytest.mark.parametrize("seed", [21, 22, 23])
def test_ferns_shaped_check_matches_oracle(gpu, seed):
    pair = _ferns_pair(seed)
    g = new_gpu_odo(pair["cam"])
    _load_maps(g, pair, rgb=False)
    tg, Rg = track(g, pair, **FERNS_FLAGS)
    T1 = pair["T1"]
    ref = OracleRuns(pair["cam"], lambda o: _load_maps(o, pair, rgb=False), (T1[:3, 3], T1[:3, :3]), FERNS_FLAGS)
    to, Ro, o = ref.main
    check_pose("ferns 80x60 seed %d" % seed, tg, Rg, to, Ro, ref.tolerance)
    assert g.iterations() == o.iterations() == [0, 10, 0, 0]
    st = o.stats
    assert g.lastICPCount == st["lastICPCount"]
    assert abs(g.lastICPError - st["lastICPError"]) <= 1e-3 * st["lastICPError"]
    # the acceptance test of Ferns::findFrame (src/lc/Ferns.cpp:275-279)
    accept_g = g.lastICPError < 0.0003 and g.lastICPCount > 2400
    accept_o = st["lastICPError"] < 0.0003 and st["lastICPCount"] > 2400
    assert accept_g == accept_o
    report("ferns 80x60 seed %d: ICP error %.3e count %d accept %s" % (seed, g.lastICPError, g.lastICPCount,
                                                                       accept_g))


@pytest.mark.parametrize("seed", [31, 32])
def test_model_to_model_check_matches_oracle(gpu, seed):
    """initICPModel(old maps) + initRGBModel + initICP(new maps) + initRGB,
    tracked with ICP+RGB, pyramid, no SO3; then getCovariance's diagonal as
    the gate (src/apps/elastic_fusion_file.cpp:462-498)."""
    from slam_gb300 import synth
    pair = synth.make_pair(seed, cam=synth.Camera().scaled(320, 240), max_deg=3.0, max_m=0.05)
    pair["live_vert"], pair["live_norm"], pair["live_rgba"] = live_maps(pair, seed)
    flags = dict(rgbOnly=False, icpWeight=10.0, pyramid=True, fastOdom=False, so3=False)
    g = new_gpu_odo(pair["cam"])
    _load_maps(g, pair, rgb=True)
    images = gpu_images(g)
    tg, Rg = track(g, pair, **flags)

    def load(o):
        _load_maps(o, pair, rgb=True)
        set_images(o, images)
    T1 = pair["T1"]
    ref = OracleRuns(pair["cam"], load, (T1[:3, 3], T1[:3, :3]), flags)
    to, Ro, o = ref.main
    tol = ref.tolerance
    check_pose("model-to-model 320x240 seed %d" % seed, tg, Rg, to, Ro, tol)
    assert ref.iterations_ok(g.iterations())
    cg, co = g.getCovariance(), o.getCovariance()
    # the handle's covariance is the inverse of its own lastA ...
    ok, err = rel_close(cg, np.linalg.inv(np.asarray(g.lastA, np.float64).reshape(6, 6)), 1e-9)
    assert ok, err
    # ... and within the conditioning-amplified FP32 sum difference of the oracle's
    A_g = np.asarray(g.lastA, np.float64).reshape(6, 6)
    A_o = o.stats["lastA"]
    dA = np.abs(A_g - A_o).max() / np.abs(A_o).max()
    bound = max(1e-6, 4 * np.linalg.cond(A_o) * dA)
    ok, err = rel_close(cg, co, bound)
    report("model-to-model seed %d: covariance rel diff %.2e (bound %.2e, cond %.1e)" % (seed, err, bound,
                                                                                         np.linalg.cond(A_o)))
    assert ok, (err, bound)
    cov_thresh = 1e-5
    assert all(cg[i, i] <= cov_thresh for i in range(6)) == all(co[i, i] <= cov_thresh for i in range(6))


SHIM_PROG = r'''
// One tracking call through the C++ shim with pitched device buffers
// (cudaMallocPitch); the inputs come from files the test writes, the pose
// and statistics go to stdout.
#include "RGBDOdometryGB.hpp"
#include <cuda_runtime.h>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

static std::vector<unsigned char> slurp(const std::string &path, size_t n) {
    std::vector<unsigned char> b(n);
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f || std::fread(b.data(), 1, n, f) != n) {
        std::fprintf(stderr, "cannot read %s\n", path.c_str());
        std::exit(4);
    }
    std::fclose(f);
    return b;
}
static void *upload(const std::vector<unsigned char> &h, int w, int rows, int bpp, size_t *pitch) {
    void *d = nullptr;
    if (cudaMallocPitch(&d, pitch, (size_t)w * bpp, rows) != cudaSuccess) std::exit(5);
    if (cudaMemcpy2D(d, *pitch, h.data(), (size_t)w * bpp, (size_t)w * bpp, rows, cudaMemcpyHostToDevice) !=
        cudaSuccess)
        std::exit(6);
    return d;
}

int main(int argc, char **argv) {
    if (argc != 7) return 8;
    const std::string dir = argv[1];
    const int W = std::atoi(argv[2]), H = std::atoi(argv[3]);
    const float fx = (float)std::atof(argv[4]), cx = (float)std::atof(argv[5]), cy = (float)std::atof(argv[6]);
    const size_t n = (size_t)W * H;
    auto mv = slurp(dir + "/mv", n * 16), mn = slurp(dir + "/mn", n * 16), mr = slurp(dir + "/mr", n * 4);
    auto d = slurp(dir + "/d", n * 2), r = slurp(dir + "/r", n * 4), pr = slurp(dir + "/pr", n * 4);
    auto Tb = slurp(dir + "/T", 64);
    float T[16];
    std::memcpy(T, Tb.data(), 64);
    size_t pv, pn, pmr, pd, prr, ppr;
    void *dmv = upload(mv, W, H, 16, &pv), *dmn = upload(mn, W, H, 16, &pn), *dmr = upload(mr, W, H, 4, &pmr);
    void *dd = upload(d, W, H, 2, &pd), *dr = upload(r, W, H, 4, &prr), *dpr = upload(pr, W, H, 4, &ppr);
    if (pv != pn) return 7;
    try {
        RGBDOdometryGB odo(W, H, cx, cy, fx, fx);
        odo.initFirstRGB((const uint8_t *)dpr, ppr);
        odo.initICPModel((const float *)dmv, (const float *)dmn, pv, 20.0f, T);
        odo.initRGBModel((const uint8_t *)dmr, pmr);
        odo.initICP((const uint16_t *)dd, pd, 20.0f);
        odo.initRGB((const uint8_t *)dr, prr);
        float t[3] = {T[3], T[7], T[11]};
        float R[9] = {T[0], T[1], T[2], T[4], T[5], T[6], T[8], T[9], T[10]};
        odo.getIncrementalTransformation(t, R, false, 10.0f, true, false, true);
        double cov[36];
        odo.getCovariance(cov);
        std::printf("%zu %zu\n", pd, pv);
        for (float v : t) std::printf("%.9g ", v);
        for (float v : R) std::printf("%.9g ", v);
        std::printf("\n%.9g %.9g\n", odo.lastICPError, odo.lastICPCount);
        for (double v : odo.lastA) std::printf("%.17g ", v);
        std::printf("\n");
        for (double v : cov) std::printf("%.17g ", v);
        std::printf("\n");
    } catch (const RGBDOdometryGB::Error &e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 3;
    }
    return 0;
}
'''


def test_cpp_shim_tracking_call(gpu, tmp_path):
    from slam_gb300 import _build, synth
    cam = synth.Camera().scaled(320, 240)
    assert cam.fx == cam.fy
    pair = synth.make_pair(41, cam=cam)
    for name, key in (("mv", "model_vert"), ("mn", "model_norm"), ("mr", "model_rgba"), ("d", "depth"),
                      ("r", "rgba"), ("pr", "prev_rgba")):
        np.ascontiguousarray(pair[key]).tofile(str(tmp_path / name))
    pair["T1"].astype(np.float32).tofile(str(tmp_path / "T"))
    src = tmp_path / "shim_track.cpp"
    src.write_text(SHIM_PROG)
    exe = tmp_path / "shim_track"
    libdir = os.path.dirname(_build.LIB)
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"), "-I" + cuda + "/include",
                           str(src), "-L" + libdir, "-lslam_gb300", "-Wl,-rpath," + libdir, "-L" + cuda + "/lib64",
                           "-lcudart", "-Wl,-rpath," + cuda + "/lib64", "-o", str(exe)])
    out = subprocess.run([str(exe), str(tmp_path), str(cam.width), str(cam.height), repr(cam.fx), repr(cam.cx),
                          repr(cam.cy)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    lines = out.stdout.strip().splitlines()
    pd, pv = (int(v) for v in lines[0].split())
    assert pd >= 320 * 2 and pv >= 320 * 16
    report("C++ shim: cudaMallocPitch pitches depth %d B (row %d B), maps %d B (row %d B)" % (pd, 640, pv, 5120))
    pose = np.array(lines[1].split(), np.float64)
    tg, Rg = pose[:3], pose[3:].reshape(3, 3)
    icp_err, icp_cnt = (float(v) for v in lines[2].split())
    lastA = np.array(lines[3].split(), np.float64).reshape(6, 6)
    cov = np.array(lines[4].split(), np.float64).reshape(6, 6)
    ref = frame_runs(pair, {}, images=pair_images(pair))
    to, Ro, o = ref.main
    _, _, flat = check_pose("C++ shim 320x240", tg, Rg, to, Ro, ref.tolerance)
    st = o.stats
    assert ref.count_ok("lastICPCount", icp_cnt, flat)
    ok, err = ref.jtj_ok(lastA, flat)
    assert ok, err
    ok, err = rel_close(cov, np.linalg.inv(lastA), 1e-9)
    assert ok, err
