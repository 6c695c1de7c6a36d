"""The allocation-free ICP reduction (odo_icp_step_noalloc).

Some callers of this tracker cannot allocate device memory once they are
running: a SLAM front end that works inside a fixed device-memory budget, or
a real-time loop in which a cudaMalloc/cudaFree would synchronise the device
and stall other streams.  For them the library exports one entry point that
takes caller-owned inputs and outputs and keeps its scratch in a fixed
device array of the library.  This file checks it through the C ABI against
the existing ICP reduction (odo_debug_icp_step) on the same maps and poses,
on two calls in a row, with the tolerance of the other parity tests, and
against the CPU oracle's ICP sums; once with maps whose row pitch is larger
than a row.  It is collected last so that a failure here does not hide the
other tests."""
import ctypes

import numpy as np
import pytest

from conftest import ANGLE_THRESH, DIST_THRESH
from gpu_helpers import intr, load_frame, new_gpu_odo, rel_close

pytestmark = pytest.mark.gpu


def _unpack(out29):
    A = np.zeros((6, 6))
    b = np.zeros(6)
    s = 0
    for i in range(6):
        for j in range(i, 7):
            if j == 6:
                b[i] = out29[s]
            else:
                A[i, j] = A[j, i] = out29[s]
            s += 1
    return A, b, out29[27:29]


def _pitched_map(m, extra):
    """Planar map [3][rows][cols] on the device with a row pitch of
    (cols + extra) floats; returns (tensor, pitch in bytes)."""
    import torch
    c, h, w = m.shape
    buf = torch.full((c * h, w + extra), float("nan"), dtype=torch.float32, device="cuda")
    buf[:, :w] = torch.from_numpy(np.ascontiguousarray(m).reshape(c * h, w)).cuda()
    return buf, (w + extra) * 4


@pytest.mark.parametrize("extra", [0, 5], ids=["tight", "pitched"])
def test_noalloc_icp_step_matches_existing_entry_point(gpu, extra):
    import torch
    from oracle import oracle
    from slam_gb300 import _native, synth
    L = _native.load()
    pair = synth.make_pair(12)
    odo = new_gpu_odo(pair["cam"])
    load_frame(odo, pair)
    T1 = pair["T1"]
    Tc = T1 @ synth.random_motion(np.random.default_rng(3), 1.0, 0.01)
    Rc = np.ascontiguousarray(Tc[:3, :3], np.float32)
    tc = np.ascontiguousarray(Tc[:3, 3], np.float32)
    Rpi = np.ascontiguousarray(np.linalg.inv(T1[:3, :3]), np.float32)
    tp = np.ascontiguousarray(T1[:3, 3], np.float32)
    fp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    stream = torch.cuda.current_stream()
    for level in (0, 1):
        host = [odo.download(w, level) for w in (1, 2, 3, 4)]
        _, h, w = host[0].shape
        maps, pitches = zip(*[_pitched_map(m, extra) for m in host])
        pitch = pitches[0]
        K = np.array(intr(pair["cam"], level), np.float32)
        expect, assoc = odo.debug_icp_step(level, Rc, tc, Rpi, tp, want_assoc=True)
        eA, eb, er = _unpack(expect)
        # the CPU oracle's icpStep on the same maps (sums compared where no
        # association decision falls on a rounding tie)
        fx, fy, cx, cy = intr(pair["cam"], level)
        o29, o_assoc, tie = oracle.Kernels(32).icp_step(Rc, tc, host[0], host[1], Rpi, tp, fx, fy, cx, cy, host[2],
                                                        host[3], DIST_THRESH, ANGLE_THRESH)
        oA, ob, orr = _unpack(o29)
        oracle_comparable = np.array_equal(o_assoc, assoc)
        torch.cuda.synchronize()
        for call in range(2):  # two calls in a row share the library's scratch array
            A = np.zeros(36, np.float32)
            b = np.zeros(6, np.float32)
            r = np.zeros(2, np.float32)
            rc = L.odo_icp_step_noalloc(maps[0].data_ptr(), maps[1].data_ptr(), maps[2].data_ptr(),
                                        maps[3].data_ptr(), pitch, w, h, fp(K), DIST_THRESH, ANGLE_THRESH, fp(Rc), fp(tc),
                                        fp(Rpi), fp(tp), ctypes.c_void_p(stream.cuda_stream), fp(A), fp(b), fp(r))
            assert rc == 0, (level, call, rc)
            assert r[1] == er[1], (level, call, r[1], er[1])  # inlier counts are exact
            for got, exp in ((A.reshape(6, 6), eA), (b, eb), (r[:1], er[:1])):
                ok, err = rel_close(got, exp, 2e-5)
                assert ok, (level, call, err)
            if oracle_comparable:
                assert r[1] == orr[1], (level, call, r[1], orr[1])
                for got, exp in ((A.reshape(6, 6), oA), (b, ob), (r[:1], orr[:1])):
                    ok, err = rel_close(got, exp, 2e-5)
                    assert ok, ("oracle", level, call, err)
            else:
                assert np.all(tie[o_assoc != assoc] != 0), level


def test_noalloc_rejects_oversized_images(built):
    from slam_gb300 import _native
    L = _native.load()
    z = np.zeros(9, np.float32)
    fp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    out = np.zeros(36, np.float32)
    # 2048 x 1024 > ODO_NOALLOC_MAX_PIXELS: refused before any CUDA call
    rc = L.odo_icp_step_noalloc(1, 1, 1, 1, 2048 * 4, 2048, 1024, fp(z), 0.1, 0.3, fp(z), fp(z), fp(z), fp(z), None,
                                fp(out), fp(out), fp(out))
    assert rc == 6
    assert b"ODO_NOALLOC_MAX_PIXELS" in L.odo_status_string(6)
