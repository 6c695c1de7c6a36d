"""Failure detection of the bounded device-side waits, without a GPU fault.

* The persistent mode's grid-wide barriers (one cooperative kernel per
  pyramid level): one block is made to return without arriving (a block that
  died), the others give up after a short poll limit, the tracking call
  returns ODO_ERR_TIMEOUT, and the same handle then tracks normally.
* The warm-start network's tensor-core pipeline: one wait is made to wait on
  an mbarrier that nothing arrives at; the kernel drains the MMAs it issued,
  releases its TMEM and reports ODO_ERR_TIMEOUT; the next product on the same
  context is correct.

Nothing here hangs: every wait has a limit, and the waits made to run out
have short ones."""
import ctypes

import pytest

from gpu_helpers import check_pose, frame_runs, gpu_images, load_frame, new_gpu_odo, track

pytestmark = pytest.mark.gpu

ODO_ERR_TIMEOUT = 5


def test_persistent_barrier_times_out_and_handle_recovers(gpu):
    from slam_gb300 import MODE_PERSISTENT, OdometryError, _native, synth
    L = _native.load()
    pair = synth.make_pair(5, cam=synth.Camera().scaled(320, 240))
    g = new_gpu_odo(pair["cam"])
    g.set_mode(MODE_PERSISTENT)
    load_frame(g, pair)
    assert L.odo_debug_set_wait_limit(g.handle, 2000, 0) == 0
    with pytest.raises(OdometryError) as e:
        track(g, pair)
    assert e.value.status == ODO_ERR_TIMEOUT
    # back to the default limit, no absent block: the same handle tracks
    assert L.odo_debug_set_wait_limit(g.handle, 1 << 26, -1) == 0
    load_frame(g, pair)
    images = gpu_images(g)
    tg, Rg = track(g, pair)
    ref = frame_runs(pair, {}, images=images)
    to, Ro, o = ref.main
    check_pose("persistent after time-out", tg, Rg, to, Ro, ref.tolerance)
    assert L.odo_debug_set_wait_limit(g.handle, 0, -1) == 1  # bad limit refused


def test_tensor_core_wait_times_out_and_context_recovers(gpu):
    import torch
    from slam_gb300 import _native
    L = _native.load()
    g = torch.Generator().manual_seed(3)
    M, N, K = 256, 64, 320
    A = torch.randn(M, K, generator=g).to(torch.bfloat16).cuda()
    B = torch.randn(N, K, generator=g).to(torch.bfloat16).cuda()
    C = torch.zeros(M, N, dtype=torch.float32, device="cuda")
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    args = (ctypes.c_void_p(A.data_ptr()), ctypes.c_void_p(B.data_ptr()), ctypes.c_void_p(C.data_ptr()), M, N, K, 64)
    assert L.odo_cnn_debug_gemm(*args, 4, s) == ODO_ERR_TIMEOUT
    assert L.odo_cnn_debug_gemm(*args, 0, s) == 0
    torch.cuda.synchronize()
    ref = A.double().cpu() @ B.double().cpu().T
    err = (C.double().cpu() - ref).abs().max().item() / ref.abs().max().item()
    assert err < 1e-5, err
