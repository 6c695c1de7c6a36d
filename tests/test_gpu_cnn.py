"""Warm-start network on the GPU: the tcgen05 GEMM against torch, and the
network's forward pass and gradients against its CPU oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def orc(built):
    from oracle import oracle
    return oracle


def _bf16(t):
    import torch
    return t.to(torch.bfloat16)


@pytest.mark.parametrize("bn", [32, 64, 128, 256])
@pytest.mark.parametrize("shape", [(128, 64, 64), (300, 96, 200), (77, 250, 1000)])
def test_umma_gemm_matches_torch(gpu, bn, shape):
    """C = A B^T with BF16 operands and FP32 accumulation: against torch's
    FP32 product of the same BF16 values (FP32 summation-order tolerance)."""
    import torch
    from slam_gb300.warmstart import debug_gemm
    M, N, K = shape
    g = torch.Generator(device="cuda").manual_seed(M * 7 + N + K)
    A = _bf16(torch.randn(M, K, device="cuda", generator=g))
    B = _bf16(torch.randn(N, K, device="cuda", generator=g))
    ref = A.float() @ B.float().T
    C = debug_gemm(A, B, bn=bn, layout=0)
    torch.cuda.synchronize()
    err = (C - ref).abs().max().item()
    tol = 1e-5 * K ** 0.5 * ref.abs().max().item() + 1e-4
    assert err <= tol, (bn, shape, err, tol)
    # the asynchronously fed kernels (B by cp.async, and by TMA as the forward
    # pass runs it): the same MMAs on the same operand values, so the same bits
    for layout in (8, 9):
        Ca = debug_gemm(A, B, bn=bn, layout=layout)
        torch.cuda.synchronize()
        assert torch.equal(Ca, C), (bn, shape, layout, (Ca - C).abs().max().item())


@pytest.mark.parametrize("bn", [32, 128])
def test_umma_gemm_fp16_operands(gpu, bn):
    """The FP16 variant (first network layer): against torch on FP16 values."""
    import torch
    from slam_gb300.warmstart import debug_gemm
    g = torch.Generator(device="cuda").manual_seed(bn)
    A = torch.randn(200, 72, device="cuda", generator=g).half()
    B = torch.randn(32, 72, device="cuda", generator=g).half()
    ref = A.float() @ B.float().T
    C = debug_gemm(A.view(torch.bfloat16), B.view(torch.bfloat16), bn=bn, layout=2)
    torch.cuda.synchronize()
    assert (C - ref).abs().max().item() <= 1e-4 * ref.abs().max().item() + 1e-4


def test_umma_operand_layout_self_check(gpu):
    """The exchanged core-matrix offsets give a different (wrong) product:
    the layout test above is sensitive to the descriptor's offsets."""
    import torch
    from slam_gb300.warmstart import debug_gemm
    g = torch.Generator(device="cuda").manual_seed(5)
    A = _bf16(torch.randn(128, 64, device="cuda", generator=g))
    B = _bf16(torch.randn(64, 64, device="cuda", generator=g))
    ref = A.float() @ B.float().T
    C1 = debug_gemm(A, B, bn=64, layout=1)
    torch.cuda.synchronize()
    assert (C1 - ref).abs().max().item() > 1e-2


def _random_batch(B, seed):
    rng = np.random.default_rng(seed)
    x = np.zeros((B, 120, 160, 8), np.float16)
    for c, (lo, hi) in enumerate([(0.5, 4.0), (0.0, 1.0), (0.5, 4.0), (0.0, 1.0)]):
        x[..., c] = rng.uniform(lo, hi, size=(B, 120, 160))
    x[rng.uniform(size=(B, 120, 160)) < 0.05, 0] = 0  # invalid depth
    lab = rng.normal(0, 0.05, size=(B, 6)).astype(np.float32)
    return x, lab


def _net_and_inputs(B, seed):
    import torch
    from slam_gb300.warmstart import WarmStartNet
    net = WarmStartNet(max_batch=max(B, 4), seed=seed)
    x, lab = _random_batch(B, seed)
    xd = torch.from_numpy(x).cuda()
    ld = torch.from_numpy(lab).cuda()
    return net, x, lab, xd, ld


def test_cnn_forward_matches_oracle(gpu, orc):
    import torch
    from slam_gb300.warmstart import DEFAULT_LOSS_METRIC
    net, x, lab, xd, ld = _net_and_inputs(3, 11)
    out = net.forward(xd)
    torch.cuda.synchronize()
    p = net.get_params()
    o_ref, loss_ref, _ = orc.cnn_run(p, x.view(np.uint16), lab, DEFAULT_LOSS_METRIC, rounding=True, want_grad=False)
    o = out.cpu().numpy().astype(np.float64)
    # The tensor cores accumulate in FP32 in their own order; where a sum lies
    # within that difference of a BF16 rounding boundary the stored activation
    # differs by one BF16 ulp (2^-8), and such flips propagate through the
    # remaining layers: agreement to ~1e-3 of the output scale, not bitwise.
    rel = np.abs(o - o_ref).max() / np.abs(o_ref).max()
    assert rel < 1e-2, rel
    e = o - lab
    assert abs(loss_ref - float(np.einsum("bi,ij,bj->", e, DEFAULT_LOSS_METRIC, e)) / 3) < 1e-2 * loss_ref


def test_cnn_gradients_match_oracle(gpu, orc):
    """Per layer, the GPU's weight and bias gradients (tensor-core products,
    FP32 accumulation) against the CPU oracle with the same BF16 rounding
    points: relative error of each gradient tensor.  A full (non-diagonal)
    loss metric."""
    net, x, lab, xd, ld = _net_and_inputs(2, 23)
    rng = np.random.default_rng(3)
    A = rng.normal(size=(6, 6))
    metric = A @ A.T + np.eye(6)
    net.set_loss_metric(metric)
    metric = metric.astype(np.float32).astype(np.float64)
    g, loss = net.gradients(xd, ld)
    p = net.get_params()
    _, loss_ref, g_ref = orc.cnn_run(p, x.view(np.uint16), lab, metric, rounding=True)
    assert abs(loss - loss_ref) <= 1e-2 * abs(loss_ref)
    w, b, total = orc.cnn_layout()
    rows = [32, 64, 128, 128, 128, 128, 768, 6]
    cols = [72, 288, 576, 1152, 1152, 1152, 768, 768]
    for l in range(8):
        for name, off, n in (("W", w[l], rows[l] * cols[l]), ("b", b[l], rows[l])):
            a, r = g[off:off + n].astype(np.float64), g_ref[off:off + n]
            # gradients are sums with heavy cancellation: the FP32 order of the
            # tensor cores moves BF16 rounding decisions of the activation
            # gradients (one BF16 ulp = 2^-8), and such differences compound
            # layer by layer going backwards; an indexing error would give a
            # cosine near 0, not near 1
            rel = np.linalg.norm(a - r) / max(np.linalg.norm(r), 1e-30)
            cos = float(a @ r) / max(np.linalg.norm(a) * np.linalg.norm(r), 1e-30)
            assert rel < 3e-2 and cos > 0.9995, (l, name, rel, cos)


def test_cnn_training_reduces_loss(gpu):
    """A few hundred Adam steps on one fixed batch: the network fits it."""
    net, x, lab, xd, ld = _net_and_inputs(16, 31)
    first = net.train_step(xd, ld, 1e-3)
    for _ in range(200):
        last = net.train_step(xd, ld, 1e-3, want_loss=False)
    last = net.train_step(xd, ld, 1e-3)
    assert last < 0.1 * first, (first, last)


def test_cnn_batch_consistency(gpu):
    """Large batches (several 128-row tiles in every product): the outputs of
    a batch equal those of its halves run alone, and the batch gradient is
    the mean of the halves' gradients (the loss is a batch mean)."""
    import torch
    from slam_gb300.warmstart import WarmStartNet
    net = WarmStartNet(max_batch=256, seed=5)
    x, lab = _random_batch(256, 41)
    xd = torch.from_numpy(x).cuda()
    ld = torch.from_numpy(lab).cuda()
    full = net.forward(xd).cpu().numpy()
    lo = net.forward(xd[:128].contiguous()).cpu().numpy()
    hi = net.forward(xd[128:].contiguous()).cpu().numpy()
    scale = np.abs(full).max()
    assert np.abs(full[:128] - lo).max() <= 1e-2 * scale
    assert np.abs(full[128:] - hi).max() <= 1e-2 * scale
    g, _ = net.gradients(xd, ld)
    g1, _ = net.gradients(xd[:128].contiguous(), ld[:128].contiguous())
    g2, _ = net.gradients(xd[128:].contiguous(), ld[128:].contiguous())
    gm = 0.5 * (g1.astype(np.float64) + g2)
    from oracle import oracle
    w, b, total = oracle.cnn_layout()
    for l in range(8):
        for name, off, n in (("W", w[l], b[l] - w[l]), ("b", b[l], (w[l + 1] if l < 7 else total) - b[l])):
            a, r = g[off:off + n].astype(np.float64), gm[off:off + n]
            rel = np.linalg.norm(a - r) / max(np.linalg.norm(r), 1e-30)
            assert rel < 3e-2, (l, name, rel)
