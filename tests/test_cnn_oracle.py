"""CPU checks of the warm-start network's oracle: its backward formulas
against central finite differences (FP64 mode), and its parameter layout
against the library's."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def orc(built):
    from oracle import oracle
    return oracle


def _params(orc, rng):
    w, b, total = orc.cnn_layout()
    rows = [32, 64, 128, 128, 128, 128, 768, 6]
    cols = [72, 288, 576, 1152, 1152, 1152, 768, 768]
    p = np.zeros(total)
    for l in range(8):
        fan = cols[l]
        sd = np.sqrt(2.0 / fan) if l < 7 else 0.1 * np.sqrt(1.0 / fan)
        p[w[l]:w[l] + rows[l] * cols[l]] = rng.normal(0, sd, rows[l] * cols[l])
        p[b[l]:b[l] + rows[l]] = rng.normal(0, 0.01, rows[l])
    return p, w, b


def test_layout_matches_library(orc):
    from slam_gb300 import _native
    assert orc.cnn_layout()[2] == _native.load().odo_cnn_param_count()


def test_oracle_backward_against_finite_differences(orc):
    rng = np.random.default_rng(0)
    B = 2
    x = np.zeros((B, 120, 160, 8), np.float16)
    for c, (lo, hi) in enumerate([(0.5, 4.0), (0.0, 1.0), (0.5, 4.0), (0.0, 1.0)]):
        x[..., c] = rng.uniform(lo, hi, size=(B, 120, 160))
    xi = x.view(np.uint16)
    p, w, b = _params(orc, rng)
    lab = rng.normal(0, 0.05, (B, 6))
    A = rng.normal(size=(6, 6))
    sc = A @ A.T + np.eye(6)
    _, _, g = orc.cnn_run(p, xi, lab, sc, rounding=False)
    # a non-zero-channel weight of every layer and every bias
    idx = [w[0] + 2, w[1] + 20, w[2] + 77, w[3] + 301, w[4] + 999, w[5] + 5, w[6] + 4242, w[7] + 100,
           b[2], b[3], b[4], b[5], b[7]]
    checked = 0
    for i in idx:
        h = 1e-7 * max(1.0, abs(p[i]))  # small enough to cross few ReLU kinks
        pp = p.copy()
        pp[i] += h
        pm = p.copy()
        pm[i] -= h
        lp = orc.cnn_run(pp, xi, lab, sc, rounding=False, want_grad=False)[1]
        lm = orc.cnn_run(pm, xi, lab, sc, rounding=False, want_grad=False)[1]
        fd = (lp - lm) / (2 * h)
        if abs(fd) < 1e-8 and abs(g[i]) < 1e-8:
            continue  # inactive unit
        checked += 1
        assert abs(g[i] - fd) <= 2e-4 * abs(fd) + 1e-7, (i, g[i], fd)
    assert checked >= 8
