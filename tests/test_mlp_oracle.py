"""The CPU restatement of the learned-closure network: its gradient against
central finite differences (float64 mode), its BF16 rounding, and the
parameter count of the architecture."""
import numpy as np

from oracle import mlp_oracle as M


def test_param_count():
    assert M.NPARAM == 9156


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(1)
    w = M.glorot(3)
    x = rng.standard_normal((37, 8))
    y = rng.standard_normal((37, 4))
    norm = (rng.uniform(-1, 1, 8), rng.uniform(0.5, 2, 8), rng.uniform(-1, 1, 4), rng.uniform(0.5, 2, 4))
    _, g = M.loss_and_grad(w, x, y, norm, quantize=False)
    for i in rng.choice(M.NPARAM, 60, replace=False):
        e = np.zeros_like(w)
        e[i] = 1e-6
        fd = (M.loss_and_grad(w + e, x, y, norm, False)[0] - M.loss_and_grad(w - e, x, y, norm, False)[0]) / 2e-6
        assert abs(fd - g[i]) <= 1e-8 + 1e-6 * abs(g[i]), i


def test_bf16_rounding_is_nearest_even():
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.5, 3.14159265, 1e-40])
    r = M.bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2 ** -6
    assert r[3] == -2.5 and r[4] == 3.140625
    # quantised and exact networks differ only by the rounding of operands
    rng = np.random.default_rng(2)
    w = M.glorot(4)
    x = rng.standard_normal((20, 8))
    norm = (np.zeros(8), np.ones(8), np.zeros(4), np.ones(4))
    ya, _ = M.forward(w, x, norm, quantize=False)
    yq, _ = M.forward(w, x, norm, quantize=True)
    assert np.abs(ya - yq).max() < 0.05 * np.abs(ya).max()
