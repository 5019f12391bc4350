"""GPU kernels of the learned closure against the CPU restatement
(oracle/mlp_oracle.py, same BF16 operand rounding, float64 accumulation).

Gradient check: the GPU gradient (tensor-core products, FP32 accumulation)
matches the restatement to 2e-3 in relative L2 norm and the loss to 1e-4;
forward outputs agree to 1e-3 of their scale.  Training lowers the loss on a
smooth synthetic target and is deterministic.
"""
import numpy as np
import pytest

from oracle import mlp_oracle as M

pytestmark = pytest.mark.gpu


def _net(seed=7):
    from hyb_gb300 import abi
    net = abi.Mlp(seed=0)
    w = M.glorot(seed).astype(np.float32)
    net.set_params(w)
    return net, w.astype(np.float64)


def _norm(rng):
    return (rng.uniform(-1, 1, 8), rng.uniform(0.5, 2, 8), rng.uniform(-1, 1, 4), rng.uniform(0.5, 2, 4))


@pytest.mark.parametrize("n", [128, 300, 8192])
def test_gradient_matches_cpu_restatement(pkg, n):
    rng = np.random.default_rng(n)
    net, w = _net()
    norm = _norm(rng)
    net.set_norm(*norm)
    x = rng.standard_normal((n, 8)).astype(np.float32) * norm[1] + norm[0]
    y = rng.standard_normal((n, 4)).astype(np.float32)
    lg, gg = net.grad(x, y)
    lo, go = M.loss_and_grad(w, x, y, tuple(np.asarray(v, np.float32) for v in norm), quantize=True)
    assert abs(lg - lo) <= 1e-4 * abs(lo), (lg, lo)
    rel = np.linalg.norm(gg - go) / np.linalg.norm(go)
    assert rel < 2e-3, rel
    for name, sl in _slices().items():
        r = np.linalg.norm(gg[sl] - go[sl]) / max(np.linalg.norm(go[sl]), 1e-30)
        assert r < 1e-2, (name, r)


def _slices():
    out, o = {}, 0
    for name, shp in M.SHAPES:
        k = int(np.prod(shp))
        out[name] = slice(o, o + k)
        o += k
    return out


def test_forward_matches_cpu_restatement(pkg):
    rng = np.random.default_rng(3)
    net, w = _net(11)
    norm = _norm(rng)
    net.set_norm(*norm)
    x = (rng.standard_normal((1000, 8)) * norm[1] + norm[0]).astype(np.float32)
    yg = net.predict(x)
    yn, _ = M.forward(w, x, tuple(np.asarray(v, np.float32) for v in norm), quantize=True)
    yo = yn * np.asarray(norm[3], np.float32) + np.asarray(norm[2], np.float32)
    assert np.abs(yg - yo).max() < 1e-3 * np.abs(yo).max()


def test_adam_steps_match_cpu_restatement(pkg):
    """Three Adam steps of one full batch each: the GPU's FP32 master weights
    after every step against the restatement's update from the same
    gradient (the network's own, read back with hyb_mlp_grad; the training
    step reduces the same tiles in the same order).  The bias corrections
    and first and second moments carry over the steps."""
    rng = np.random.default_rng(21)
    net, w = _net(13)
    norm = _norm(rng)
    net.set_norm(*norm)
    n, lr = 3000, 1e-3
    x = (rng.standard_normal((n, 8)) * norm[1] + norm[0]).astype(np.float32)
    y = rng.standard_normal((n, 4)).astype(np.float32)
    net.set_data(x, y)
    wc = w.astype(np.float32)
    m1 = np.zeros_like(wc)
    m2 = np.zeros_like(wc)
    for t in (1, 2, 3):
        _, g = net.grad(x, y)
        net.train_epoch(np.arange(n), batch=n, lr=lr)
        wc, m1, m2 = M.adam_step(wc, m1, m2, g, t, lr)
        wg = net.params()
        # FP32 rounding of the update (about lr) and of the weight itself
        tol = 1e-5 * lr + 2.0 * np.spacing(np.abs(wc))
        assert np.all(np.abs(wg - wc) <= tol), (t, np.abs(wg - wc).max())
        assert np.abs(wg - w).max() > 0.5 * lr          # the weights did move


def test_training_lowers_loss_and_is_deterministic(pkg):
    rng = np.random.default_rng(5)
    x = rng.uniform(-1, 1, (40000, 8)).astype(np.float32)
    y = np.stack([np.sin(x[:, 0] + x[:, 1]), x[:, 2] * x[:, 3], np.tanh(2 * x[:, 4]), x[:, 5] ** 2 - x[:, 6]],
                 1).astype(np.float32)
    norm = (x.mean(0), x.std(0), y.mean(0), y.std(0))
    runs = []
    for _ in range(2):
        net, _w = _net(1)
        net.set_norm(*norm)
        net.set_data(x, y)
        prng = np.random.default_rng(9)
        losses = [net.train_epoch(prng.permutation(len(x)), batch=8192, lr=1e-3) for _ in range(60)]
        runs.append((losses, net.params()))
    losses = runs[0][0]
    assert losses[-1] < 0.1 * losses[0], losses
    assert np.array_equal(runs[0][1], runs[1][1])
