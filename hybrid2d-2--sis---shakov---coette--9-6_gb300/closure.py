"""Training data, training and use of the learned closure (hyb_mlp_*).

Samples come from the solver's own FP64 GPU runs of planar Couette cases over
the parameter ranges of the single large and batched workloads (Kn
log-uniform in [1e-3, 1], plate speed 0.05..0.8, wall-temperature ratio
0.8..1.5, 32..256 cells across):
* single runs that iterate with the synthetic solve and the distribution
  correction (32..128 cells, 24^2 velocities);
* FP64 batches of 256 instances of the batched workload's meshes and
  velocity grids (24^2, 32^2), advanced by the reference iteration through
  hyb_batch_step at five times that time step, about 0.5 M samples per
  batch from iterations 900..1200.
Snapshots are taken in the late phase of each run (300..600 for the single
runs), because the closure is used on near-steady states (the HoT of early
transients is one to two orders of magnitude larger and would swamp them).

The shipped weights come from 240 single runs (249 k samples).  Adding four
batches (2.2 M samples, --batches 4) lowers the held-out sample loss to
0.0036 but makes the closure solve worse on the converged held-out states
(field error 0.077 at Kn 0.12, against 0.036 with the NSF closure alone and
0.0085 with the shipped network): the batch states, advanced without the
synthetic solve, are not the near-steady states the closure is used on, so
the batches are off by default.
hyb_closure_samples returns the network inputs and the Convert_NS HoT
targets of every j-face; the channel is x-invariant, so one column of faces
is kept per snapshot.  Validation uses a held-out grid of Kn values that no
training case draws exactly.

    python -c "import __graft_entry__ as g; g.load_package(); \
               from hyb_gb300 import closure; closure.main()"

writes closure_weights.npz (weights, normalisation, loss history, sample
counts) next to this file unless --out says otherwise.
"""
import argparse
import math
import os
import time

import numpy as np

from . import abi, cases

HERE = os.path.dirname(os.path.abspath(__file__))
WEIGHTS = os.path.join(HERE, "closure_weights.npz")
HOLDOUT_KN = (0.002, 0.007, 0.03, 0.12, 0.5)
# synthetic solve of the data runs: LU-SGS inner solve with the distribution correction
GSIS = dict(max_inner=20, inner_tol=0.0, inner_rtol=1e-2, cfl=20.0, ns_solver=0, correct_f=1)


def data_cases(n, seed=20261204, kns=None):
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        ncy = int(rng.choice([32, 64, 128]))
        kn = float(kns[k]) if kns is not None else float(10 ** rng.uniform(-3.0, 0.0))
        out.append(cases.Case(name=f"closure-{k}", ncx=4, ncy=ncy, nvx=24, nvy=24, vmax=5.0, kn=kn,
                              uw=float(rng.uniform(0.05, 0.8)), t_bottom=1.0,
                              t_top=float(rng.uniform(0.8, 1.5)), dt=0.01 * 64.0 / ncy))
    return out


def run_case(case, iters=600, start=300, every=20):
    """Samples (x, y) of one run: one face column at every snapshot taken
    from iteration `start` on."""
    s = abi.Solver(case, precision=0)
    s.init_maxwellian()
    s.gsis(**GSIS)
    s.step(start, residual=False)
    xs, ys = [], []
    col = np.arange(case.ny) * (case.nx - 1)          # faces of column i = 1
    for _ in range((iters - start) // every + 1):
        x, y = s.closure_samples()
        xs.append(x[col])
        ys.append(y[col])
        s.step(every, residual=False)
    s.close()
    return np.concatenate(xs), np.concatenate(ys)


def generate(case_list, iters=600, start=300, every=20):
    xs, ys, failed = [], [], 0
    for c in case_list:
        try:
            x, y = run_case(c, iters, start, every)
        except abi.HybError:
            failed += 1
            continue
        if not _sane(x, y):
            failed += 1
            continue
        xs.append(x)
        ys.append(y)
    return np.concatenate(xs), np.concatenate(ys), failed


def batch_cases(n, seed):
    """Instances of the batched workload's ranges (4 x {32, 64, 128, 256}
    cells, 24^2 or 32^2 velocities, plate speed 0.05..0.8, wall-temperature
    ratio 0.8..1.5) with Kn log-uniform in [1e-3, 1]."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        ncy = int(rng.choice([32, 64, 128, 256]))
        nv = int(rng.choice([24, 32]))
        out.append(cases.Case(name=f"closure-batch-{seed}-{k}", ncx=4, ncy=ncy, nvx=nv, nvy=nv, vmax=5.0,
                              kn=float(10 ** rng.uniform(-3.0, 0.0)), uw=float(rng.uniform(0.05, 0.8)),
                              t_bottom=1.0, t_top=float(rng.uniform(0.8, 1.5)), dt=0.05 * 64.0 / ncy))
    return out


# a sample set is kept only when every value is finite and in the physical
# range of these channels (inputs within 1e3, HoT within 1e2 in NS units)
def _sane(x, y):
    return bool(np.isfinite(x).all() and np.isfinite(y).all() and np.abs(x).max() < 1e3 and np.abs(y).max() < 1e2)


def generate_batch(seed, n=256, iters=1200, start=900, every=20):
    """Samples of one FP64 batch of n instances (hyb_batch_*, the reference
    iteration at five times the time step of the synthetic-solve runs, so
    that the late phase is near-steady without the synthetic solve): one
    face column of every instance at every snapshot taken from iteration
    `start` on.  Instances with a value outside the physical range are
    dropped whole."""
    cl = batch_cases(n, seed)
    b = abi.Batch(cl, precision=0)
    b.init_maxwellian()
    b.step(start, residual=False)
    xs = [[] for _ in cl]
    ys = [[] for _ in cl]
    for _ in range((iters - start) // every + 1):
        for k, c in enumerate(cl):
            x, y = b.instance(k).closure_samples()
            col = np.arange(c.ny) * (c.nx - 1)
            xs[k].append(x[col])
            ys[k].append(y[col])
        b.step(every, residual=False)
    b.close()
    X, Y, failed = [], [], 0
    for k in range(len(cl)):
        x, y = np.concatenate(xs[k]), np.concatenate(ys[k])
        if _sane(x, y):
            X.append(x)
            Y.append(y)
        else:
            failed += 1
    return np.concatenate(X), np.concatenate(Y), failed


def norm_of(x, y):
    return x.mean(0), np.maximum(x.std(0), 1e-6), y.mean(0), np.maximum(y.std(0), 1e-9)


def val_loss(net, xv, yv, norm):
    p = net.predict(xv)
    return float(np.mean(((p - yv) / norm[3]) ** 2))


def fit(x, y, xv, yv, epochs=300, batch=8192, lr=1e-3, seed=0):
    """Adam on the GPU; returns the network, normalisation, per-epoch training
    loss, held-out loss every 10 epochs, device milliseconds of training."""
    net = abi.Mlp(seed=seed)
    norm = norm_of(x, y)
    net.set_norm(*norm)
    net.set_data(x, y)
    rng = np.random.default_rng(seed)
    hist, vhist, train_ms = [], [], 0.0
    for e in range(epochs):
        hist.append(net.train_epoch(rng.permutation(len(x)), batch=batch, lr=lr))
        train_ms += net.last_ms()
        if e % 10 == 9 or e == epochs - 1:
            vhist.append(val_loss(net, xv, yv, norm))
    return net, norm, np.array(hist), np.array(vhist), train_ms


def save(path, net, norm, **extra):
    np.savez(path, weights=net.params(), in_mean=norm[0], in_std=norm[1], out_mean=norm[2], out_std=norm[3],
             **extra)


def load(path=WEIGHTS, device=0):
    d = np.load(path)
    net = abi.Mlp(seed=0, device=device)
    net.set_params(d["weights"])
    net.set_norm(d["in_mean"], d["in_std"], d["out_mean"], d["out_std"])
    return net


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--cases", type=int, default=240)
    ap.add_argument("--iters", type=int, default=600)
    ap.add_argument("--start", type=int, default=300)
    ap.add_argument("--every", type=int, default=20)
    ap.add_argument("--batches", type=int, default=0,
                    help="add FP64 batches of 256 instances (about 0.5 M samples each; see the module notes)")
    ap.add_argument("--epochs", type=int, default=300)
    ap.add_argument("--out", default=WEIGHTS)
    a = ap.parse_args(argv)
    t0 = time.perf_counter()
    x, y, nf = generate(data_cases(a.cases), a.iters, a.start, a.every)
    n_gsis = len(x)
    for k in range(a.batches):
        xb, yb, fb = generate_batch(20261205 + k, every=a.every)
        x, y, nf = np.concatenate([x, xb]), np.concatenate([y, yb]), nf + fb
    xv, yv, nfv = generate(data_cases(len(HOLDOUT_KN), seed=7, kns=HOLDOUT_KN), a.iters, a.start, a.every)
    t_data = time.perf_counter() - t0
    net, norm, hist, vhist, train_ms = fit(x, y, xv, yv, epochs=a.epochs)
    flops = 6.0 * 9156 * len(x) * a.epochs          # forward + backward, 2 flops per multiply-add
    save(a.out, net, norm, loss=hist, val_loss=vhist, n_train=len(x), n_train_gsis=n_gsis, n_val=len(xv),
         failed=nf + nfv, data_s=t_data, train_ms=train_ms,
         train_steps=a.epochs * math.ceil(len(x) / 8192), train_tflops=flops / (train_ms / 1000.0) / 1e12)
    print(f"samples {len(x)} train ({n_gsis} from synthetic-solve runs) / {len(xv)} held-out, "
          f"failed runs {nf + nfv}, data {t_data:.1f}s; "
          f"loss {hist[0]:.4g} -> {hist[-1]:.4g}, held-out {vhist[-1]:.4g}; "
          f"train {train_ms / 1000:.2f}s device ({flops / (train_ms / 1000) / 1e12:.3f} TFLOP/s)")
    return 0
