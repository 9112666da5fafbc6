"""Learned resonance proposal (no counterpart in the reference; the plain search it
accelerates is examples/roots_newton_polygon_rsvd.cpp:172-265 and its Newton step
source/utilities/find_roots.cpp:117-217).

A small MLP (34 -> 4 x 512 GELU -> 128, BF16 products with FP32 accumulation on the
GPU, see csrc/mlp.cu) maps a scatterer, its inner refraction index and the start of
a k-window to log10 sigma_min(k) at 128 points across the window.  The local minima
of the predicted curve become candidate brackets; every candidate is confirmed by
safeguarded Newton on sigma_min' with sigma_min'' (hbem_refine_brackets), so each
reported resonance is verified exactly like the plain search's.  The plain sweep on
a dense grid stays the fallback and the judge of recall.

Scatterer family: Fourier-sum radius r(t) = s (1 + sum_{m=1..8} a_m cos mt + b_m sin mt),
a_m, b_m ~ N(0, 0.05/m) (redrawn if min r < 0.3 s), s = 0.25, sampled into N = 50
line panels; c_i ~ U[2, 25], c_o = 1; windows [k0, k0 + 2], k0 ~ U[0.5, 8].  The
scale and panel count match the circle of the plain benchmark (radius 0.25, N = 50,
k in [0.5, 10]), so that T(k) is of order 100 and every label is a dense sigma_min.
"""
import math
import time

import numpy as np

from . import api, geometry

FAMILY = dict(scale=0.25, N=50, order=11, c_o=1.0, c_lo=2.0, c_hi=25.0, k_lo=0.5, k_hi=8.0, width=2.0, npts=128,
              modes=8)
N_IN, WIDTH, DEPTH, N_OUT = 34, 512, 4, 128


def draw(seed):
    """(a, b, c_i, k0) of scatterer `seed`."""
    a, b = geometry.random_fourier_coeffs(seed, modes=FAMILY["modes"])
    rng = np.random.default_rng(seed + 10_000_000)
    c_i = float(rng.uniform(FAMILY["c_lo"], FAMILY["c_hi"]))
    k0 = float(rng.uniform(FAMILY["k_lo"], FAMILY["k_hi"]))
    return a, b, c_i, k0


def mesh(a, b):
    kinds, par = geometry.fourier_curve(a, b, FAMILY["N"])
    par = par.copy()
    par[:, :4] *= FAMILY["scale"]
    return kinds, par


def features(a, b, c_i, k0):
    """34 inputs: a_1..a_16, b_1..b_16 (x 20; modes above 8 are zero in this family),
    c_i / 25, k0 / 10."""
    x = np.zeros(N_IN, np.float32)
    x[:len(a)] = 20.0 * np.asarray(a)
    x[16:16 + len(b)] = 20.0 * np.asarray(b)
    x[32] = c_i / 25.0
    x[33] = k0 / 10.0
    return x


def window(k0):
    return k0 + FAMILY["width"] * np.arange(FAMILY["npts"]) / (FAMILY["npts"] - 1)


def operator(a, b):
    return api.SolutionsOperator(api.BuilderData(mesh(a, b), order=FAMILY["order"]))


def dataset(seeds):
    """Features and labels log10 sigma_min(k) on the window (dense sigma on the GPU)."""
    X = np.zeros((len(seeds), N_IN), np.float32)
    Y = np.zeros((len(seeds), N_OUT), np.float32)
    for r, s in enumerate(seeds):
        a, b, c_i, k0 = draw(s)
        so = operator(a, b)
        sig = so.sweep_sigma(window(k0), FAMILY["c_o"], c_i, d=0)[:, 0]
        X[r] = features(a, b, c_i, k0)
        Y[r] = np.log10(np.maximum(sig, 1e-300))
    return X, Y


def train(X, Y, epochs=60, batch=256, lr=1e-3, seed=0, net=None, log=None):
    """Adam with a cosine learning-rate decay over shuffled mini-batches."""
    net = net or api.MLP(N_IN, WIDTH, DEPTH, N_OUT, seed=seed)
    rng = np.random.default_rng(seed)
    n = X.shape[0]
    steps = epochs * max(1, n // batch)
    step = 0
    losses = []
    for ep in range(epochs):
        perm = rng.permutation(n)
        for j in range(0, n - batch + 1, batch):
            idx = perm[j:j + batch]
            rate = lr * 0.5 * (1.0 + math.cos(math.pi * step / steps))
            losses.append(net.train_step(X[idx], Y[idx], rate))
            step += 1
        if log:
            log(ep, float(np.mean(losses[-max(1, n // batch):])))
    return net, losses


def local_minima(curve):
    c = np.asarray(curve)
    return [j for j in range(1, c.size - 1) if c[j] < c[j - 1] and c[j] <= c[j + 1]]


def propose(net, cases):
    """Candidate brackets per case (a, b, c_i, k0): the predicted curve's local minima,
    each bracketed by +-2 grid steps."""
    X = np.stack([features(*c) for c in cases])
    pred = net.forward(X)
    h = FAMILY["width"] / (FAMILY["npts"] - 1)
    out = []
    for c, p in zip(cases, pred):
        ks = window(c[3])
        mins = local_minima(p)
        out.append((np.array([ks[j] - 2 * h for j in mins]), np.array([ks[j] + 2 * h for j in mins])))
    return out, pred


def evaluate(net, seeds, plain_points=210, tol=1e-8, match=1e-6):
    """Plain search (plain_points-point grid on each window, Newton from every bracketed
    minimum) against the learned proposal (+ Newton from its brackets) on the same
    windows: counts, recall, roots outside the plain set, evaluations and times."""
    import torch
    cases = [draw(s) for s in seeds]
    ops = [operator(a, b) for (a, b, _, _) in cases]
    c_o = FAMILY["c_o"]
    for so, (a, b, c_i, k0) in zip(ops[:1], cases[:1]):      # warm-up
        so.find_resonances_plain(k0, k0 + FAMILY["width"], plain_points, c_o, c_i, tol=tol)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    plain, plain_evals = [], 0
    for so, (a, b, c_i, k0) in zip(ops, cases):
        r, _, ne = so.find_resonances_plain(k0, k0 + FAMILY["width"], plain_points, c_o, c_i, tol=tol)
        plain.append(r)
        plain_evals += ne
    torch.cuda.synchronize()
    t_plain = time.perf_counter() - t0
    t0 = time.perf_counter()
    brackets, _ = propose(net, cases)
    learned, learned_evals = [], 0
    for so, (a, b, c_i, k0), (lo, hi) in zip(ops, cases, brackets):
        r, ne = so.refine_brackets(lo, hi, c_o, c_i, tol=tol)
        learned.append(r)
        learned_evals += ne
    torch.cuda.synchronize()
    t_learned = time.perf_counter() - t0
    n_plain = sum(r.size for r in plain)
    n_learned = sum(r.size for r in learned)
    found = sum(int(np.sum([np.min(np.abs(l - p)) <= match if l.size else False for p in pr]))
                for pr, l in zip(plain, learned))
    extra = sum(int(np.sum([np.min(np.abs(pr - x)) > match if pr.size else True for x in l]))
                for pr, l in zip(plain, learned))
    return {"windows": len(seeds), "plain_roots": n_plain, "learned_roots": n_learned,
            "recall": found / n_plain if n_plain else None, "learned_not_in_plain": extra,
            "plain_evals": plain_evals, "learned_evals": learned_evals,
            "plain_seconds": t_plain, "learned_seconds": t_learned,
            "plain_res_per_s": n_plain / t_plain, "learned_res_per_s": n_learned / t_learned}


def save(net, path):
    np.savez_compressed(path, params=net.get_params(), dims=np.array(net.dims))


def load(path):
    d = np.load(path)
    dims = [int(v) for v in d["dims"]]
    net = api.MLP(dims[0], dims[1], len(dims) - 2, dims[-1])
    net.set_params(d["params"])
    return net


if __name__ == "__main__":
    import argparse
    import json
    ap = argparse.ArgumentParser(description="generate the training windows, train the proposal network, save it")
    ap.add_argument("--train", type=int, default=4000, help="training scatterers (seeds 10000..)")
    ap.add_argument("--test", type=int, default=200, help="held-out scatterers (seeds 20000..)")
    ap.add_argument("--epochs", type=int, default=60)
    ap.add_argument("--out", default="proposal_mlp.npz")
    ap.add_argument("--data", default=None, help="npz with X, Y, Xt, Yt to reuse")
    ap.add_argument("--eval", type=int, default=0, help="held-out windows for the plain-versus-learned comparison")
    args = ap.parse_args()
    t0 = time.perf_counter()
    if args.data:
        d = np.load(args.data)
        X, Y, Xt, Yt = d["X"], d["Y"], d["Xt"], d["Yt"]
    else:
        X, Y = dataset(list(range(10000, 10000 + args.train)))
        Xt, Yt = dataset(list(range(20000, 20000 + args.test)))
        np.savez_compressed(args.out.replace(".npz", "_data.npz"), X=X, Y=Y, Xt=Xt, Yt=Yt)
    t1 = time.perf_counter()
    net, losses = train(X, Y, epochs=args.epochs, log=lambda e, l: print("epoch", e, "loss", l, flush=True))
    t2 = time.perf_counter()
    test_mse = float(np.mean((net.forward(Xt) - Yt) ** 2))
    save(net, args.out)
    out = {"data_seconds": t1 - t0, "train_seconds": t2 - t1, "final_train_loss": losses[-1],
           "test_mse_log10": test_mse}
    if args.eval:
        out["evaluation"] = evaluate(net, list(range(20000, 20000 + args.eval)))
    print(json.dumps(out))
