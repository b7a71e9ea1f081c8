"""Accuracy reachable by the learned near-singular quadrature's network --
TEST INFRASTRUCTURE ONLY (a CPU experiment with the float64 reference network
of oracle/lq.py; the product never imports it).

Trains the 14 -> 256 -> 256 -> 256 -> 16 network (bf16 weights) with Adam and
a cosine learning-rate schedule on seeded labels of the reference's 64 x 64
fallback rule, with targets standardised per output, and prints the held-out
relative error per pair (|Y - T| / |T| over the 16 outputs).

    python -m oracle.lq_accuracy [training pairs] [steps]
"""
import sys
import time

import numpy as np

from oracle import lq


def data(n, seed):
    c, rt, k = lq.sample_pairs(n, seed)
    X, h = lq.features(c, rt, k)
    return X, lq.targets(lq.labels(c, rt, k, 3), h)


def run(ntr=20480, steps=3000, batch=512, lr0=1e-3, seed=3):
    X, T = data(ntr, 4)
    Xv, Tv = data(2048, 5)
    mu, sd = T.mean(0), T.std(0)
    Tn = (T - mu) / sd
    flat = lq.pack(lq.init_params(seed)).astype(np.float64)
    m1 = np.zeros_like(flat)
    m2 = np.zeros_like(flat)
    nb = ntr // batch
    for s in range(steps):
        r0 = (s % nb) * batch
        lr = lr0 * 0.5 * (1.0 + np.cos(np.pi * s / steps))
        _, g = lq.mlp_loss_grad(lq.unpack(flat.astype(np.float32)), X[r0:r0 + batch], Tn[r0:r0 + batch])
        g = np.concatenate([np.concatenate([a.ravel(), b]) for a, b in g])
        m1 = 0.9 * m1 + 0.1 * g
        m2 = 0.999 * m2 + 0.001 * g * g
        flat -= lr * (m1 / (1 - 0.9 ** (s + 1))) / (np.sqrt(m2 / (1 - 0.999 ** (s + 1))) + 1e-8)
    Y, _ = lq.mlp_forward(lq.unpack(flat.astype(np.float32)), Xv)
    Y = Y * sd + mu
    rel = np.linalg.norm(Y - Tv, axis=1) / np.linalg.norm(Tv, axis=1)
    return np.quantile(rel, [0.5, 0.9, 1.0]), np.linalg.norm(Y - Tv) / np.linalg.norm(Tv)


if __name__ == "__main__":
    ntr = int(sys.argv[1]) if len(sys.argv) > 1 else 20480
    steps = int(sys.argv[2]) if len(sys.argv) > 2 else 3000
    t0 = time.time()
    q, tot = run(ntr, steps)
    print("pairs %d steps %d (%.0f s): held-out relative error per pair median %.3g, 90%% %.3g, max %.3g; overall %.3g"
          % (ntr, steps, time.time() - t0, q[0], q[1], q[2], tot))
