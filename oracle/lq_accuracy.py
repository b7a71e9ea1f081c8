"""Accuracy reachable by the learned near-singular quadrature's network --
TEST INFRASTRUCTURE ONLY (a CPU experiment with the float64 reference network
of oracle/lq.py; the product never imports it).

Trains the 14 -> 256 -> 256 -> 256 -> 16 network (bf16 weights) with Adam and
a cosine learning-rate schedule on seeded labels of the reference's 64 x 64
fallback rule, with targets standardised per output, and prints the held-out
relative error per pair (|Y - T| / |T| over the 16 outputs).  Then, on the
near-singular pairs of cubed spheres (4 and 8 quadrangles per face), it
compares the network and the plain 12 x 12 rule against the 64 x 64 rule.

    python -m oracle.lq_accuracy [training pairs] [steps] [uniform | mesh]

(mesh: training pairs from lq.sample_mesh_pairs, placed as a surface mesh
places its near-singular pairs).
"""
import sys
import time

import numpy as np

from oracle import lq


def data(n, seed, sampler="uniform"):
    c, rt, k = (lq.sample_mesh_pairs if sampler == "mesh" else lq.sample_pairs)(n, seed)
    X, h = lq.features(c, rt, k)
    return X, lq.targets(lq.labels(c, rt, k, 3), h)


def run(ntr=20480, steps=3000, batch=512, lr0=1e-3, seed=3, sampler="uniform"):
    X, T = data(ntr, 4, sampler)
    Xv, Tv = data(2048, 5, sampler)
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
    return np.quantile(rel, [0.5, 0.9, 1.0]), np.linalg.norm(Y - Tv) / np.linalg.norm(Tv), (flat, mu, sd)


def sphere_near_pairs(nface=4, radius=1.0, n_in=1.5, lambda0=1.0, n_host=1.33):
    """(node, quadrangle) pairs of a cubed sphere's exterior domain on which
    the 12 x 12 and the 64 x 64 rules differ by more than 1e-6 (relative):
    the near-singular pairs the fallback rule integrates.  Returns corners,
    rt, k of those pairs."""
    import os
    import tempfile
    from bem3_emf_b2_gb300 import meshgen
    from oracle import port
    wd = tempfile.mkdtemp()
    nodes, elems = meshgen.cubed_sphere(nface, radius)
    meshgen.write_mesh(os.path.join(wd, "mesh.msh"), nodes, elems)
    o = port.Obj(os.path.join(wd, "mesh.msh"), [n_in], lambda0, n_host)
    sid = o.sids[0]
    P = [(sid[t], tn, sid[s]) for t in range(1, len(sid)) for tn in range(4) for s in range(1, len(sid)) if s != t]
    c = np.array([o.corner[e] for _, _, e in P])
    rt = np.array([o.ren[td, tn] for td, tn, _ in P])
    k = np.full(len(P), o.kn[0])
    gl, gh = lq.labels(c, rt, k, 2), lq.labels(c, rt, k, 3)
    near = np.linalg.norm(gl - gh, axis=1) > 1e-6 * np.linalg.norm(gh, axis=1)
    return c[near], rt[near], k[near]


def compare_on_sphere(model, nface=4):
    """relative error quantiles (median, 90 %, max), against the 64 x 64 rule,
    of the network and of the 12 x 12 rule on a cubed sphere's near-singular
    pairs"""
    flat, mu, sd = model
    c, rt, k = sphere_near_pairs(nface)
    X, h = lq.features(c, rt, k)
    gh = lq.labels(c, rt, k, 3)
    gl = lq.labels(c, rt, k, 2)
    Y, _ = lq.mlp_forward(lq.unpack(flat.astype(np.float32)), X)
    net = lq.untarget(Y * sd + mu, h)
    nrm = np.linalg.norm(gh, axis=1)
    q = [0.5, 0.9, 1.0]
    return (len(c), np.quantile(np.linalg.norm(net - gh, axis=1) / nrm, q),
            np.quantile(np.linalg.norm(gl - gh, axis=1) / nrm, q))


if __name__ == "__main__":
    ntr = int(sys.argv[1]) if len(sys.argv) > 1 else 20480
    steps = int(sys.argv[2]) if len(sys.argv) > 2 else 3000
    sampler = sys.argv[3] if len(sys.argv) > 3 else "uniform"
    t0 = time.time()
    q, tot, model = run(ntr, steps, sampler=sampler)
    print("%s pairs %d steps %d (%.0f s): held-out relative error per pair median %.3g, 90%% %.3g, max %.3g; overall %.3g"
          % (sampler, ntr, steps, time.time() - t0, q[0], q[1], q[2], tot))
    for nface in (4, 8):
        n, e_net, e_gl = compare_on_sphere(model, nface)
        print("cubed sphere %d x %d per face: %d near-singular pairs; error against the 64 x 64 rule "
              "(median, 90%%, max): network %.3g %.3g %.3g, 12 x 12 rule %.3g %.3g %.3g"
              % ((nface, nface, n) + tuple(e_net) + tuple(e_gl)))
