"""CPU: training data and reference network of the learned near-singular
quadrature (oracle/lq.py, oracle/port/bem_port.c port_quad_labels_c).

The labels are pinned to the reference's own outputs: every off-diagonal
(node, quadrangle) entry of the golden G_0, H_0 (produced by the reference,
tests/golden) equals either the 12 x 12 rule or the 64 x 64 fallback rule of
port_quad_labels_c, and the fallback rule is the one that matches where the
two differ (the near-singular pairs the network is to replace)."""
import os

import numpy as np
import pytest

from oracle import lq, port
from tests._scenes import load_case, write_inputs


@pytest.mark.parametrize("case", ["sphere2", "cube1"])
def test_labels_match_the_reference_fallback(case, tmp_path):
    meta, gold = load_case(case)
    wd = str(tmp_path)
    write_inputs(meta, wd)
    o = port.Obj(os.path.join(wd, "mesh.msh"), [complex(a, b) for a, b in meta["n"]], meta["wave"]["lambda0"],
                 meta["wave"]["ni"])
    sid = o.sids[0]
    rows, pairs = [], []
    for t in range(1, len(sid)):
        for tn in range(4):
            for s in range(1, len(sid)):
                if s != t:
                    rows.append((t - 1) * 4 + tn)
                    pairs.append((sid[t], tn, sid[s], s))
    corners = np.array([o.corner[e] for _, _, e, _ in pairs])
    rt = np.array([o.ren[td, tn] for td, tn, _, _ in pairs])
    k = np.full(len(pairs), o.kn[0])
    gl, gh = lq.labels(corners, rt, k, 2), lq.labels(corners, rt, k, 3)
    ref = np.zeros_like(gl)
    for q, (row, (_, _, _, s)) in enumerate(zip(rows, pairs)):
        g = gold["G_0"][row, 4 * (s - 1):4 * s]
        h = gold["H_0"][row, 4 * (s - 1):4 * s]
        ref[q] = np.stack([np.concatenate([g, h]).real, np.concatenate([g, h]).imag], 1).ravel()
    scale = np.linalg.norm(ref, axis=1)
    e_gl = np.linalg.norm(gl - ref, axis=1) / scale
    e_gh = np.linalg.norm(gh - ref, axis=1) / scale
    assert np.all(np.minimum(e_gl, e_gh) <= 1e-10), np.minimum(e_gl, e_gh).max()
    fallback = e_gh <= 1e-10
    differ = np.linalg.norm(gl - gh, axis=1) / scale > 1e-6
    assert (fallback & differ).sum() > 0, "no near-singular pair in the case"
    # where the reference used the fallback and the rules differ, the GL rule is wrong
    assert np.all(e_gl[fallback & differ] > 1e-8)


def test_pairs_and_features_are_invariant():
    c, rt, k = lq.sample_pairs(300, 11)
    X, h = lq.features(c, rt, k)
    T = lq.targets(lq.labels(c, rt, k, 3), h)
    assert X.shape == (300, 14) and T.shape == (300, 16)
    d = np.linalg.norm(rt - c.mean(1), axis=1) / h
    assert d.min() >= 0.0 and d.max() <= 3.0
    rng = np.random.default_rng(3)
    q = rng.standard_normal((1, 4))
    R = lq._quat_to_rot(q / np.linalg.norm(q))[0]
    s, sh = 0.37, np.array([1.0, -4.0, 2.5])
    X2, h2 = lq.features((c @ R.T) * s + sh, (rt @ R.T) * s + sh, k / s)
    T2 = lq.targets(lq.labels((c @ R.T) * s + sh, (rt @ R.T) * s + sh, k / s, 3), h2)
    assert np.abs(X2 - X).max() <= 1e-12
    assert np.abs(T2 - T).max() <= 1e-11 * np.abs(T).max()


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.5e-3, 3.0e38], np.float32)
    r = lq.bf16_round(x)
    assert r[0] == 1.0 and r[1] == 1.0  # tie to even
    assert r[2] == np.float32(1.0 + 4 * 2 ** -8)
    assert np.all(np.abs(r - x) <= np.abs(x) * 2 ** -8)


def test_reference_network_gradient_by_finite_differences():
    widths = (14, 12, 9, 16)
    ps = [(W.astype(np.float64), b.astype(np.float64) + 0.1) for W, b in lq.init_params(2, widths)]
    rng = np.random.default_rng(4)
    X = rng.standard_normal((7, 14))
    T = rng.standard_normal((7, 16))
    loss, grads = lq.mlp_loss_grad(ps, X, T, quant=False)
    eps = 1e-6
    for li in range(len(ps)):
        for which in (0, 1):
            P = ps[li][which]
            for idx in [tuple(rng.integers(0, s) for s in P.shape) for _ in range(4)]:
                old = P[idx]
                P[idx] = old + eps
                lp, _ = lq.mlp_loss_grad(ps, X, T, quant=False)
                P[idx] = old - eps
                lm, _ = lq.mlp_loss_grad(ps, X, T, quant=False)
                P[idx] = old
                fd = (lp - lm) / (2 * eps)
                assert abs(fd - grads[li][which][idx]) <= 1e-7 * max(1.0, abs(fd)), (li, which, idx)


def test_bar_for_a_learned_rule_on_sphere_pairs():
    """The bar a learned replacement of the 64 x 64 fallback rule has to
    beat: on a cubed sphere's near-singular pairs (the rules differ by more
    than 1e-6) the plain 12 x 12 rule stays within 1e-3 of the 64 x 64 rule
    (relative, per pair over G_p, H_p)."""
    from oracle import lq_accuracy
    c, rt, k = lq_accuracy.sphere_near_pairs(3)
    gl, gh = lq.labels(c, rt, k, 2), lq.labels(c, rt, k, 3)
    e = np.linalg.norm(gl - gh, axis=1) / np.linalg.norm(gh, axis=1)
    assert len(c) > 100
    assert e.max() <= 1e-3, e.max()


def test_mesh_like_pairs():
    """lq.sample_mesh_pairs: the observation point is a neighbouring
    quadrangle's collocation node -- off the element, within about two
    element sizes of its centre -- and, like the sphere's near-singular
    pairs, mostly integrated to better than 1e-3 by the 12 x 12 rule."""
    c, rt, k = lq.sample_mesh_pairs(400, 21)
    X, h = lq.features(c, rt, k)
    d = np.linalg.norm(rt - c.mean(1), axis=1) / h
    assert d.min() > 0.5 and d.max() < 2.5, (d.min(), d.max())
    gl, gh = lq.labels(c, rt, k, 2), lq.labels(c, rt, k, 3)
    e = np.linalg.norm(gl - gh, axis=1) / np.linalg.norm(gh, axis=1)
    assert np.quantile(e, 0.9) < 1e-3
