"""CPU: the adaptive order's rules for far triangle pairs (the double-float
quadrature's reg_order, csrc/gb_quad_df.cuh) restated in numpy FP64 on
seeded random triangles at the tier boundaries, against the reference's
three sub-quadrangle map with a 40-point rule: the kernel values G, H, the
derivative sets and F, each times the three shape-function monomials, stay
within 1e-12 of the kernel's natural scale (sum of |kernel| x weight, the
scale the tiers were calibrated on).

Tiers checked (ka = |k| a, a = |c1| + |c2|, D = |R0| / a): the conical
product rule of n x n points for D >= 3 and ka <= 3.6 (n = 5 for ka <= 0.6
and D >= 8, 6 for ka <= 1.2 and D >= 5, 7 for ka <= 2.4, else 8), and the
sub-quadrangle rules of the nearer or faster-varying pairs."""
import numpy as np
import pytest
from numpy.polynomial.legendre import leggauss
from scipy.special import roots_jacobi

S3 = np.sqrt(3.0)


def subquad(n):
    x, w = leggauss(n)
    X, Y = [a.ravel() for a in np.meshgrid(x, x, indexing="ij")]
    W = np.outer(w, w).ravel() * (1 + 0.25 * X + 0.25 * Y)
    zs = [0.125 * (3 + 2 * X + 2 * Y + X * Y), 0.0625 * (-3 + X - 5 * Y - X * Y), 0.0625 * (-3 - 5 * X + Y - X * Y)]
    es = [0.125 * S3 * (-X + Y), 0.0625 * S3 * (3 + 3 * X + Y + X * Y), 0.0625 * S3 * (-3 - X - 3 * Y - X * Y)]
    return np.concatenate(zs), np.concatenate(es), np.concatenate([W] * 3)


def conical(n):
    xj, wj = roots_jacobi(n, 0.0, 1.0)
    xl, wl = leggauss(n)
    s, t = (1 + xj) / 2, (1 + xl) / 2
    S, T = [a.ravel() for a in np.meshgrid(s, t, indexing="ij")]
    W = 24.0 * np.outer(wj / 4, wl / 2).ravel()
    return 1 - 1.5 * S, S3 * S * (0.5 - T), W


def order(D, ka):
    """the tier table for a triangle: ('c', n) conical or ('s', n) sub-quadrangles"""
    if D >= 3.0 and ka <= 3.6:
        return ("c", 5 if (ka <= 0.6 and D >= 8.0) else (6 if (ka <= 1.2 and D >= 5.0) else (7 if ka <= 2.4 else 8)))
    nD = 12 if D < 2.0 else (9 if D < 3.0 else (6 if D < 5.0 else 5))
    nk = 5 if ka <= 1.2 else (6 if ka <= 2.4 else (8 if ka <= 4.5 else 12))
    return ("s", min(max(nD, nk), 12))


REF = subquad(40)


def integrals(rule, c1, c2, n, rt, k, v):
    Z, E, W = rule
    r = Z[:, None] * c1 + E[:, None] * c2
    R = r - rt
    aR = np.linalg.norm(R, axis=1)
    ph = np.exp(1j * k * aR)
    cb = 1j * k * aR - 1
    rdW = (R @ n) / aR
    rdv = (R @ v) / aR
    K = [ph / aR, cb * ph * rdW / aR ** 2, cb * ph * rdv / aR ** 2,
         ph * ((k * aR) ** 2 + 3 * cb) * rdv * rdW / aR ** 3 - cb * ph * (n @ v) / aR ** 3, rdW / aR ** 2 + 0j]
    N = [np.ones_like(Z), Z, E]
    vals = np.array([np.sum(W * Ki * Nj) for Ki in K for Nj in N])
    scl = np.array([np.sum(W * np.abs(Ki)) for Ki in K for Nj in N])  # the kernel's natural scale
    return vals, scl


@pytest.mark.parametrize("ka,D", [(0.6, 8.0), (0.6, 5.0), (1.2, 5.0), (0.6, 3.0), (2.4, 3.0), (3.6, 3.0),
                                  (4.0, 3.0), (1.2, 2.5), (0.5, 1.5)])
def test_triangle_tiers_within_1e12(ka, D):
    rng = np.random.default_rng(int(ka * 100 + D * 10))
    kind, nq = order(D, ka)
    rule = conical(nq) if kind == "c" else subquad(nq)
    worst = 0.0
    for _ in range(12):
        c1 = rng.normal(size=3)
        c1 /= np.linalg.norm(c1)
        c2 = rng.normal(size=3)
        c2 -= c2.dot(c1) * c1
        c2 /= np.linalg.norm(c2)
        c2 = rng.uniform(0.6, 1.0) * c2 + rng.uniform(-0.4, 0.4) * c1
        a = np.linalg.norm(c1) + np.linalg.norm(c2)
        n = np.cross(c1, c2)
        n /= np.linalg.norm(n)
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        rt = D * a * d
        k = ka / a * np.exp(1j * rng.uniform(0, 0.05))
        v = rng.normal(size=3)
        v -= v.dot(d) * d
        v /= np.linalg.norm(v)
        ref, scl = integrals(REF, c1, c2, n, rt, k, v)
        got, _ = integrals(rule, c1, c2, n, rt, k, v)
        worst = max(worst, float(np.max(np.abs(got - ref) / scl)))
    assert worst < 1e-12, (kind, nq, worst)
