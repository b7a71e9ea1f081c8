"""Learned near-singular quadrature: training data and the CPU reference of the
network -- TEST INFRASTRUCTURE ONLY (tests/ and the label generation of the
training set; the product never imports it).

Labels.  A near-singular (observation node, bilinear element) pair is
integrated by the reference with its fallback rule: when |Re dF| > 0.5
(d3b1_elem.c:503) dcoef_bd_node_t2 switches to bil_dcoef_v2_GH
(bil_dcoef_v2.c:235-326), a 64 x 64 Gauss-Legendre rule.  The labels are that
rule's G_p and H_p (p = 0..3, CC[0..7]) from the C restatement
(oracle/port/bem_port.c port_quad_labels_c), pinned to the reference's own
fallback outputs in tests/test_lq_data.py.

Canonical frame.  G and H do not change under a rigid motion of the pair, and
under a scaling by h (with k -> k / h) G scales as h and H does not change.  So
a pair is described by its element's corners in a frame at the observation
point -- z along the element's normal at its centre (cw[:, 0]), x along the
first edge projected into the plane normal to z -- divided by the element
size h = 2 sqrt(|cw[:, 0]|) (the square root of the bilinear map's area at the
centre), and by k h: 12 + 2 inputs.  The outputs are G_p / h and H_p (real and
imaginary parts, 16).

Network.  14 -> 256 -> 256 -> 256 -> 16, GELU (erf form) on the hidden
layers, weights rounded to bfloat16 (round to nearest even) for the products,
FP32 master copies; mlp_forward / mlp_loss_grad restate it in float64 for the
gradient checks of the device kernels.
"""
import ctypes
import math

import numpy as np

from oracle import port

WIDTHS = (14, 256, 256, 256, 16)


# ---------------------------------------------------------------- pairs
def sample_pairs(n, seed, aspect=(1.0, 4.0), dist=(0.0, 3.0), warp=0.05, jitter=0.1, kh=(0.0, 2.5), kh_imag=(0.0, 0.1)):
    """Seeded random (element, observation point, k) triples: a rectangle of
    aspect ratio U[aspect] and unit area, corners jittered in-plane by up to
    `jitter` and out of plane by up to `warp` (fractions of the size), randomly
    rotated and placed; the observation point at U[dist] x size from the centre
    in a uniformly random direction; k h with real part U[kh] and imaginary
    part U[kh_imag].  Returns corners (n, 4, 3), rt (n, 3), k (n,) complex."""
    rng = np.random.default_rng(seed)
    a = rng.uniform(*aspect, n)
    sx, sy = np.sqrt(a), 1.0 / np.sqrt(a)
    base = np.array([[-0.5, -0.5], [0.5, -0.5], [0.5, 0.5], [-0.5, 0.5]])
    c = np.zeros((n, 4, 3))
    c[:, :, 0] = base[None, :, 0] * sx[:, None]
    c[:, :, 1] = base[None, :, 1] * sy[:, None]
    c[:, :, :2] += rng.uniform(-jitter, jitter, (n, 4, 2))
    c[:, :, 2] += rng.uniform(-warp, warp, (n, 4))
    scale = np.exp(rng.uniform(np.log(0.05), np.log(2.0), n))
    q = rng.standard_normal((n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    R = _quat_to_rot(q)
    shift = rng.uniform(-5.0, 5.0, (n, 3))
    corners = np.einsum("nij,nkj->nki", R, c) * scale[:, None, None] + shift[:, None, :]
    centre = corners.mean(1)
    u = rng.standard_normal((n, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    h = element_size(corners)
    rt = centre + u * (rng.uniform(*dist, n) * h)[:, None]
    k = (rng.uniform(*kh, n) + 1j * rng.uniform(*kh_imag, n)) / h
    return corners, rt, k


def sample_mesh_pairs(n, seed, aspect=(1.0, 2.0), fold=0.5, jitter=0.05, kh=(0.0, 2.5), kh_imag=(0.0, 0.1)):
    """Seeded (element, node) pairs placed the way a surface mesh places its
    near-singular pairs: the observation point is a collocation node
    (zeta, eta = +-1/sqrt 3) of a neighbouring quadrangle that shares an edge
    with the element (or, for a quarter of the pairs, only a corner), folded
    about the shared edge (or tilted about the corner) by up to `fold`
    radians.  Element: rectangle of aspect ratio U[aspect], corners jittered
    by up to `jitter`; the pair then rotated, scaled and placed at random.
    Returns corners (n, 4, 3), rt (n, 3), k (n,) complex."""
    rng = np.random.default_rng(seed)
    a = rng.uniform(*aspect, n)
    sx, sy = np.sqrt(a), 1.0 / np.sqrt(a)
    base = np.array([[-0.5, -0.5], [0.5, -0.5], [0.5, 0.5], [-0.5, 0.5]])
    c = np.zeros((n, 4, 3))
    c[:, :, 0] = base[None, :, 0] * sx[:, None]
    c[:, :, 1] = base[None, :, 1] * sy[:, None]
    c[:, :, :2] += rng.uniform(-jitter, jitter, (n, 4, 2))
    g = 0.5773502691896257645091
    zn = rng.choice([-g, g], n)
    en = rng.choice([-g, g], n)
    rt = np.zeros((n, 3))
    corner = rng.random(n) < 0.25
    ang = rng.uniform(-fold, fold, n)
    for i in range(n):
        # neighbour rectangle of the same size, its local point (in the
        # element's plane before folding): shifted by one element along x,
        # or diagonally for a corner neighbour
        side = rng.integers(4)
        dx, dy = [(1, 0), (-1, 0), (0, 1), (0, -1)][side]
        if corner[i]:
            dx, dy = rng.choice([-1, 1]), rng.choice([-1, 1])
        p = np.array([dx * sx[i] + 0.5 * zn[i] * sx[i], dy * sy[i] + 0.5 * en[i] * sy[i], 0.0])
        # fold about the shared edge (or tilt about the shared corner)
        pivot = np.array([0.5 * dx * sx[i], 0.5 * dy * sy[i], 0.0])
        axis = np.array([-dy, dx, 0.0]) if not corner[i] else np.array([-dy * sy[i], dx * sx[i], 0.0])
        axis /= np.linalg.norm(axis)
        v = p - pivot
        ca, sa = np.cos(ang[i]), np.sin(ang[i])
        v = v * ca + np.cross(axis, v) * sa + axis * np.dot(axis, v) * (1 - ca)
        rt[i] = pivot + v
    scale = np.exp(rng.uniform(np.log(0.05), np.log(2.0), n))
    q = rng.standard_normal((n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    R = _quat_to_rot(q)
    shift = rng.uniform(-5.0, 5.0, (n, 3))
    corners = np.einsum("nij,nkj->nki", R, c) * scale[:, None, None] + shift[:, None, :]
    rt = np.einsum("nij,nj->ni", R, rt) * scale[:, None] + shift
    h = element_size(corners)
    k = (rng.uniform(*kh, n) + 1j * rng.uniform(*kh_imag, n)) / h
    return corners, rt, k


def _quat_to_rot(q):
    w, x, y, z = q.T
    return np.stack([np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)], -1),
                     np.stack([2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)], -1),
                     np.stack([2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], -1)], -2)


def _cw0(corners):
    """cw[:, 0] of the reference's bilinear element (setup2.c:666-745)"""
    rc = np.transpose(corners, (0, 2, 1))  # [n][xyz][corner]
    out = np.zeros((corners.shape[0], 3))
    for d in range(3):
        a, b = (d + 1) % 3, (d + 2) % 3
        out[:, d] = 0.125 * ((rc[:, a, 0] - rc[:, a, 2]) * (rc[:, b, 1] - rc[:, b, 3]) -
                             (rc[:, a, 1] - rc[:, a, 3]) * (rc[:, b, 0] - rc[:, b, 2]))
    return out


def element_size(corners):
    return 2.0 * np.sqrt(np.linalg.norm(_cw0(corners), axis=1))


def features(corners, rt, k):
    """(n, 14) network inputs and the sizes h (n,)"""
    corners = np.asarray(corners, float)
    h = element_size(corners)
    ez = _cw0(corners)
    ez /= np.linalg.norm(ez, axis=1, keepdims=True)
    e1 = corners[:, 1] - corners[:, 0]
    ex = e1 - (e1 * ez).sum(1, keepdims=True) * ez
    ex /= np.linalg.norm(ex, axis=1, keepdims=True)
    ey = np.cross(ez, ex)
    rel = (corners - np.asarray(rt, float)[:, None, :]) / h[:, None, None]
    loc = np.stack([(rel * ex[:, None, :]).sum(2), (rel * ey[:, None, :]).sum(2), (rel * ez[:, None, :]).sum(2)], 2)
    kh = np.asarray(k) * h
    return np.concatenate([loc.reshape(-1, 12), kh.real[:, None], kh.imag[:, None]], 1), h


def labels(corners, rt, k, type_=3):
    """(n, 16): re, im of G_0..G_3, H_0..H_3 by the rule type_ (3: the GHN
    64 x 64 rule of the reference's fallback)"""
    corners = np.ascontiguousarray(corners, float)
    rt = np.ascontiguousarray(rt, float)
    kk = np.ascontiguousarray(np.stack([np.real(k), np.imag(k)], 1), float)
    n = corners.shape[0]
    out = np.zeros((n, 16))
    L = port.lib()
    L.port_quad_labels_c(ctypes.c_int(n), corners.ctypes.data_as(ctypes.c_void_p), rt.ctypes.data_as(ctypes.c_void_p),
                         kk.ctypes.data_as(ctypes.c_void_p), ctypes.c_int(type_), out.ctypes.data_as(ctypes.c_void_p))
    return out


def targets(lab, h):
    """network outputs from labels: G / h, H"""
    t = lab.copy()
    t[:, :8] /= h[:, None]
    return t


def untarget(t, h):
    lab = np.asarray(t, float).copy()
    lab[:, :8] *= h[:, None]
    return lab


# ---------------------------------------------------------------- network
def bf16_round(x):
    """float32 -> nearest bfloat16 (ties to even), returned as float32"""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32)


def gelu(z):
    from scipy.special import erf
    return 0.5 * z * (1.0 + erf(z / math.sqrt(2.0)))


def gelu_grad(z):
    from scipy.special import erf
    return 0.5 * (1.0 + erf(z / math.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / math.sqrt(2.0 * math.pi)


def init_params(seed, widths=WIDTHS):
    """[(W [in][out], b [out]) ...] float32, uniform +-sqrt(6 / (in + out))"""
    rng = np.random.default_rng(seed)
    ps = []
    for a, b in zip(widths[:-1], widths[1:]):
        lim = math.sqrt(6.0 / (a + b))
        ps.append((rng.uniform(-lim, lim, (a, b)).astype(np.float32), np.zeros(b, np.float32)))
    return ps


def pack(ps):
    return np.concatenate([np.concatenate([W.ravel(), b]) for W, b in ps]).astype(np.float32)


def unpack(v, widths=WIDTHS):
    ps, o = [], 0
    for a, b in zip(widths[:-1], widths[1:]):
        W = v[o:o + a * b].reshape(a, b)
        o += a * b
        ps.append((W, v[o:o + b]))
        o += b
    return ps


def mlp_forward(ps, X, quant=True):
    """float64 forward with bfloat16-rounded weights (quant=False: the
    weights as given, for finite-difference checks); returns (Y, cache)"""
    A = np.asarray(X, np.float64)
    cache = []
    for i, (W, b) in enumerate(ps):
        Wq = bf16_round(W).astype(np.float64) if quant else np.asarray(W, np.float64)
        Z = A @ Wq + b.astype(np.float64)
        cache.append((A, Z, Wq))
        A = gelu(Z) if i + 1 < len(ps) else Z
    return A, cache


def mlp_loss_grad(ps, X, T, quant=True):
    """mean over the batch of the summed squared error, and its gradient
    with respect to every weight and bias (through the bfloat16 weights as
    if they were the master weights)"""
    Y, cache = mlp_forward(ps, X, quant)
    B = X.shape[0]
    D = Y - np.asarray(T, np.float64)
    loss = float((D * D).sum() / B)
    dZ = 2.0 * D / B
    grads = [None] * len(ps)
    for i in range(len(ps) - 1, -1, -1):
        A, Z, Wq = cache[i]
        grads[i] = (A.T @ dZ, dZ.sum(0))
        if i > 0:
            dZ = (dZ @ Wq.T) * gelu_grad(cache[i - 1][1])
    return loss, grads
