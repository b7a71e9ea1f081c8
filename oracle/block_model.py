"""Block elimination of a single-interface object's coupled system -- TEST
INFRASTRUCTURE ONLY (a numpy model of bem3_emf_b2_gb300/csrc/gb_schur.cu for
tests/ and CPU experiments; the product never imports it).

The coupled matrix A (reference solve_bieq2.c:241-316) of an object whose
elements all separate domain 0 (outside) from domain 1 (inside) has 4 x 4
node-sized blocks built from G0, H0, G1, H1 and the node normals.  The
device path eliminates dU through the exterior rows, then U_0..U_2 through
M = X0 + X1 (X_d = G_d^-1 H_d), which leaves the Schur complement
S = X1 + beta X0 - sigma delta sum_c D_c M^-1 D_c for U_3 (delta = k0^2 - k1^2,
beta = k0^2 / k1^2, sigma = 1 - beta).  node_blocks and block_solve restate
that in complex128; block_preconditioner does it in complex64 with either
pivoted LUs or butterfly-randomised LUs without interchanges (Parker 1995),
for refinement experiments:

    python -m oracle.block_model [quadrangles per cube face]
    python -m oracle.block_model 8 bf16   # GMRES with bf16-stored factors
"""
import os
import sys
import tempfile
import time

import numpy as np
import scipy.linalg as sla


def node_blocks(o, G, H, did):
    """G_d, H_d of an oracle object (port.Obj) with rows in the domain's
    collocation order (the A build's row order) and columns at the global node
    ids eni[|sid[s]|][l]"""
    sid = o.sids[did]
    rows, cols, cn = [], [], []
    for t in range(1, len(sid)):
        for tn in range(4):
            if tn == 3 and not o.etype[abs(sid[t])]:
                continue
            rows.append((t - 1) * 4 + tn)
    for s in range(1, len(sid)):
        e = abs(sid[s])
        for l in range(4 if o.etype[e] else 3):
            cols.append((s - 1) * 4 + l)
            cn.append(o.eni[e, l])
    Gh = np.zeros((len(rows), o.NN), complex)
    Hh = np.zeros((len(rows), o.NN), complex)
    Gh[:, cn] = G[np.ix_(rows, cols)]
    Hh[:, cn] = H[np.ix_(rows, cols)]
    return Gh, Hh


def constants(o):
    """delta, beta, sigma and the nodes' unit normals vn [NN][3]"""
    k0, k1 = o.kn[0], o.kn[1]
    delta, beta = k0 * k0 - k1 * k1, k0 * k0 / (k1 * k1)
    vn = np.zeros((o.NN, 3))
    for e in range(1, o.Ne + 1):
        for l in range(4 if o.etype[e] else 3):
            w = o.wen[e, l]
            vn[o.eni[e, l]] = w / np.linalg.norm(w)
    return delta, beta, 1.0 - beta, vn


def _apply(nn, inv, r, dt):
    """one correction with the five inverses (the six device products)"""
    G0i, G1i, X0, Minv, Si, delta, beta, sigma, vn = inv
    R0 = np.stack([r[c * nn:(c + 1) * nn] for c in range(4)], 1).astype(dt)
    R1 = np.stack([r[(4 + c) * nn:(5 + c) * nn] for c in range(4)], 1).astype(dt)
    T0 = G0i @ R0
    Y = G1i @ R1 + T0 * np.array([1.0, 1.0, 1.0, beta], dt)
    MY = Minv @ Y[:, :3]
    U3 = Si @ (Y[:, 3] - dt(sigma) * (vn * MY).sum(1))
    U = np.concatenate([MY - dt(delta) * (Minv @ (vn * U3[:, None]).astype(dt)), U3[:, None]], 1)
    dU = X0 @ U - T0
    return np.concatenate([U.T.ravel(), dU.T.ravel()]).astype(complex)


def _factors(o, GH, inv, dt):
    G0, H0 = node_blocks(o, *GH[0], 0)
    G1, H1 = node_blocks(o, *GH[1], 1)
    delta, beta, sigma, vn = constants(o)
    G0i, G1i = inv(G0.astype(dt)), inv(G1.astype(dt))
    X0, X1 = G0i @ H0.astype(dt), G1i @ H1.astype(dt)
    Minv = inv(X0 + X1)
    S = X1 + dt(beta) * X0 - dt(sigma * delta) * (vn @ vn.T).astype(dt) * Minv
    return (G0i, G1i, X0, Minv, inv(S), delta, beta, sigma, vn.astype(np.float32 if dt == np.complex64 else float))


def block_solve(o, GH, r):
    """x = A^-1 r by the block elimination in complex128 (GH: {d: (G, H)})"""
    return _apply(o.NN, _factors(o, GH, np.linalg.inv, np.complex128), r, np.complex128)


def _butterfly(rng, n):
    h = n // 2
    r0 = np.exp(rng.uniform(-0.5, 0.5, h) / 10)
    r1 = np.exp(rng.uniform(-0.5, 0.5, h) / 10)
    B = np.zeros((n, n))
    B[:h, :h], B[:h, h:], B[h:, :h], B[h:, h:] = np.diag(r0), np.diag(r1), np.diag(r0), -np.diag(r1)
    return B / np.sqrt(2.0)


def _rbt(rng, n):
    """depth-2 recursive butterfly (n divisible by 4)"""
    low = np.zeros((n, n))
    h = n // 2
    low[:h, :h], low[h:, h:] = _butterfly(rng, h), _butterfly(rng, h)
    return _butterfly(rng, n) @ low


def _lu_nopiv(A, nb=64):
    """blocked right-looking LU without interchanges, in A's precision"""
    A = A.copy()
    n = A.shape[0]
    for k in range(0, n, nb):
        e = min(k + nb, n)
        for j in range(k, e):
            A[j + 1:, j] /= A[j, j]
            A[j + 1:, j + 1:e] -= np.outer(A[j + 1:, j], A[j, j + 1:e])
        if e < n:
            L11 = np.tril(A[k:e, k:e], -1) + np.eye(e - k, dtype=A.dtype)
            A[k:e, e:] = sla.solve_triangular(L11, A[k:e, e:], lower=True, unit_diagonal=True)
            A[e:, e:] -= A[e:, k:e] @ A[k:e, e:]
    return A


def inverse_pivoted32(A):
    return sla.lu_solve(sla.lu_factor(A.astype(np.complex64)), np.eye(A.shape[0], dtype=np.complex64))


def inverse_butterfly32(A, seed=0):
    """A^-1 = V (U^T A V)^-1 U^T with the LU of U^T A V taken without
    interchanges in complex64"""
    rng = np.random.default_rng(seed)
    n = A.shape[0]
    U, V = _rbt(rng, n).astype(np.float32), _rbt(rng, n).astype(np.float32)
    F = _lu_nopiv(U.T @ A.astype(np.complex64) @ V)
    L = np.tril(F, -1) + np.eye(n, dtype=F.dtype)
    Finv = sla.solve_triangular(np.triu(F), sla.solve_triangular(L, np.eye(n, dtype=F.dtype), lower=True,
                                                                 unit_diagonal=True))
    return (V @ Finv @ U.T).astype(np.complex64)


def refine(o, GH, inv, b, tol=1e-13, itmax=30):
    """FP64 refinement x += P (b - A x) with the complex64 block factors;
    returns the relative residual after each correction"""
    P = _factors(o, GH, inv, np.complex64)
    A = o.build_A(GH)
    x = np.zeros_like(b)
    r = b.copy()
    hist = []
    for _ in range(itmax):
        x = x + _apply(o.NN, P, r, np.complex64)
        r = b - A @ x
        hist.append(np.linalg.norm(r) / np.linalg.norm(b))
        if hist[-1] < tol:
            break
    return hist


def bf16_round(x):
    """each real component of a complex array rounded to bfloat16 (8
    significant bits, round to nearest even on the FP32 bits), returned as
    complex64: the 16-bit storage of the factors modelled on the CPU"""
    f = np.ascontiguousarray(x.astype(np.complex64)).view(np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return u.astype(np.uint32).view(np.float32).view(np.complex64)


def gmres_with_factors(o, GH, b, store=None, restart=30, tol=1e-13):
    """GMRES(restart) from zero on the coupled matrix A (complex128),
    preconditioned by the block elimination's complex64 factors (pivoted
    LUs), their five matrices optionally passed through `store` (e.g.
    bf16_round); returns (iterations, true relative residual)"""
    import scipy.sparse.linalg as spla
    P = list(_factors(o, GH, inverse_pivoted32, np.complex64))
    if store is not None:
        P[:5] = [store(m) for m in P[:5]]
    A = o.build_A(GH)
    M = spla.LinearOperator(A.shape, matvec=lambda r: _apply(o.NN, P, r, np.complex64), dtype=complex)
    res = []
    x, _ = spla.gmres(A, b, rtol=tol, restart=restart, maxiter=20, M=M, callback=lambda r: res.append(r),
                      callback_type="pr_norm")
    return len(res), float(np.linalg.norm(b - A @ x) / np.linalg.norm(b))


if __name__ == "__main__":
    if len(sys.argv) > 2 and sys.argv[2] == "bf16":
        # the 24,576-element sphere's geometry (radius 3, n = 1.5 + 0.01i in
        # 1.33) at a coarser resolution: GMRES with FP32 and bf16-stored factors
        from bem3_emf_b2_gb300 import meshgen
        from oracle import port
        nface = int(sys.argv[1])
        wd = tempfile.mkdtemp()
        nodes, elems = meshgen.cubed_sphere(nface, 3.0)
        meshgen.write_mesh(os.path.join(wd, "mesh.msh"), nodes, elems)
        o = port.Obj(os.path.join(wd, "mesh.msh"), [complex(1.5, 0.01)], 1.0, 1.33)
        GH = {d: o.rows(d)[:2] for d in range(2)}
        b = np.random.default_rng(1).standard_normal(8 * o.NN) * (1 + 1j)
        for name, store in (("complex FP32 factors", None), ("bf16-stored factors", bf16_round)):
            it, rr = gmres_with_factors(o, GH, b, store)
            print("%d per face (NN = %d), %s: %d GMRES(30) iterations, true relative residual %.1e"
                  % (nface, o.NN, name, it, rr))
        sys.exit(0)
    from bem3_emf_b2_gb300 import meshgen
    from oracle import port
    nface = int(sys.argv[1]) if len(sys.argv) > 1 else 8
    wd = tempfile.mkdtemp()
    nodes, elems = meshgen.cubed_sphere(nface, 1.0)
    meshgen.write_mesh(os.path.join(wd, "mesh.msh"), nodes, elems)
    o = port.Obj(os.path.join(wd, "mesh.msh"), [1.5], 1.0, 1.33)
    GH = {d: o.rows(d)[:2] for d in range(2)}
    b = np.random.default_rng(1).standard_normal(8 * o.NN) * (1 + 1j)
    for name, inv in (("pivoted", inverse_pivoted32), ("butterfly", inverse_butterfly32)):
        t0 = time.time()
        hist = refine(o, GH, inv, b)
        print("%d x %d per face (NN = %d), %s FP32 LUs: %d corrections %s (%.0f s)"
              % (nface, nface, o.NN, name, len(hist), ["%.1e" % h for h in hist], time.time() - t0))
