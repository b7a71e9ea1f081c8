"""CPU: the block elimination behind LU mode 3 (bem3_emf_b2_gb300/csrc/
gb_schur.cu) is exact for the reference's coupled matrix.

The coupled matrix A of an object with one interface is built by the oracle
(port.Obj.build_A, restating solve_bieq2.c:209-341) from the golden G, H that
the reference itself produced.  The same steps as the device code -- node-
column gathers of G_d, H_d, X_d = G_d^-1 H_d, M = X0 + X1, M3 = X1 + beta X0,
S = M3 - sigma delta sum_c D_c M^-1 D_c, and the six products of a
correction -- are restated here in complex128 and must solve A x = b to
rounding, for a random b with every block populated."""
import os

import numpy as np
import pytest

from oracle import port
from tests._scenes import load_case, write_inputs


def _node_blocks(o, G, H, did):
    """G_d, H_d with rows in the domain's collocation order (the A build's
    rowk) and columns at the global node ids eni[|sid[s]|][l]."""
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


def _block_solve(o, GH, r):
    nn = o.NN
    G0, H0 = _node_blocks(o, *GH[0], 0)
    G1, H1 = _node_blocks(o, *GH[1], 1)
    k0, k1 = o.kn[0], o.kn[1]
    delta, beta = k0 * k0 - k1 * k1, k0 * k0 / (k1 * k1)
    sigma = 1.0 - beta
    vn = np.zeros((nn, 3))
    for e in range(1, o.Ne + 1):
        for l in range(4 if o.etype[e] else 3):
            w = o.wen[e, l]
            vn[o.eni[e, l]] = w / np.linalg.norm(w)
    G0i, G1i = np.linalg.inv(G0), np.linalg.inv(G1)
    X0, X1 = G0i @ H0, G1i @ H1
    Minv = np.linalg.inv(X0 + X1)
    S = X1 + beta * X0 - sigma * delta * (vn @ vn.T) * Minv
    Si = np.linalg.inv(S)
    R0 = np.stack([r[c * nn:(c + 1) * nn] for c in range(4)], 1)
    R1 = np.stack([r[(4 + c) * nn:(5 + c) * nn] for c in range(4)], 1)
    T0 = G0i @ R0
    Y = G1i @ R1 + T0 * np.array([1.0, 1.0, 1.0, beta])
    MY = Minv @ Y[:, :3]
    U3 = Si @ (Y[:, 3] - sigma * (vn * MY).sum(1))
    U = np.concatenate([MY - delta * (Minv @ (vn * U3[:, None])), U3[:, None]], 1)
    dU = X0 @ U - T0
    return np.concatenate([U.T.ravel(), dU.T.ravel()])


@pytest.mark.parametrize("case", ["cube1", "sphere2", "cone_mix", "cone_tri"])
def test_block_elimination_solves_the_reference_system(case, tmp_path):
    meta, gold = load_case(case)
    wd = str(tmp_path)
    write_inputs(meta, wd)
    o = port.Obj(os.path.join(wd, "mesh.msh"), [complex(a, b) for a, b in meta["n"]], meta["wave"]["lambda0"],
                 meta["wave"]["ni"])
    # the objects the device path accepts: one interface, domain 0 outside
    assert o.MN == 1 and set(o.md[1:].tolist()) == {0} and set(o.sd[1:].tolist()) == {1}
    GH = {d: (gold["G_%d" % d], gold["H_%d" % d]) for d in range(2)}
    A = o.build_A(GH)
    rng = np.random.default_rng(7)
    b = rng.standard_normal(A.shape[0]) + 1j * rng.standard_normal(A.shape[0])
    x = _block_solve(o, GH, b)
    assert np.linalg.norm(A @ x - b) <= 1e-12 * np.linalg.norm(A) * np.linalg.norm(x)
    xd = np.linalg.solve(A, b)
    assert np.linalg.norm(x - xd) <= 1e-10 * np.linalg.norm(xd)
