"""CPU: the block elimination behind LU mode 3 (bem3_emf_b2_gb300/csrc/
gb_schur.cu) is exact for the reference's coupled matrix.

The coupled matrix A of an object with one interface is built by the oracle
(port.Obj.build_A, restating solve_bieq2.c:209-341) from the golden G, H that
the reference itself produced.  The same steps as the device code -- node-
column gathers of G_d, H_d, X_d = G_d^-1 H_d, M = X0 + X1, M3 = X1 + beta X0,
S = M3 - sigma delta sum_c D_c M^-1 D_c, and the six products of a
correction -- are restated in complex128 (oracle/block_model.py) and must
solve A x = b to rounding, for a random b with every block populated."""
import os

import numpy as np
import pytest

from oracle import block_model, port
from tests._scenes import load_case, write_inputs


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
    x = block_model.block_solve(o, GH, b)
    assert np.linalg.norm(A @ x - b) <= 1e-12 * np.linalg.norm(A) * np.linalg.norm(x)
    xd = np.linalg.solve(A, b)
    assert np.linalg.norm(x - xd) <= 1e-10 * np.linalg.norm(xd)


@pytest.mark.parametrize("inverse", ["pivoted", "butterfly"])
def test_fp32_block_factors_refine_to_1e13(inverse, tmp_path):
    """The complex-FP32 block factors as the correction of an FP64
    refinement on the reference's A: to a relative residual of 1e-13 within
    6 corrections, with pivoted LUs (the device path) and with
    butterfly-randomised LUs without interchanges of the node matrices."""
    meta, gold = load_case("sphere2")
    wd = str(tmp_path)
    write_inputs(meta, wd)
    o = port.Obj(os.path.join(wd, "mesh.msh"), [complex(a, b) for a, b in meta["n"]], meta["wave"]["lambda0"],
                 meta["wave"]["ni"])
    GH = {d: (gold["G_%d" % d], gold["H_%d" % d]) for d in range(2)}
    inv = block_model.inverse_pivoted32 if inverse == "pivoted" else block_model.inverse_butterfly32
    b = np.random.default_rng(9).standard_normal(8 * o.NN) * (1.0 - 0.5j)
    hist = block_model.refine(o, GH, inv, b)
    assert hist[-1] < 1e-13 and len(hist) <= 6, hist
