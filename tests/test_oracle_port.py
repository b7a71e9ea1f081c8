"""The CPU oracle (oracle/port) against the reference's own outputs.

Pins the C restatement of the element quadrature and assembly, and the numpy
restatement of setup and of the coupled matrix / inverse, to the golden
fixtures that the reference itself produced (tests/golden)."""
import os
import tempfile

import numpy as np
import pytest

from bem3_emf_b2_gb300 import formats
from oracle import port
from tests._scenes import load_case, write_inputs

TOL = 1e-10


def _obj(meta, wd):
    write_inputs(meta, wd)
    n_media = [complex(a, b) for a, b in meta["n"]]
    w = meta["wave"]
    return port.Obj(os.path.join(wd, "mesh.msh"), n_media, w["lambda0"], w["ni"])


@pytest.mark.parametrize("case", ["cube1", "sphere2", "cone_mix", "cone_tri"])
def test_port_cmatrix_matches_reference(case, tmp_path):
    meta, gold = load_case(case)
    o = _obj(meta, str(tmp_path))
    assert o.NN == meta["NN"]
    for d in range(o.MN + 1):
        N = 4 * (len(o.sids[d]) - 1)
        rows = np.arange(N) if N <= 48 else np.arange(0, N, 5)   # a subset keeps the CPU suite short
        G, H, dG, dH, dF = o.rows(d, rows)
        d2 = np.stack([2 * rows, 2 * rows + 1], 1).ravel()
        for name, mine, ref in (("G", G, gold["G_%d" % d][rows]), ("H", H, gold["H_%d" % d][rows]),
                                ("dG", dG, gold["dG_%d" % d][d2]), ("dH", dH, gold["dH_%d" % d][d2]),
                                ("dF", dF, gold["dF_%d" % d][rows])):
            err = formats.rel_fro(mine, ref)
            assert err <= TOL, "%s domain %d: %g" % (name, d, err)


def test_port_inverse_matches_reference(tmp_path):
    meta, gold = load_case("cube1")
    o = _obj(meta, str(tmp_path))
    GH = {d: (gold["G_%d" % d], gold["H_%d" % d]) for d in range(o.MN + 1)}
    A = o.build_A(GH)
    inv = port.lapack_inverse(A)
    assert formats.rel_fro(inv, gold["invA"]) <= TOL


def test_port_domain_id(tmp_path):
    meta, _ = load_case("sphere2")
    o = _obj(meta, str(tmp_path))
    pts = np.array([[0.0, 0.0, 0.0], [0.0, 0.0, 1.0], [0.1, 0.05, -0.02], [2.0, 0.0, 0.0]])
    assert list(o.domain_id(pts)) == [1, 0, 1, 0]


@pytest.mark.parametrize("case", ["cube1", "sphere2", "cone_mix", "cone_tri"])
def test_port_single_object_solve_matches_reference(case, tmp_path):
    """The oracle's single-object solve (incident plane wave at the nodes,
    vectorised coupled matrix and right-hand side, LAPACK LU solve, boundary
    value store) reproduces the reference's own .dat boundary values."""
    meta, gold = load_case(case)
    o = _obj(meta, str(tmp_path))
    bv, GH, X = port.solve_single(o, [meta["wave"]])
    for d in range(o.MN + 1):
        for k in ("U", "dU"):
            err = formats.rel_fro(bv[d][k][1:], gold["o0_d%d_%s" % (d, k)][1:])
            assert err <= TOL, "%s domain %d: %g" % (k, d, err)
    if o.NN <= 200:
        A1, A0 = port.build_A_dense(o, GH), o.build_A(GH)
        assert np.array_equal(A1 != 0, A0 != 0) and formats.rel_fro(A1, A0) <= 1e-15
