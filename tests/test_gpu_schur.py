"""Block elimination of the coupled system (gb_set_lu_pivoting mode 3, the default).

For an object whose elements all separate the exterior domain 0 from the
interior domain 1, the chosen form's corrections can go through node-sized
FP32 inverses (G0^-1, G1^-1, X0 = G0^-1 H0, M^-1, S^-1; gb_schur.cu) instead
of the dense factors of the 8 NN x 8 NN coupled matrix (reference
solve_bieq2.c:241-316 builds that matrix, lu_dec_A inverts it).  The FP64
refinement around the corrections is the same, so force and torque must
agree with the dense factors to the refinement's accuracy."""
import ctypes
import os
import time

import numpy as np
import pytest

from bem3_emf_b2_gb300 import meshgen
from tests._scenes import load_case, write_inputs


def _lib():
    from bem3_emf_b2_gb300 import lib
    L = lib()
    vp, ci = ctypes.c_void_p, ctypes.c_int
    L.gb_set_lu_pivoting.argtypes = [vp, ci]
    L.gb_set_lu_pivoting.restype = ci
    L.gb_lu_info.argtypes = [vp, vp, vp]
    L.gb_lu_info.restype = ci
    return L


def _lu_info(L, o):
    kind, fb = ctypes.c_int(), ctypes.c_int()
    L.gb_lu_info(o, ctypes.byref(kind), ctypes.byref(fb))
    return kind.value, fb.value


def _rel(F1, N1, F0, N0):
    return np.linalg.norm(np.concatenate([F1 - F0, N1 - N0])) / np.linalg.norm(np.concatenate([F0, N0]))


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["sphere2", "cube1", "cone_mix", "cone_tri"])
def test_block_elimination_matches_dense_factors(case, gb_build, tmp_path):
    from bem3_emf_b2_gb300 import Scene
    L = _lib()
    meta, _ = load_case(case)
    wd = str(tmp_path)
    write_inputs(meta, wd)
    sc = Scene(os.path.join(wd, "medium.txt"), os.path.join(wd, "mesh.msh"), os.path.join(wd, "ipw.txt"))
    o = sc.obj()
    assert _lu_info(L, o) == (0, 0)
    assert L.gb_set_lu_pivoting(o, 0) == 0
    F0, N0 = sc.step(form=1)
    assert _lu_info(L, o)[0] == 1
    assert L.gb_set_lu_pivoting(o, 3) == 0
    F3, N3 = sc.step(form=1)
    kind, fb = _lu_info(L, o)
    it3, rr3 = sc.ir_info()
    assert (kind, fb) == (2, 0), (kind, fb)
    assert rr3 <= 1e-13 and it3 <= 10, (it3, rr3)  # single-pass TF32 node factors
    # a second step reuses the block buffers
    F4, N4 = sc.step(form=1)
    assert _lu_info(L, o) == (2, 0)
    assert L.gb_set_lu_pivoting(o, 4) != 0
    sc.close()
    d = _rel(F3, N3, F0, N0)
    assert d <= 1e-11, "block elimination vs dense factors, force/torque %g" % d
    assert _rel(F4, N4, F3, N3) <= 1e-13


@pytest.mark.gpu
def test_block_elimination_sphere384(gb_build, tmp_path):
    """The 384-element sphere (12,288 unknowns): same force and torque as the
    dense factors, and the step times of both printed."""
    from bem3_emf_b2_gb300 import Scene
    L = _lib()
    wd = str(tmp_path)
    nodes, elems = meshgen.cubed_sphere(8, 1.0)
    meshgen.write_mesh(os.path.join(wd, "mesh.msh"), nodes, elems)
    meshgen.write_medium(os.path.join(wd, "medium.txt"), [1.5])
    meshgen.write_ipw(os.path.join(wd, "ipw.txt"), [dict(lambda0=1.0, ni=1.33, power=1.0, e0x=1.0, e0y=0.0,
                                                          theta=0.0, phi=0.0)])
    sc = Scene(os.path.join(wd, "medium.txt"), os.path.join(wd, "mesh.msh"), os.path.join(wd, "ipw.txt"))
    o = sc.obj()
    res = {}
    for mode in (0, 3):
        assert L.gb_set_lu_pivoting(o, mode) == 0
        ts = []
        for _ in range(3):
            t0 = time.perf_counter()
            F, N = sc.step(form=1)
            ts.append(time.perf_counter() - t0)
        res[mode] = (F, N, min(ts), sc.ir_info(), _lu_info(L, o))
    sc.close()
    print("sphere384 step s: dense %.4f  block %.4f  (refinement %s / %s)" %
          (res[0][2], res[3][2], res[0][3], res[3][3]))
    assert res[3][4] == (2, 0)
    assert res[3][3][1] <= 1e-13
    d = _rel(res[3][0], res[3][1], res[0][0], res[0][1])
    assert d <= 1e-11, d


@pytest.mark.gpu
def test_block_elimination_sphere1536(gb_build, tmp_path):
    """The 1,536-element sphere (49,152 unknowns, 16 x 16 quadrangles per
    face): the dense FP32 factors need 19 GB and (8/3) (8 NN)^3 flop, the block
    factors 5 NN^2 complex FP32 and about 32 NN^3 -- same force and torque."""
    from bem3_emf_b2_gb300 import Scene
    L = _lib()
    wd = str(tmp_path)
    nodes, elems = meshgen.cubed_sphere(16, 1.0)
    meshgen.write_mesh(os.path.join(wd, "mesh.msh"), nodes, elems)
    meshgen.write_medium(os.path.join(wd, "medium.txt"), [1.5])
    meshgen.write_ipw(os.path.join(wd, "ipw.txt"), [dict(lambda0=1.0, ni=1.33, power=1.0, e0x=1.0, e0y=0.0,
                                                          theta=0.0, phi=0.0)])
    sc = Scene(os.path.join(wd, "medium.txt"), os.path.join(wd, "mesh.msh"), os.path.join(wd, "ipw.txt"))
    o = sc.obj()
    res = {}
    for mode in (3, 0):
        assert L.gb_set_lu_pivoting(o, mode) == 0
        t0 = time.perf_counter()
        F, N = sc.step(form=1)
        res[mode] = (F, N, time.perf_counter() - t0, sc.ir_info(), _lu_info(L, o))
    sc.close()
    print("sphere1536 step s: block %.3f  dense %.3f  (refinement %s / %s)" %
          (res[3][2], res[0][2], res[3][3], res[0][3]))
    assert res[3][4] == (2, 0)
    assert res[3][3][1] <= 1e-13
    d = _rel(res[3][0], res[3][1], res[0][0], res[0][1])
    assert d <= 1e-10, d


def _bv(L, sc, meta):
    """U, dU of every domain of the scene's object (reference layout)."""
    o = sc.obj()
    out = []
    for d, ne in enumerate(meta["sb_Ne"]):
        U = np.zeros((ne + 1, 4, 4), complex)
        dU = np.zeros((ne + 1, 4, 4), complex)
        assert L.gb_bv_download(o, d, U.ctypes.data, dU.ctypes.data, None, None, None, None) == 0
        out += [U[1:], dU[1:]]
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["sphere2", "cube1", "cone_mix", "cone_tri"])
def test_fp64_block_elimination_matches_dense_inverse(case, gb_build, tmp_path):
    """The plain FP64 form of a one-interface object factorises by the same
    block elimination in complex FP64 (gb_factor_fp64); its boundary values
    must equal those of the dense FP64 inverse (the reference's lu_dec_A) to
    <= 1e-10 relative, force and torque to <= 1e-11, and both must reproduce
    the reference's golden force."""
    from bem3_emf_b2_gb300 import Scene
    from tests._scenes import parse_analysis
    L = _lib()
    vp, ci = ctypes.c_void_p, ctypes.c_int
    L.gb_bv_download.argtypes = [vp, ci] + [vp] * 6
    L.gb_bv_download.restype = ci
    meta, _ = load_case(case)
    wd = str(tmp_path)
    write_inputs(meta, wd)
    sc = Scene(os.path.join(wd, "medium.txt"), os.path.join(wd, "mesh.msh"), os.path.join(wd, "ipw.txt"))
    o = sc.obj()
    assert L.gb_set_lu_pivoting(o, 0) == 0
    F0, N0 = sc.step(form=0)
    assert _lu_info(L, o)[0] == 0  # dense inverse
    b0 = _bv(L, sc, meta)
    assert L.gb_set_lu_pivoting(o, 3) == 0
    F3, N3 = sc.step(form=0)
    assert _lu_info(L, o) == (3, 0)
    it, rr = sc.ir_info()
    assert rr <= 1e-13 and it <= 3, (it, rr)
    b3 = _bv(L, sc, meta)
    sc.close()
    for x, y in zip(b3, b0):
        e = np.linalg.norm(x - y) / max(np.linalg.norm(y), 1e-300)
        assert e <= 1e-10, e
    assert _rel(F3, N3, F0, N0) <= 1e-11
    ref = parse_analysis(meta["analysis"])["force_0_0"]
    err = np.linalg.norm(np.concatenate([F3, N3]) - ref) / np.linalg.norm(ref)
    assert err <= 1e-9, err
