"""GPU: FP64 GMRES refinement of the chosen form's solves.

The chosen form solves A x = b with lower-precision factors as preconditioner
and FP64 GMRES(20) on A (gb_set_refinement mode 0, the default).  Checks:
  * GMRES and classical refinement (mode 1) give the same force and torque on
    the golden scenes (dense butterfly factors and block elimination), both
    to a relative residual <= 1e-13;
  * with single-pass TF32 factors (gb_set_tc_passes(1), ~1e-3 relative error
    in the factors) GMRES converges with no fallback to the 3-pass result, in
    no more steps than classical refinement needs with the same factors;
  * a high-contrast absorbing sphere (n = 0.06 + 4i, the reference's
    verification material) converges under GMRES and matches the FP64 form.
"""
import ctypes
import os

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
    L.gb_set_refinement.argtypes = [vp, ci]
    L.gb_set_refinement.restype = ci
    L.gb_set_tc_passes.argtypes = [ci]
    L.gb_set_tc_passes.restype = ci
    L.gb_get_tc_passes.restype = ci
    L.gb_lu_info.argtypes = [vp, vp, vp]
    L.gb_lu_info.restype = ci
    return L


def _lu_info(L, o):
    kind, fb = ctypes.c_int(), ctypes.c_int()
    L.gb_lu_info(o, ctypes.byref(kind), ctypes.byref(fb))
    return kind.value, fb.value


def _rel(F1, N1, F0, N0):
    return np.linalg.norm(np.concatenate([F1 - F0, N1 - N0])) / np.linalg.norm(np.concatenate([F0, N0]))


def _scene(wd):
    from bem3_emf_b2_gb300 import Scene
    return Scene(os.path.join(wd, "medium.txt"), os.path.join(wd, "mesh.msh"), os.path.join(wd, "ipw.txt"))


@pytest.mark.gpu
@pytest.mark.parametrize("case,lu_mode", [("sphere2", 0), ("cone_mix", 0), ("sphere2", 3), ("cone_tri", 3)])
def test_gmres_matches_classical_refinement(case, lu_mode, gb_build, tmp_path):
    L = _lib()
    meta, _ = load_case(case)
    wd = str(tmp_path)
    write_inputs(meta, wd)
    sc = _scene(wd)
    o = sc.obj()
    assert L.gb_set_lu_pivoting(o, lu_mode) == 0
    assert L.gb_set_refinement(o, 1) == 0
    F1, N1 = sc.step(form=1)
    it1, rr1 = sc.ir_info()
    assert L.gb_set_refinement(o, 0) == 0
    F0, N0 = sc.step(form=1)
    it0, rr0 = sc.ir_info()
    assert L.gb_set_refinement(o, 2) != 0
    info = _lu_info(L, o)
    sc.close()
    print("%s lu mode %d: classical %d corrections (%.1e), GMRES %d iterations (%.1e)" % (case, lu_mode, it1, rr1,
                                                                                       it0, rr0))
    assert rr0 <= 1e-13 and rr1 <= 1e-13
    assert info[1] == 0
    assert it0 <= it1 + 1  # the final FP64 residual check
    assert _rel(F0, N0, F1, N1) <= 1e-11


@pytest.mark.gpu
def test_gmres_absorbs_single_pass_tf32_factors(gb_build, tmp_path):
    """384-element sphere, dense butterfly factors (LU mode 0)."""
    L = _lib()
    wd = str(tmp_path)
    nodes, elems = meshgen.cubed_sphere(8, 1.0)
    meshgen.write_mesh(os.path.join(wd, "mesh.msh"), nodes, elems)
    meshgen.write_medium(os.path.join(wd, "medium.txt"), [1.5])
    meshgen.write_ipw(os.path.join(wd, "ipw.txt"), [dict(lambda0=1.0, ni=1.33, power=1.0, e0x=1.0, e0y=0.0)])
    sc = _scene(wd)
    o = sc.obj()
    assert L.gb_set_lu_pivoting(o, 0) == 0
    default = L.gb_get_tc_passes()
    try:
        assert L.gb_set_tc_passes(3) == 0
        F3, N3 = sc.step(form=1)
        it3, _ = sc.ir_info()
        assert L.gb_set_tc_passes(1) == 0
        assert L.gb_set_tc_passes(2) != 0
        F1, N1 = sc.step(form=1)
        it1, rr1 = sc.ir_info()
        kind, fb = _lu_info(L, o)
        assert (kind, fb) == (1, 0), (kind, fb)  # butterfly factors kept: no fallback
        assert rr1 <= 1e-13
        d = _rel(F1, N1, F3, N3)
        assert d <= 1e-10, d
        # classical refinement with the same single-pass factors: GMRES
        # minimises the residual over the Krylov space that contains the
        # classical iterates, so it never needs more steps
        assert L.gb_set_refinement(o, 1) == 0
        failed = False
        try:
            sc.step(form=1)
        except RuntimeError:
            failed = True
        itc, rrc = sc.ir_info()
        kind, fb2 = _lu_info(L, o)
        print("single-pass TF32 factors: GMRES %d iterations (3-pass: %d); classical %d corrections (%.1e), "
              "fallback %s, failed %s" % (it1, it3, itc, rrc, fb2 > fb, failed))
        assert failed or fb2 > fb or it1 <= itc
    finally:
        L.gb_set_tc_passes(default)
        sc.close()


@pytest.mark.gpu
def test_gmres_high_contrast_sphere(gb_build, tmp_path):
    """n = 0.06 + 4i sphere (radius 0.2, 6 x 6 quadrangles per face), the
    reference's verification2 material: chosen form (block elimination,
    GMRES) against the FP64 form."""
    L = _lib()
    wd = str(tmp_path)
    nodes, elems = meshgen.cubed_sphere(6, 0.2)
    meshgen.write_mesh(os.path.join(wd, "mesh.msh"), nodes, elems)
    meshgen.write_medium(os.path.join(wd, "medium.txt"), [complex(0.06, 4.0)])
    meshgen.write_ipw(os.path.join(wd, "ipw.txt"), [dict(lambda0=1.0, ni=1.0, power=1.0, e0x=1.0, e0y=0.0)])
    sc = _scene(wd)
    o = sc.obj()
    F64, N64 = sc.step(form=0)
    F, N = sc.step(form=1)
    it, rr = sc.ir_info()
    kind, fb = _lu_info(L, o)
    sc.close()
    print("high-contrast sphere: GMRES %d iterations, residual %.1e, factors %d, fallbacks %d" % (it, rr, kind, fb))
    assert rr <= 1e-13
    assert _rel(F, N, F64, N64) <= 1e-9
