"""GPU: the chosen (mixed-precision) form against the plain FP64 form and the
reference.  Double-float regular-pair assembly + complex-FP32 LU + FP64
iterative refinement must reproduce the FP64 form's radiation force and
torque to <= 1e-6 relative (the tolerance of the chosen form) -- in practice
the refinement reaches a relative residual of 1e-13 and the double-float
matrices agree with FP64 to ~1e-14 -- and the reference's force (golden)
too."""
import os

import numpy as np
import pytest

from tests._scenes import load_case, parse_analysis, write_inputs


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["sphere2", "cone_mix", "cone_tri"])
def test_mixed_form_force_matches_fp64_and_reference(case, gb_build, tmp_path):
    from bem3_emf_b2_gb300 import Scene
    meta, _ = load_case(case)
    wd = str(tmp_path)
    write_inputs(meta, wd)
    sc = Scene(os.path.join(wd, "medium.txt"), os.path.join(wd, "mesh.msh"), os.path.join(wd, "ipw.txt"))
    F64, N64 = sc.step(form=0)
    F32, N32 = sc.step(form=1)
    it, rr = sc.ir_info()
    sc.close()
    assert rr <= 1e-12 and it >= 1
    ref = parse_analysis(meta["analysis"])["force_0_0"]
    for F, N in ((F64, N64), (F32, N32)):
        v = np.concatenate([F, N])
        err = np.linalg.norm(v - ref) / np.linalg.norm(ref)
        assert err <= 1e-6, "force/torque relative error %g" % err
    d = np.linalg.norm(np.concatenate([F32 - F64, N32 - N64])) / np.linalg.norm(np.concatenate([F64, N64]))
    assert d <= 1e-9, "mixed vs FP64 force/torque %g" % d


@pytest.mark.gpu
def test_fp32_far_pair_assembly_error(gb_build, tmp_path):
    """gb_assemble2(precision 1): FP32 regular far pairs.  The matrices must
    stay within 3e-7 relative Frobenius of the FP64 assembly (measured about
    1e-7 on G and 2e-7 on dH) and precision 0 must be the FP64 path itself."""
    import ctypes
    from bem3_emf_b2_gb300 import Scene, formats, lib
    import bench
    L = lib()
    vp, ci = ctypes.c_void_p, ctypes.c_int
    L.gb_assemble2.argtypes = [vp, ci, ci, ci]
    L.gb_assemble2.restype = ci
    L.gb_cmatrix_download.argtypes = [vp, ci] + [vp] * 5
    wd = str(tmp_path)
    bench.write_sphere(wd, 6)
    sc = Scene(os.path.join(wd, "medium.txt"), os.path.join(wd, "mesh.msh"), os.path.join(wd, "ipw.txt"))
    o = sc.obj()
    N = 4 * 6 * 36
    for d in range(2):
        out = {}
        for prec in (0, 1):
            assert L.gb_assemble2(o, d, 2, prec) == 0, L.gb_last_error()
            m = [np.zeros((N, N), complex), np.zeros((N, N), complex), np.zeros((2 * N, N), complex),
                 np.zeros((2 * N, N), complex)]
            assert L.gb_cmatrix_download(o, d, m[0].ctypes.data, m[1].ctypes.data, m[2].ctypes.data, m[3].ctypes.data,
                                         None) == 0
            out[prec] = m
        errs = [formats.rel_fro(a, b) for a, b in zip(out[1], out[0])]
        assert max(errs) <= 3e-7, errs
        assert max(errs) > 0.0  # the FP32 path did run
    sc.close()


def _download(L, o, d, N):
    m = [np.zeros((N, N), complex), np.zeros((N, N), complex), np.zeros((2 * N, N), complex),
         np.zeros((2 * N, N), complex), np.zeros((N, 3))]
    assert L.gb_cmatrix_download(o, d, *[x.ctypes.data for x in m]) == 0, L.gb_last_error()
    return m


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["sphere2", "cone_mix", "cone_tri", "cube1", "sphere_nf6"])
def test_double_float_assembly_matches_fp64(case, gb_build, tmp_path):
    """gb_assemble2(precision 2): regular pairs in double-float.  G, H, dG, dH
    and dF must agree with the FP64 assembly to <= 1e-12 relative Frobenius
    (measured 3e-15 .. 4e-14), and the chosen scene form (form 1) must give the
    force and torque of form 3 (same factorisation, FP64 assembly) to 1e-11."""
    import ctypes
    from bem3_emf_b2_gb300 import Scene, formats, lib
    import bench
    L = lib()
    vp, ci = ctypes.c_void_p, ctypes.c_int
    L.gb_assemble2.argtypes = [vp, ci, ci, ci]
    L.gb_assemble2.restype = ci
    L.gb_cmatrix_download.argtypes = [vp, ci] + [vp] * 5
    L.gb_form_precision.argtypes = [ci]
    L.gb_form_precision.restype = ci
    assert [L.gb_form_precision(f) for f in range(4)] == [0, 3, 1, 0]
    wd = str(tmp_path)
    if case == "sphere_nf6":
        bench.write_sphere(wd, 6)
        Ns = [4 * 6 * 36] * 2
    else:
        meta, _ = load_case(case)
        write_inputs(meta, wd)
        Ns = [4 * x for x in meta["sb_Ne"]]
    sc = Scene(os.path.join(wd, "medium.txt"), os.path.join(wd, "mesh.msh"), os.path.join(wd, "ipw.txt"))
    o = sc.obj()
    for d in range(len(Ns)):
        assert L.gb_assemble2(o, d, 2, 0) == 0, L.gb_last_error()
        a = _download(L, o, d, Ns[d])
        assert L.gb_assemble2(o, d, 2, 2) == 0, L.gb_last_error()
        b = _download(L, o, d, Ns[d])
        errs = [formats.rel_fro(x, y) for x, y in zip(b, a)]
        assert max(errs) <= 1e-12, errs
        # precision 3 (the chosen form): far pairs with the adaptive order
        assert L.gb_assemble2(o, d, 2, 3) == 0, L.gb_last_error()
        c = _download(L, o, d, Ns[d])
        errs3 = [formats.rel_fro(x, y) for x, y in zip(c, a)]
        print("%s domain %d: precision 2 %.1e, precision 3 %.1e" % (case, d, max(errs), max(errs3)))
        assert max(errs3) <= 1e-10, errs3
    F3, N3 = sc.step(form=3)
    F1, N1 = sc.step(form=1)
    sc.close()
    d = np.linalg.norm(np.concatenate([F1 - F3, N1 - N3])) / np.linalg.norm(np.concatenate([F3, N3]))
    assert d <= 1e-11, "double-float vs FP64 assembly, force/torque %g" % d


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["sphere2", "cone_mix", "cone_tri", "cube1"])
def test_butterfly_lu_matches_tournament_lu(case, gb_build, tmp_path):
    """The chosen form factorises the randomised matrix U^T A V without
    interchanges (gb_set_lu_pivoting 0); with tournament
    pivoting (mode 1) the same refinement must give the same force and torque
    to the refinement's accuracy, and the randomised factors must have been
    used without a fallback on these scenes."""
    import ctypes
    from bem3_emf_b2_gb300 import Scene, lib
    L = lib()
    vp, ci = ctypes.c_void_p, ctypes.c_int
    L.gb_set_lu_pivoting.argtypes = [vp, ci]
    L.gb_set_lu_pivoting.restype = ci
    L.gb_lu_info.argtypes = [vp, vp, vp]
    L.gb_lu_info.restype = ci
    meta, _ = load_case(case)
    wd = str(tmp_path)
    write_inputs(meta, wd)
    sc = Scene(os.path.join(wd, "medium.txt"), os.path.join(wd, "mesh.msh"), os.path.join(wd, "ipw.txt"))
    o = sc.obj()
    assert L.gb_set_lu_pivoting(o, 0) == 0  # dense butterfly factors (the default is block elimination)
    F0, N0 = sc.step(form=1)
    rbt, fb = ctypes.c_int(), ctypes.c_int()
    L.gb_lu_info(o, ctypes.byref(rbt), ctypes.byref(fb))
    it0, rr0 = sc.ir_info()
    assert rbt.value == 1 and fb.value == 0, (rbt.value, fb.value)
    assert rr0 <= 1e-13
    assert L.gb_set_lu_pivoting(o, 1) == 0
    F1, N1 = sc.step(form=1)
    L.gb_lu_info(o, ctypes.byref(rbt), ctypes.byref(fb))
    assert rbt.value == 0
    # the fallback path: butterfly factors, refinement declared stalled at its
    # first check, tournament refactorisation, refinement continued
    assert L.gb_set_lu_pivoting(o, 2) == 0
    F2, N2 = sc.step(form=1)
    L.gb_lu_info(o, ctypes.byref(rbt), ctypes.byref(fb))
    it2, rr2 = sc.ir_info()
    assert rbt.value == 0 and fb.value == 1, (rbt.value, fb.value)
    assert rr2 <= 1e-13
    assert L.gb_set_lu_pivoting(o, 4) != 0
    sc.close()
    d = np.linalg.norm(np.concatenate([F1 - F0, N1 - N0])) / np.linalg.norm(np.concatenate([F0, N0]))
    assert d <= 1e-11, "butterfly vs tournament LU, force/torque %g" % d
    d2 = np.linalg.norm(np.concatenate([F2 - F0, N2 - N0])) / np.linalg.norm(np.concatenate([F0, N0]))
    assert d2 <= 1e-11, "after the fallback, force/torque %g" % d2


@pytest.mark.gpu
@pytest.mark.parametrize("case,prec,tol", [("sphere2", 2, 1e-11), ("cone_mix", 2, 1e-11), ("sphere2", 3, 1e-10),
                                           ("cone_mix", 3, 1e-10)])
def test_double_float_field_kernels_match_fp64(case, prec, tol, gb_build, tmp_path):
    """After a precision-2 (3) assembly the object's field kernels (potentials and
    fields at points: modes 0-3; fields on the boundary) integrate the regular
    GLN pairs in double-float (with the adaptive order).  With the same boundary values they must give
    the FP64 kernels' values to <= 1e-11 relative (vector norm)."""
    import ctypes
    from bem3_emf_b2_gb300 import Scene, lib
    L = lib()
    vp, ci = ctypes.c_void_p, ctypes.c_int
    L.gb_assemble2.argtypes = [vp, ci, ci, ci]
    L.gb_assemble2.restype = ci
    L.gb_domain_id.argtypes = [vp, ci, vp, vp]
    L.gb_domain_id.restype = ci
    L.gb_field_points.argtypes = [vp, ci, ci, ci, vp, vp, vp, vp, vp]
    L.gb_field_points.restype = ci
    L.gb_field_bd.argtypes = [vp, ci, ci, vp, vp, vp, vp]
    L.gb_field_bd.restype = ci
    meta, _ = load_case(case)
    wd = str(tmp_path)
    write_inputs(meta, wd)
    sc = Scene(os.path.join(wd, "medium.txt"), os.path.join(wd, "mesh.msh"), os.path.join(wd, "ipw.txt"))
    o = sc.obj()
    sc.step(form=0)  # boundary values; the field kernels are FP64 after a precision-0 assembly
    rng = np.random.default_rng(5)
    n = 256
    d = rng.standard_normal((n, 3))
    d /= np.linalg.norm(d, axis=1)[:, None]
    rt = np.ascontiguousarray(d * rng.uniform(0.3, 3.0, n)[:, None])
    v = np.ascontiguousarray(rng.standard_normal((n, 3)))
    did = np.zeros(n, np.int32)
    assert L.gb_domain_id(o, n, rt.ctypes.data, did.ctypes.data) == 0, L.gb_last_error()
    keep = did >= 0
    rt, v, did = np.ascontiguousarray(rt[keep]), np.ascontiguousarray(v[keep]), np.ascontiguousarray(did[keep])
    n = len(did)
    ne = meta["sb_Ne"][0]
    t = np.ascontiguousarray(rng.integers(1, ne + 1, 64).astype(np.int32))
    zt = np.ascontiguousarray(rng.uniform(-0.3, 0.3, (64, 2)))
    dbd = np.zeros(64, np.int32)

    def fields():
        res = []
        for mode, width in ((0, 4), (1, 6), (2, 6), (3, 8)):
            out = np.zeros((n, width), complex)
            flag = np.zeros(n, np.int32)
            assert L.gb_field_points(o, mode, 2, n, rt.ctypes.data, v.ctypes.data, did.ctypes.data, out.ctypes.data,
                                     flag.ctypes.data) == 0, L.gb_last_error()
            res.append(out)
        out = np.zeros((64, 6), complex)
        assert L.gb_field_bd(o, 2, 64, dbd.ctypes.data, t.ctypes.data, zt.ctypes.data, out.ctypes.data) == 0, \
            L.gb_last_error()
        res.append(out)
        return res
    f64 = fields()
    for dd in range(len(meta["sb_Ne"])):
        assert L.gb_assemble2(o, dd, 2, prec) == 0, L.gb_last_error()
    fdf = fields()
    sc.close()
    for a, b in zip(fdf, f64):
        err = np.linalg.norm(a - b) / np.linalg.norm(b)
        assert err <= tol, err
        assert np.array_equal(a == 0, b == 0)  # the same near-boundary cutoffs
