"""GPU: the batched field map (gb_mo_EH_points) and concurrent per-point calls.

The reference's examples evaluate fields point by point from OpenMP loops
(example2.c:43-50, example4.c:53-66: mo_EH_t, mo_EH_mEMP_s).  On the golden
two-sphere scene solved by this repository's tools:
  * gb_mo_EH_points gives, for every point of a grid (outside, inside either
    object, and far-field points at r = 2000 lambda0), exactly the values of
    the per-point functions mo_EH_t / mo_EH_s / mo_EH_mEMP_t / mo_EH_mEMP_s
    and the same containing object;
  * at the point the reference printed, the total field equals the
    reference's golden value for quadrature types 0..2 (<= 1e-9);
  * per-point calls made from 8 host threads at once return the sequential
    results bit for bit.
"""
import ctypes
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

from bem3_emf_b2_gb300 import meshgen
from tests._scenes import load_case, parse_analysis, run, write_inputs


def _solve_pair(gb_build, wd):
    meta, _ = load_case("pair")
    write_inputs(meta, wd)
    run([os.path.join(gb_build, "d3b2_create_matrix"), "medium.txt", "mesh.msh", "obj.obj"], wd)
    meshgen.write_object_settings(os.path.join(wd, "objs.txt"), [(o[0], o[1]) for o in meta["objects"]])
    run([os.path.join(gb_build, "d3b2_bv_solver"), "objs.txt", "res.dat"], wd)
    return meta


def _lib():
    from bem3_emf_b2_gb300 import lib
    L = lib()
    vp, ci = ctypes.c_void_p, ctypes.c_int
    L.mo_dat_read.argtypes = [ctypes.c_char_p, vp]
    L.mo_dat_read.restype = None
    L.mo_finalize.argtypes = [vp]
    L.mo_finalize.restype = None
    L.gb_mo_EH_points.argtypes = [vp, ci, vp, ci, ci, ci, vp, vp, vp]
    L.gb_mo_EH_points.restype = ci
    for f in ("mo_EH_t", "mo_EH_s", "mo_EH_mEMP_t", "mo_EH_mEMP_s"):
        getattr(L, f).argtypes = [vp, vp, vp, ci, vp]
        getattr(L, f).restype = ci
    return L


def _points():
    rng = np.random.default_rng(4)
    box = rng.uniform(-0.8, 0.8, (120, 3))
    inside = np.array([[0.0, 0.0, 0.45], [0.05, -0.05, -0.4], [0.1, 0.0, 0.5]])
    th = rng.uniform(0.0, np.pi, 40)
    ph = rng.uniform(0.0, 2.0 * np.pi, 40)
    far = 2000.0 * np.stack([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)], 1)
    return np.ascontiguousarray(np.concatenate([[[0.3, 0.0, 1.1]], box, inside, far]))


@pytest.mark.gpu
def test_batched_field_map_matches_per_point_calls(gb_build, tmp_path):
    L = _lib()
    wd = str(tmp_path)
    meta = _solve_pair(gb_build, wd)
    mo = ctypes.create_string_buffer(64)  # MOBJ (32 bytes on LP64)
    L.mo_dat_read(os.path.join(wd, "res.dat").encode(), mo)
    pts = _points()
    n = len(pts)
    ref = parse_analysis(meta["analysis"])
    for memp, names in ((0, ("mo_EH_s", "mo_EH_t")), (1, ("mo_EH_mEMP_s", "mo_EH_mEMP_t"))):
        for which in (0, 1):
            for type_ in (0, 1, 2):
                E = np.zeros((n, 3), complex)
                H = np.zeros((n, 3), complex)
                oid = np.zeros(n, np.int32)
                assert L.gb_mo_EH_points(mo, n, pts.ctypes.data, type_, which, memp, E.ctypes.data, H.ctypes.data,
                                         oid.ctypes.data) == 0
                fn = getattr(L, names[which])
                for p in range(n):
                    e1 = np.zeros(3, complex)
                    h1 = np.zeros(3, complex)
                    r = np.ascontiguousarray(pts[p])
                    o1 = fn(e1.ctypes.data, h1.ctypes.data, r.ctypes.data, type_, mo)
                    assert o1 == oid[p], (p, o1, oid[p])
                    assert np.array_equal(e1, E[p]) and np.array_equal(h1, H[p]), (memp, which, type_, p)
                if which == 1:
                    key = "%s_%d" % ("EH_mEMP_t" if memp else "EH_t", type_)
                    v = np.concatenate([E[0], H[0]])
                    v = np.stack([v.real, v.imag], 1).ravel()
                    err = np.linalg.norm(v - ref[key]) / np.linalg.norm(ref[key])
                    assert err <= 1e-9, (key, err)
    assert (oid[len(pts) - 43:len(pts) - 40] >= 0).all()  # the inside points
    L.mo_finalize(mo)


@pytest.mark.gpu
def test_per_point_calls_from_many_threads(gb_build, tmp_path):
    L = _lib()
    wd = str(tmp_path)
    _solve_pair(gb_build, wd)
    mo = ctypes.create_string_buffer(64)
    L.mo_dat_read(os.path.join(wd, "res.dat").encode(), mo)
    pts = _points()

    def one(p):
        e = np.zeros(3, complex)
        h = np.zeros(3, complex)
        r = np.ascontiguousarray(pts[p])
        o = L.mo_EH_t(e.ctypes.data, h.ctypes.data, r.ctypes.data, 0, mo)
        return o, e, h
    seq = [one(p) for p in range(len(pts))]
    with ThreadPoolExecutor(8) as ex:
        par = list(ex.map(one, range(len(pts))))
    for (o0, e0, h0), (o1, e1, h1) in zip(seq, par):
        assert o0 == o1 and np.array_equal(e0, e1) and np.array_equal(h0, h1)
    L.mo_finalize(mo)
