"""GB300-native BEM hot path of bem3_emf_b2 (boundary-integral assembly, dense
complex LU/inverse, multi-object iteration, field and force sums) behind the
reference's C API.

The product is the in-tree shared library ``_build/libbem3gb.so`` (C host
library + sm_103a CUDA kernels, C ABI in include/gb_bem.h, include/gb_scene.h,
include/bem3_emf_b2.h) and the drop-in tools next to it.  This module only
loads that library for Python callers (tests, bench): there is no Python or
CPU implementation of the kernels, and a missing library is an error.
"""
import ctypes
import os

PKG = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(PKG, "_build")
LIBPATH = os.path.join(BUILD, "libbem3gb.so")

_lib = None


def lib():
    """The loaded libbem3gb.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIBPATH):
        raise RuntimeError("libbem3gb.so is not built (run bem3_emf_b2_gb300.build.build()); "
                           "the BEM kernels have no fallback")
    L = ctypes.CDLL(LIBPATH)
    c_int, c_dbl, vp = ctypes.c_int, ctypes.c_double, ctypes.c_void_p
    L.gb_last_error.restype = ctypes.c_char_p
    L.gb_device_count.restype = c_int
    L.gb_zgesv.argtypes = [c_int, c_int, vp, vp]
    L.gb_zgesv.restype = c_int
    L.gbh_scene_open.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p]
    L.gbh_scene_open.restype = vp
    L.gbh_scene_step.argtypes = [vp, c_int, c_int, vp, vp, vp]
    L.gbh_scene_step.restype = c_int
    L.gbh_scene_drop_device.argtypes = [vp]
    L.gbh_scene_h2d_bytes.argtypes = [vp]
    L.gbh_scene_h2d_bytes.restype = ctypes.c_size_t
    L.gbh_scene_d2h_bytes.argtypes = [vp]
    L.gbh_scene_d2h_bytes.restype = ctypes.c_size_t
    L.gbh_scene_close.argtypes = [vp]
    L.gbh_scene_stream.argtypes = [vp]
    L.gbh_scene_stream.restype = vp
    L.gb_launch_count.restype = ctypes.c_ulonglong
    L.gbh_scene_obj.argtypes = [vp]
    L.gbh_scene_obj.restype = vp
    for name in ("gb_assemble",):
        getattr(L, name).argtypes = [vp, c_int, c_int]
    for name in ("gb_invA_compute", "gb_factor_mixed", "gb_solve_mEMP", "gb_solve_EH"):
        getattr(L, name).argtypes = [vp]
        getattr(L, name).restype = c_int
    L.gb_ir_info.argtypes = [vp, vp, vp]
    L.gbh_mscene_open.argtypes = [c_int, vp, vp, ctypes.c_char_p, vp, vp, vp]
    L.gbh_mscene_open.restype = vp
    L.gbh_mscene_step.argtypes = [vp, c_int, c_int, vp, vp, vp]
    L.gbh_mscene_step.restype = c_int
    for name in ("gbh_mscene_drop_device", "gbh_mscene_close"):
        getattr(L, name).argtypes = [vp]
        getattr(L, name).restype = None
    for name in ("gbh_mscene_h2d_bytes", "gbh_mscene_d2h_bytes"):
        getattr(L, name).argtypes = [vp]
        getattr(L, name).restype = ctypes.c_size_t
    L.gbh_set_quiet.argtypes = [c_int]
    L.gbh_set_quiet.restype = None
    L.gbh_last_iteration.argtypes = [vp, vp]
    L.gbh_last_iteration.restype = None
    L.gbh_mscene_phase_times.argtypes = [vp]
    L.gbh_mscene_phase_times.restype = None
    L.gb_ktime_enable.argtypes = [c_int]
    L.gb_ktime_enable.restype = None
    L.gb_ktime_read.argtypes = [vp, vp, vp, vp]
    L.gb_ktime_read.restype = c_int
    L.gb_ktime_list.argtypes = [c_int, vp]
    L.gb_ktime_list.restype = c_int
    L.gb_form_precision.argtypes = [c_int]
    L.gb_form_precision.restype = c_int
    _lib = L
    return L


def last_error():
    return lib().gb_last_error().decode()


def ktime_list():
    """[(device ms, M, N, K)] of each recorded tensor-core launch (not cleared)"""
    import numpy as np
    L = lib()
    n = L.gb_ktime_list(0, None)
    if n < 0:
        raise RuntimeError(last_error())
    rec = np.zeros(4 * max(n, 1))
    if L.gb_ktime_list(n, rec.ctypes.data) != n:
        raise RuntimeError(last_error())
    return [tuple(rec[4 * i:4 * i + 4]) for i in range(n)]


def ktime_read():
    """(device ms, launches, complex-equivalent flops, HBM bytes) of the
    tensor-core trailing-update launches recorded since gb_ktime_enable(1)."""
    ms, n, fl, by = ctypes.c_double(), ctypes.c_long(), ctypes.c_double(), ctypes.c_double()
    if lib().gb_ktime_read(ctypes.byref(ms), ctypes.byref(n), ctypes.byref(fl), ctypes.byref(by)) != 0:
        raise RuntimeError(last_error())
    return ms.value, n.value, fl.value, by.value


class Scene:
    """A single-object scene set up from the reference's input files and
    solved on the GPU (gb_scene.h)."""

    def __init__(self, medium, mesh, ipw):
        L = lib()
        self.h = L.gbh_scene_open(medium.encode(), mesh.encode(), ipw.encode())
        if not self.h:
            raise RuntimeError("gbh_scene_open failed")

    def step(self, form=1, type_=2, rc=(0.0, 0.0, 0.0)):
        import numpy as np
        rcv = np.ascontiguousarray(rc, float)
        F = np.zeros(3)
        N = np.zeros(3)
        rc_ = lib().gbh_scene_step(self.h, form, type_, rcv.ctypes.data, F.ctypes.data, N.ctypes.data)
        if rc_ != 0:
            raise RuntimeError("gbh_scene_step failed: %s" % last_error())
        return F, N

    def drop_device(self):
        lib().gbh_scene_drop_device(self.h)

    def h2d_bytes(self):
        return int(lib().gbh_scene_h2d_bytes(self.h))

    def d2h_bytes(self):
        return int(lib().gbh_scene_d2h_bytes(self.h))

    def stream(self):
        return lib().gbh_scene_stream(self.h)

    def obj(self):
        return lib().gbh_scene_obj(self.h)

    def ir_info(self):
        it = ctypes.c_int(0)
        rr = ctypes.c_double(0.0)
        lib().gb_ir_info(self.obj(), ctypes.byref(it), ctypes.byref(rr))
        return it.value, rr.value

    def close(self):
        if self.h:
            lib().gbh_scene_close(self.h)
            self.h = None


class MultiScene:
    """A multi-object scene (gbh_mscene_*): objects placed by rotation (axis
    rv, angle th) and translation tv, solved together by the multiple-
    scattering iteration on the GPU."""

    def __init__(self, media, meshes, ipw, rv=None, th=None, tv=None, quiet=True):
        import numpy as np
        L = lib()
        n = len(meshes)
        self.n = n
        self._keep = [m.encode() for m in media] + [m.encode() for m in meshes]
        med = (ctypes.c_char_p * n)(*self._keep[:n])
        msh = (ctypes.c_char_p * n)(*self._keep[n:])
        self._rv = np.ascontiguousarray(rv if rv is not None else np.tile([1.0, 0.0, 0.0], n), float).reshape(-1)
        self._th = np.ascontiguousarray(th if th is not None else np.zeros(n), float).reshape(-1)
        self._tv = np.ascontiguousarray(tv if tv is not None else np.zeros(3 * n), float).reshape(-1)
        L.gbh_set_quiet(1 if quiet else 0)
        self.h = L.gbh_mscene_open(n, ctypes.cast(med, ctypes.c_void_p), ctypes.cast(msh, ctypes.c_void_p), ipw.encode(),
                                   self._rv.ctypes.data, self._th.ctypes.data, self._tv.ctypes.data)
        if not self.h:
            raise RuntimeError("gbh_mscene_open failed")

    def step(self, form=1, type_=2, rc=None):
        """rc: torque reference points (n x 3); default the translation points"""
        import numpy as np
        F = np.zeros(3 * self.n)
        N = np.zeros(3 * self.n)
        rcp = None
        if rc is not None:
            rca = np.ascontiguousarray(rc, float).reshape(-1)
            rcp = rca.ctypes.data
        if lib().gbh_mscene_step(self.h, form, type_, rcp, F.ctypes.data, N.ctypes.data) != 0:
            raise RuntimeError("gbh_mscene_step failed: %s" % last_error())
        return F.reshape(self.n, 3), N.reshape(self.n, 3)

    def beams(self, beams_file, form=1, type_=2, rc=None):
        """every plane wave of beams_file as its own incident field
        (gbh_mscene_beams): force, torque [nbeam][n][3]"""
        import numpy as np
        L = lib()
        vp, ci = ctypes.c_void_p, ctypes.c_int
        L.gbh_mscene_beams.argtypes = [vp, ci, ci, ctypes.c_char_p, vp, vp, vp, vp]
        L.gbh_mscene_beams.restype = ci
        with open(beams_file) as f:
            nmax = int([l for l in f.read().splitlines() if l.strip() and not l.startswith("#")][0].split()[0])
        F = np.zeros((nmax, self.n, 3))
        N = np.zeros((nmax, self.n, 3))
        nb = ctypes.c_int(0)
        rcp = None
        if rc is not None:
            rca = np.ascontiguousarray(rc, float).reshape(-1)
            rcp = rca.ctypes.data
        if L.gbh_mscene_beams(self.h, form, type_, beams_file.encode(), rcp, F.ctypes.data, N.ctypes.data,
                              ctypes.byref(nb)) != 0:
            raise RuntimeError("gbh_mscene_beams failed: %s" % last_error())
        return F[:nb.value], N[:nb.value]

    def phase_times(self):
        """(assembly, factorisation, iteration + E/H, force) seconds of the last step"""
        import numpy as np
        t = np.zeros(4)
        lib().gbh_mscene_phase_times(t.ctypes.data)
        return dict(zip(("assembly", "factorisation", "iteration_eh", "force"), t.tolist()))

    def iteration(self):
        it, cc = ctypes.c_int(0), ctypes.c_double(0.0)
        lib().gbh_last_iteration(ctypes.byref(it), ctypes.byref(cc))
        return it.value, cc.value

    def drop_device(self):
        lib().gbh_mscene_drop_device(self.h)

    def field_map(self, pts, type_=2, which=0, memp=1):
        """E, H (n x 3 complex) and containing object at points pts (n x 3) of the
        solved scene (gb_mo_EH_points): scattered (which 0), total (1) or
        incident (2) field; memp 1 the potential-derivative (far-field) form"""
        import numpy as np
        L = lib()
        vp, ci = ctypes.c_void_p, ctypes.c_int
        L.gb_mo_EH_points.argtypes = [vp, ci, vp, ci, ci, ci, vp, vp, vp]
        L.gb_mo_EH_points.restype = ci
        p = np.ascontiguousarray(pts, float).reshape(-1, 3)
        n = len(p)
        E = np.zeros((n, 3), complex)
        H = np.zeros((n, 3), complex)
        oid = np.zeros(n, np.int32)
        if L.gb_mo_EH_points(self.h, n, p.ctypes.data, type_, which, memp, E.ctypes.data, H.ctypes.data,
                             oid.ctypes.data) != 0:
            raise RuntimeError("gb_mo_EH_points failed: %s" % last_error())
        return E, H, oid

    def h2d_bytes(self):
        return int(lib().gbh_mscene_h2d_bytes(self.h))

    def d2h_bytes(self):
        return int(lib().gbh_mscene_d2h_bytes(self.h))

    def close(self):
        if self.h:
            lib().gbh_mscene_close(self.h)
            self.h = None
