"""GPU: domain ids of points (reference domain_id, setup2.c:944-978) against
the oracle's restatement, on the golden sphere (bilinear quadrangles) and the
mixed cone (quadrangles and triangles): random points inside and outside,
points near the surface (element centres moved by +-1e-3 and +-1e-7 of the
element size along the normal) and points on element planes (element
centres, where the reference reports the element's domain).  The kernel
decides in FP32 where that is safe and in FP64 otherwise; the ids must be the
oracle's exactly."""
import ctypes
import os

import numpy as np
import pytest

from oracle import port
from tests._scenes import load_case, write_inputs


def _points(o, rng):
    ne = o.Ne
    c = o.corner[1:].mean(axis=1)  # element centres (corner means)
    w = o.wen[1:, 0]
    nrm = w / np.linalg.norm(w, axis=1)[:, None]
    size = np.sqrt(np.linalg.norm(w, axis=1))
    ext = np.abs(o.corner[1:].reshape(-1, 3)).max()
    pts = [rng.uniform(-1.5 * ext, 1.5 * ext, (512, 3)), c[: min(ne, 64)]]
    for f in (1e-3, -1e-3, 1e-7, -1e-7):
        k = min(ne, 64)
        pts.append(c[:k] + f * size[:k, None] * nrm[:k])
    return np.ascontiguousarray(np.concatenate(pts))


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["sphere2", "cone_mix"])
def test_domain_id_matches_oracle(case, gb_build, tmp_path):
    from bem3_emf_b2_gb300 import Scene, lib
    L = lib()
    vp, ci = ctypes.c_void_p, ctypes.c_int
    L.gb_domain_id.argtypes = [vp, ci, vp, vp]
    L.gb_domain_id.restype = ci
    meta, _ = load_case(case)
    wd = str(tmp_path)
    write_inputs(meta, wd)
    w = meta["wave"]
    o = port.Obj(os.path.join(wd, "mesh.msh"), [complex(a, b) for a, b in meta["n"]], w["lambda0"], w["ni"])
    pts = _points(o, np.random.default_rng(3))
    ref = np.asarray(o.domain_id(pts))
    sc = Scene(os.path.join(wd, "medium.txt"), os.path.join(wd, "mesh.msh"), os.path.join(wd, "ipw.txt"))
    did = np.zeros(len(pts), np.int32)
    assert L.gb_domain_id(sc.obj(), len(pts), pts.ctypes.data, did.ctypes.data) == 0
    sc.close()
    bad = np.nonzero(did != ref)[0]
    print("%s: %d points, ids %s, %d differ" % (case, len(pts), np.bincount(ref - ref.min()), len(bad)))
    assert len(bad) == 0, [(pts[i].tolist(), int(did[i]), int(ref[i])) for i in bad[:5]]
