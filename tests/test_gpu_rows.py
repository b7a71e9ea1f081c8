"""GPU: row-block assembly (gb_assemble_rows) -- the rows of a domain's
coefficient matrices into caller buffers, without the N x N matrices.

  * blocks of an odd number of rows reproduce the full-domain assembly
    (gb_assemble2) bit for bit, FP64 and the chosen form's precision;
  * on a planar-quadrangle cube (the 38,400-element cube's generator at
    6 x 6 per face, side 6, n = 1.6 in 1.33) sampled rows match the oracle
    (reference create_cmatrix_domain, solve_bieq2.c:98-184) to 1e-10.
"""
import ctypes
import os

import numpy as np
import pytest

from bem3_emf_b2_gb300 import formats, meshgen
from tests._scenes import load_case, write_inputs


def _lib():
    from bem3_emf_b2_gb300 import lib
    L = lib()
    vp, ci = ctypes.c_void_p, ctypes.c_int
    L.gb_assemble2.argtypes = [vp, ci, ci, ci]
    L.gb_assemble2.restype = ci
    L.gb_assemble_rows.argtypes = [vp, ci, ci, ci, ci, ci, vp, vp, vp, vp, vp]
    L.gb_assemble_rows.restype = ci
    L.gb_cmatrix_rows.argtypes = [vp, ci, ci, vp, vp, vp, vp, vp, vp]
    L.gb_cmatrix_rows.restype = ci
    L.gb_obj_stream.argtypes = [vp]
    L.gb_obj_stream.restype = vp
    return L


def _rows(L, o, did, row0, nrow, N, prec):
    import torch
    G = torch.zeros((nrow, N), dtype=torch.complex128, device="cuda")
    H = torch.zeros_like(G)
    dG = torch.zeros((2 * nrow, N), dtype=torch.complex128, device="cuda")
    dH = torch.zeros_like(dG)
    dF = torch.zeros((nrow, 3), dtype=torch.float64, device="cuda")
    rc = L.gb_assemble_rows(o, did, row0, nrow, 2, prec, G.data_ptr(), H.data_ptr(), dG.data_ptr(), dH.data_ptr(),
                            dF.data_ptr())
    assert rc == 0, L.gb_last_error()
    torch.cuda.ExternalStream(L.gb_obj_stream(o)).synchronize()
    return [x.cpu().numpy() for x in (G, H, dG, dH, dF)]


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["sphere2", "cone_mix"])
def test_row_blocks_reproduce_full_assembly(case, gb_build, tmp_path):
    from bem3_emf_b2_gb300 import Scene
    L = _lib()
    meta, _ = load_case(case)
    wd = str(tmp_path)
    write_inputs(meta, wd)
    sc = Scene(os.path.join(wd, "medium.txt"), os.path.join(wd, "mesh.msh"), os.path.join(wd, "ipw.txt"))
    o = sc.obj()
    for prec in (0, 3):
        for d, ne in enumerate(meta["sb_Ne"]):
            N = 4 * ne
            assert L.gb_assemble2(o, d, 2, prec) == 0, L.gb_last_error()
            rows = np.arange(N, dtype=np.int32)
            full = [np.zeros((N, N), complex), np.zeros((N, N), complex), np.zeros((2 * N, N), complex),
                    np.zeros((2 * N, N), complex), np.zeros((N, 3))]
            assert L.gb_cmatrix_rows(o, d, N, rows.ctypes.data, *[x.ctypes.data for x in full]) == 0
            blk = [[], [], [], [], []]
            for r0 in range(0, N, 7):
                part = _rows(L, o, d, r0, min(7, N - r0), N, prec)
                for i in range(5):
                    blk[i].append(part[i])
            for name, a, b in zip(("G", "H", "dG", "dH", "dF"), [np.concatenate(x) for x in blk], full):
                assert np.array_equal(a, b), "precision %d domain %d %s" % (prec, d, name)
    assert L.gb_assemble_rows(o, 0, -1, 3, 2, 0, 1, 1, 1, 1, 1) != 0
    assert L.gb_assemble_rows(o, 0, 0, 4 * meta["sb_Ne"][0] + 1, 2, 0, 1, 1, 1, 1, 1) != 0
    sc.close()


@pytest.mark.gpu
def test_cube_rows_match_oracle(gb_build, tmp_path):
    from bem3_emf_b2_gb300 import Scene
    from oracle import port
    L = _lib()
    wd = str(tmp_path)
    nodes, elems = meshgen.cube(6, 6.0)
    meshgen.write_mesh(os.path.join(wd, "mesh.msh"), nodes, elems)
    meshgen.write_medium(os.path.join(wd, "medium.txt"), [1.6])
    meshgen.write_ipw(os.path.join(wd, "ipw.txt"), [dict(lambda0=1.0, ni=1.33, power=1.0, e0x=1.0, e0y=0.0)])
    ob = port.Obj(os.path.join(wd, "mesh.msh"), [1.6], 1.0, 1.33)
    sc = Scene(os.path.join(wd, "medium.txt"), os.path.join(wd, "mesh.msh"), os.path.join(wd, "ipw.txt"))
    o = sc.obj()
    N = 4 * ob.Ne
    for d in range(2):
        rows = np.unique(np.linspace(0, N - 1, 40).astype(np.int32))
        ref = ob.rows(d, rows)
        for prec in (0, 3):
            got = [[], [], [], [], []]
            for r in rows:
                part = _rows(L, o, d, int(r), 1, N, prec)
                for i in range(5):
                    got[i].append(part[i])
            for name, a, b in zip(("G", "H", "dG", "dH", "dF"), [np.concatenate(x) for x in got], ref):
                err = formats.rel_fro(a, b)
                assert err <= 1e-10, "precision %d domain %d %s: %g" % (prec, d, name, err)
    sc.close()


@pytest.mark.gpu
def test_work_list_assembly_matches_per_domain(gb_build, tmp_path):
    """gb_assemble_objects (every domain of several objects of uneven size in
    one launch per phase) gives bit for bit the matrices of gb_assemble2 per
    domain, FP64 and the chosen form's precision."""
    from bem3_emf_b2_gb300 import Scene
    L = _lib()
    vp, ci = ctypes.c_void_p, ctypes.c_int
    L.gb_assemble_objects.argtypes = [vp, ci, ci, ci]
    L.gb_assemble_objects.restype = ci
    L.gb_cmatrix_download.argtypes = [vp, ci, vp, vp, vp, vp, vp]
    scenes, metas = [], []
    for case in ("sphere2", "cone_mix", "cone_tri"):
        meta, _ = load_case(case)
        wd = os.path.join(str(tmp_path), case)
        os.makedirs(wd)
        write_inputs(meta, wd)
        scenes.append(Scene(os.path.join(wd, "medium.txt"), os.path.join(wd, "mesh.msh"), os.path.join(wd, "ipw.txt")))
        metas.append(meta)
    objs = (ctypes.c_void_p * len(scenes))(*[s.obj() for s in scenes])

    def download(o, meta):
        out = []
        for d, ne in enumerate(meta["sb_Ne"]):
            N = 4 * ne
            m = [np.zeros((N, N), complex), np.zeros((N, N), complex), np.zeros((2 * N, N), complex),
                 np.zeros((2 * N, N), complex), np.zeros((N, 3))]
            assert L.gb_cmatrix_download(o, d, *[x.ctypes.data for x in m]) == 0
            out.append(m)
        return out
    for prec in (0, 3):
        ref = []
        for sc, meta in zip(scenes, metas):
            for d in range(len(meta["sb_Ne"])):
                assert L.gb_assemble2(sc.obj(), d, 2, prec) == 0, L.gb_last_error()
            ref.append(download(sc.obj(), meta))
        assert L.gb_assemble_objects(ctypes.cast(objs, vp), len(scenes), 2, prec) == 0, L.gb_last_error()
        for sc, meta, r in zip(scenes, metas, ref):
            got = download(sc.obj(), meta)
            for d in range(len(r)):
                for a, b in zip(got[d], r[d]):
                    assert np.array_equal(a, b), (meta["case"], prec, d)
    for sc in scenes:
        sc.close()
