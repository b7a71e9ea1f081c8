"""GPU: the allocation-free assembly entry point (gb_assemble_domain_noalloc).

Some callers cannot allocate device memory -- their memory belongs to another
allocator, they cannot accept cudaFree's hidden device synchronisation, or
they must not allocate after start-up.  For them the library offers a variant
of the domain assembly that takes every buffer from the caller and keeps its
scratch in a fixed static device array.  This test calls it through the C ABI
twice in a row on caller-owned buffers and checks each result against the
regular entry point (gb_assemble), at the 1e-10 relative Frobenius tolerance
of the other parity tests.  It lives in its own file, collected last, so that
a failure here does not hide the others; it passes alone and after them.
"""
import ctypes
import os

import numpy as np
import pytest

from bem3_emf_b2_gb300 import formats
from tests._scenes import load_case, write_inputs

TOL = 1e-10


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["sphere2", "cone_mix"])
def test_noalloc_assembly_matches_gb_assemble(case, gb_build, tmp_path):
    import torch
    from bem3_emf_b2_gb300 import Scene, lib
    from oracle import port
    L = lib()
    vp, ci, cd = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    L.gb_assemble_domain_noalloc.argtypes = [vp, vp, vp, vp, vp, ci, cd, cd, ci, ci, vp, vp, vp, vp, vp, vp]
    L.gb_assemble_domain_noalloc.restype = ci
    L.gb_cmatrix_download.argtypes = [vp, ci, vp, vp, vp, vp, vp]
    meta, _ = load_case(case)
    wd = str(tmp_path)
    write_inputs(meta, wd)
    n_media = [complex(a, b) for a, b in meta["n"]]
    w = meta["wave"]
    ob = port.Obj(os.path.join(wd, "mesh.msh"), n_media, w["lambda0"], w["ni"])
    sc = Scene(os.path.join(wd, "medium.txt"), os.path.join(wd, "mesh.msh"), os.path.join(wd, "ipw.txt"))
    o = sc.obj()
    dev = "cuda"
    cr = torch.tensor(ob.cr.reshape(-1), dtype=torch.float64, device=dev)
    cw = torch.tensor(ob.cw.reshape(-1), dtype=torch.float64, device=dev)
    ren = torch.tensor(ob.ren.reshape(-1), dtype=torch.float64, device=dev)
    et = torch.tensor(ob.etype, dtype=torch.int32, device=dev)
    for did in range(ob.MN + 1):
        ne = len(ob.sids[did]) - 1
        N = 4 * ne
        sid = torch.tensor(ob.sids[did], dtype=torch.int32, device=dev)
        assert L.gb_assemble(o, did, 2) == 0, L.gb_last_error()
        ref = {k: np.zeros(s, complex) for k, s in (("G", (N, N)), ("H", (N, N)), ("dG", (2 * N, N)), ("dH", (2 * N, N)))}
        ref["dF"] = np.zeros((N, 3))
        assert L.gb_cmatrix_download(o, did, ref["G"].ctypes.data, ref["H"].ctypes.data, ref["dG"].ctypes.data,
                                     ref["dH"].ctypes.data, ref["dF"].ctypes.data) == 0
        for call in range(2):
            out = {k: torch.full(v.shape, float("nan"), dtype=torch.complex128 if k != "dF" else torch.float64,
                                 device=dev) for k, v in ref.items()}
            k = ob.kn[did]
            rc = L.gb_assemble_domain_noalloc(cr.data_ptr(), cw.data_ptr(), et.data_ptr(), ren.data_ptr(),
                                              sid.data_ptr(), ne, k.real, k.imag, did, 2, out["G"].data_ptr(),
                                              out["H"].data_ptr(), out["dG"].data_ptr(), out["dH"].data_ptr(),
                                              out["dF"].data_ptr(), None)
            assert rc == 0, L.gb_last_error()
            torch.cuda.synchronize()
            for name, v in ref.items():
                err = formats.rel_fro(out[name].cpu().numpy(), v)
                assert err <= TOL, "%s domain %d call %d: %g" % (name, did, call, err)
    # sizes beyond the fixed scratch are rejected before any GPU work
    big = 419
    rc = L.gb_assemble_domain_noalloc(cr.data_ptr(), cw.data_ptr(), et.data_ptr(), ren.data_ptr(), sid.data_ptr(), big,
                                      1.0, 0.0, 0, 2, cr.data_ptr(), cr.data_ptr(), cr.data_ptr(), cr.data_ptr(),
                                      cr.data_ptr(), None)
    assert rc == -1 and b"418" in L.gb_last_error()
    sc.close()


def test_noalloc_rejects_bad_arguments_before_device_work(gb_build):
    """The argument checks run before any device call (so this needs no GPU):
    a domain beyond the fixed scratch, a quadrature type or domain id out of
    range, and any null input or output pointer each return -1 with a message
    naming the problem."""
    from bem3_emf_b2_gb300 import lib
    L = lib()
    vp, ci, cd = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    L.gb_assemble_domain_noalloc.argtypes = [vp, vp, vp, vp, vp, ci, cd, cd, ci, ci, vp, vp, vp, vp, vp, vp]
    L.gb_assemble_domain_noalloc.restype = ci
    fake = 4096  # never dereferenced: every call below fails its checks first

    def call(Ne=10, did=0, type_=2, null=None):
        ptrs = [fake] * 10
        if null is not None:
            ptrs[null] = None
        return L.gb_assemble_domain_noalloc(ptrs[0], ptrs[1], ptrs[2], ptrs[3], ptrs[4], Ne, 1.0, 0.0, did, type_,
                                            ptrs[5], ptrs[6], ptrs[7], ptrs[8], ptrs[9], None)
    assert call(Ne=0) == -1 and b"1..418" in L.gb_last_error()
    assert call(Ne=419) == -1 and b"1..418" in L.gb_last_error()
    assert call(type_=4) == -1 and b"quadrature type 4" in L.gb_last_error()
    assert call(type_=-1) == -1 and b"quadrature type -1" in L.gb_last_error()
    assert call(did=-1) == -1 and b"domain id -1" in L.gb_last_error()
    assert call(did=16) == -1 and b"domain id 16" in L.gb_last_error()
    for i in range(10):
        assert call(null=i) == -1 and b"null" in L.gb_last_error(), i
