"""GPU: siblings of the 24,576-element sphere (radius 3, n = 1.5 + 0.01i in
1.33, lambda0 = 1: the geometry and media of the 64 x 64-per-face sphere) at
8, 16 and 24 quadrangles per face.

  * sampled rows of G, H, dG, dH, dF at 8 and 16 per face against the oracle
    (reference create_cmatrix_domain, solve_bieq2.c:98-184): FP64,
    double-float and the chosen form's adaptive order <= 1e-10;
  * the chosen form's radiation force against the Mie series: the error falls
    with the mesh (measured 33 %, 3.5 %, 0.74 %: faster than h^2 between 16
    and 24 per face) and is below 1 % at 24 per face;
  * chosen form against the plain FP64 form at 16 per face: force and torque
    <= 1e-6 (the metric's tolerance); both times printed.
"""
import os
import time

import numpy as np
import pytest

from bem3_emf_b2_gb300 import meshgen
from oracle import port
from tests import _mie
from tests.test_gpu_parity_scale import _lib, _rows_check

N_IN = complex(1.5, 0.01)


def _write(wd, nf):
    os.makedirs(wd, exist_ok=True)
    nodes, elems = meshgen.cubed_sphere(nf, 3.0)
    meshgen.write_mesh(os.path.join(wd, "mesh.msh"), nodes, elems)
    meshgen.write_medium(os.path.join(wd, "medium.txt"), [N_IN])
    meshgen.write_ipw(os.path.join(wd, "ipw.txt"), [dict(lambda0=1.0, ni=1.33, power=1.0, e0x=1.0, e0y=0.0)])


def _scene(wd):
    from bem3_emf_b2_gb300 import Scene
    return Scene(os.path.join(wd, "medium.txt"), os.path.join(wd, "mesh.msh"), os.path.join(wd, "ipw.txt"))


@pytest.mark.gpu
@pytest.mark.parametrize("nf", [8, 16])
def test_sphere3_rows_match_oracle(nf, gb_build, tmp_path):
    L = _lib()
    wd = str(tmp_path)
    _write(wd, nf)
    ob = port.Obj(os.path.join(wd, "mesh.msh"), [N_IN], 1.0, 1.33)
    sc = _scene(wd)
    _rows_check(L, sc, ob, 48, 1e-10)
    sc.close()


@pytest.mark.gpu
def test_sphere3_force_converges_to_mie_and_matches_fp64(gb_build, tmp_path):
    ref = _mie.radiation_force_z(N_IN, 1.33, 3.0, 1.0)
    fz = {}
    for nf in (8, 16, 24):
        wd = str(tmp_path / ("nf%d" % nf))
        _write(wd, nf)
        sc = _scene(wd)
        t0 = time.perf_counter()
        F1, N1 = sc.step(form=1)
        t1 = time.perf_counter() - t0
        fz[nf] = F1[2]
        msg = "sphere r=3, %d per face (%d elements): chosen %.2f s, Fz %.10e (Mie %.10e, rel %.2e)" % (
            nf, 6 * nf * nf, t1, F1[2], ref, abs(F1[2] - ref) / abs(ref))
        if nf == 16:
            t0 = time.perf_counter()
            F0, N0 = sc.step(form=0)
            t0 = time.perf_counter() - t0
            v0, v1 = np.concatenate([F0, N0]), np.concatenate([F1, N1])
            d = np.linalg.norm(v1 - v0) / np.linalg.norm(v0)
            msg += "; FP64 form %.2f s, force/torque difference %.2e" % (t0, d)
            assert d <= 1e-6, d
        print(msg)
        sc.close()
    err = {nf: abs(v - ref) / abs(ref) for nf, v in fz.items()}
    print("errors against Mie %s" % err)
    assert err[24] < err[16] < err[8], err
    assert err[24] < 1e-2, err
