"""GPU: the sphere against the Mie series.  The radiation force of the
dielectric sphere (radius 1, n = 1.5 in 1.33, lambda0 = 1, the bench's
scene) computed by the chosen form on cubed spheres of 8, 12 and 16
quadrangles per face must converge to the Mie value: errors decreasing with
the mesh, and the Richardson extrapolation of the two finest meshes (error
~ h^2 for the bilinear elements) within 0.5 % of the Mie series; the
transverse force components vanish by symmetry."""
import os

import numpy as np
import pytest

from tests import _mie


@pytest.mark.gpu
def test_sphere_force_converges_to_mie(gb_build, tmp_path):
    from bem3_emf_b2_gb300 import Scene, meshgen
    ref = _mie.radiation_force_z(1.5, 1.33, 1.0, 1.0)
    fz = {}
    for nf in (8, 12, 16):
        wd = str(tmp_path / ("nf%d" % nf))
        os.makedirs(wd)
        nodes, elems = meshgen.cubed_sphere(nf, 1.0)
        meshgen.write_mesh(os.path.join(wd, "mesh.msh"), nodes, elems)
        meshgen.write_medium(os.path.join(wd, "medium.txt"), [1.5])
        meshgen.write_ipw(os.path.join(wd, "ipw.txt"), [dict(lambda0=1.0, ni=1.33, power=1.0, e0x=1.0, e0y=0.0)])
        sc = Scene(os.path.join(wd, "medium.txt"), os.path.join(wd, "mesh.msh"), os.path.join(wd, "ipw.txt"))
        F, N = sc.step(form=1)
        sc.close()
        assert abs(F[0]) <= 1e-6 * abs(F[2]) and abs(F[1]) <= 1e-6 * abs(F[2])
        fz[nf] = F[2]
    err = {nf: abs(v - ref) / ref for nf, v in fz.items()}
    assert err[16] < err[12] < err[8], err
    rich = (fz[16] * 16 ** 2 - fz[12] * 12 ** 2) / (16 ** 2 - 12 ** 2)
    assert abs(rich - ref) / ref <= 5e-3, (fz, ref, rich)
