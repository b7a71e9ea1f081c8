"""GPU: the multi-object scene API (gbh_mscene_*) on the two-sphere golden
scene -- both objects assembled, factorised and iterated on the device
without intermediate files.  The plain FP64 form must reproduce the
reference's force and torque on each object (golden, <= 1e-9 relative on the
combined vector), the chosen form to <= 1e-6, and the iteration must stop at
the reference's count (the reference's stopping rule on the same cc)."""
import os

import numpy as np
import pytest

from tests._scenes import load_case, parse_analysis, write_inputs


@pytest.mark.gpu
@pytest.mark.parametrize("form,tol", [(0, 1e-9), (1, 1e-6)])
def test_mscene_pair_matches_reference(form, tol, gb_build, tmp_path):
    from bem3_emf_b2_gb300 import MultiScene
    meta, _ = load_case("pair")
    wd = str(tmp_path)
    write_inputs(meta, wd)
    objs = meta["objects"]
    n = len(objs)
    med = [os.path.join(wd, "medium.txt")] * n
    msh = [os.path.join(wd, "mesh.msh")] * n
    tv = np.array([o[1] for o in objs], float)
    sc = MultiScene(med, msh, os.path.join(wd, "ipw.txt"), tv=tv)
    F, N = sc.step(form=form, rc=np.zeros((n, 3)))
    it, cc = sc.iteration()
    sc.close()
    gold = parse_analysis(meta["analysis"])
    for m in range(n):
        ref = gold["force_%d_0" % m]
        v = np.concatenate([F[m], N[m]])
        err = np.linalg.norm(v - ref) / np.linalg.norm(ref)
        assert err <= tol, "object %d form %d: force/torque relative error %g" % (m, form, err)
    assert it == len(meta["cc"]) + 1, (it, len(meta["cc"]))


@pytest.mark.gpu
def test_two_cone_scene_chosen_matches_fp64(gb_build, tmp_path):
    """The two-cone scene of the bench's --workload cones (cone 2 rotated pi
    about x and shifted 1.5 along x, circular polarisation) on a reduced mesh
    (m = 5: 300 triangles per cone): the chosen form reproduces the plain FP64
    form's force and torque on each cone to <= 1e-9 relative, with the same
    number of multiple-scattering iterations."""
    import bench
    from bem3_emf_b2_gb300 import MultiScene
    wd = str(tmp_path)
    bench.write_cones(wd, 5)
    med = [os.path.join(wd, "medium.txt")] * 2
    msh = [os.path.join(wd, "cone.msh")] * 2
    rv = np.array([[1.0, 0.0, 0.0], [1.0, 0.0, 0.0]])
    th = np.array([0.0, np.pi])
    tv = np.array([[0.0, 0.0, 0.0], [1.5, 0.0, 0.0]])
    sc = MultiScene(med, msh, os.path.join(wd, "ipw.txt"), rv=rv, th=th, tv=tv)
    F64, N64 = sc.step(form=0)
    it64, _ = sc.iteration()
    F32, N32 = sc.step(form=1)
    it32, _ = sc.iteration()
    sc.close()
    assert it64 == it32
    for m in range(2):
        v64 = np.concatenate([F64[m], N64[m]])
        v32 = np.concatenate([F32[m], N32[m]])
        err = np.linalg.norm(v32 - v64) / np.linalg.norm(v64)
        assert err <= 1e-9, "cone %d: %g" % (m, err)
