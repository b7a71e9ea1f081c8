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
