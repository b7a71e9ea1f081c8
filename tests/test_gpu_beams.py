"""GPU: many incident beams as right-hand sides of one multi-object scene
(gbh_mscene_beams) -- a seeded sibling of the 48-object, 32-beam scene:
spheres, cubes and cones of random size, index and orientation, plane waves
of random direction and polarisation.

  * each beam's force and torque equal those of a separate scene step whose
    ipw.txt holds only that wave (the reference sums the waves of ipw.txt,
    so one beam is one reference run): <= 1e-10;
  * the chosen form's beams match the plain FP64 form's: <= 1e-9;
  * for one beam, the converged boundary values of every object satisfy the
    oracle's coupled equations with the incident field rebuilt by the oracle
    (plane wave + the other objects' scattered potentials): relative
    residual over sampled rows <= 1e-9.
"""
import ctypes
import os

import numpy as np
import pytest

from bem3_emf_b2_gb300 import formats, meshgen
from oracle import port

NOBJ, NBEAM = 3, 4


def _write(wd):
    objs = meshgen.batch_scene(5, NOBJ, box=5.0, size=(0.4, 0.8), elems=(60, 220))
    med, msh = [], []
    for i, o in enumerate(objs):
        meshgen.write_mesh(os.path.join(wd, "o%d.msh" % i), o["nodes"], o["elems"])
        meshgen.write_medium(os.path.join(wd, "m%d.txt" % i), [o["n"]])
        med.append(os.path.join(wd, "m%d.txt" % i))
        msh.append(os.path.join(wd, "o%d.msh" % i))
    waves = meshgen.random_waves(9, NBEAM)
    meshgen.write_ipw(os.path.join(wd, "beams.txt"), waves)
    for b, w in enumerate(waves):
        meshgen.write_ipw(os.path.join(wd, "beam%d.txt" % b), [w])
    return objs, med, msh, waves


@pytest.mark.gpu
def test_beams_match_single_beam_scenes_and_fp64(gb_build, tmp_path):
    from bem3_emf_b2_gb300 import MultiScene
    wd = str(tmp_path)
    objs, med, msh, waves = _write(wd)
    sc = MultiScene(med, msh, os.path.join(wd, "beams.txt"))
    F1, N1 = sc.beams(os.path.join(wd, "beams.txt"), form=1)
    F0, N0 = sc.beams(os.path.join(wd, "beams.txt"), form=0)
    sc.close()
    assert F1.shape == (NBEAM, NOBJ, 3)
    for b in range(NBEAM):
        one = MultiScene(med, msh, os.path.join(wd, "beam%d.txt" % b))
        Fb, Nb = one.step(form=1)
        one.close()
        v = np.concatenate([Fb.ravel(), Nb.ravel()])
        d = np.linalg.norm(np.concatenate([F1[b].ravel(), N1[b].ravel()]) - v) / np.linalg.norm(v)
        assert d <= 1e-10, (b, d)
        d0 = np.linalg.norm(np.concatenate([F0[b].ravel() - F1[b].ravel(), N0[b].ravel() - N1[b].ravel()])) / \
            np.linalg.norm(np.concatenate([F0[b].ravel(), N0[b].ravel()]))
        assert d0 <= 1e-9, (b, d0)
    # the beams differ: they are separate right-hand sides, not one summed field
    assert np.linalg.norm(F1[0] - F1[1]) > 1e-3 * np.linalg.norm(F1[0])


@pytest.mark.gpu
def test_beam_solution_satisfies_oracle_equations(gb_build, tmp_path):
    from bem3_emf_b2_gb300 import MultiScene, lib
    L = lib()
    L.mo_dat_write.argtypes = [ctypes.c_char_p, ctypes.c_void_p]
    L.mo_dat_write.restype = None
    wd = str(tmp_path)
    objs, med, msh, waves = _write(wd)
    sc = MultiScene(med, msh, os.path.join(wd, "beam1.txt"))
    sc.step(form=1)
    L.mo_dat_write(os.path.join(wd, "res.dat").encode(), sc.h)
    sc.close()
    dat = formats.read_dat(os.path.join(wd, "res.dat"))
    obs = [port.Obj(msh[i], [o["n"]], 1.0, 1.33) for i, o in enumerate(objs)]
    bvs = [[dict(U=sb["U"], dU=sb["dU"], E=sb["E"], dE=sb["dE"], H=sb["H"], dH=sb["dH"]) for sb in o["sb"]]
           for o in dat]
    for m, ob in enumerate(obs):
        Ui, dUi = port.incident(ob, [waves[1]])
        ext = np.nonzero(ob.md[1:] == 0)[0] + 1
        pts = ob.ren[ext].reshape(-1, 3)
        v = (ob.wen[ext] / np.linalg.norm(ob.wen[ext], axis=2)[..., None]).reshape(-1, 3)
        for q, oq in enumerate(obs):
            if q == m:
                continue
            out, ret = oq.field(3, 2, pts, bvs[q], v)
            assert (ret == 0).all()
            Ui[ext] += out[:, :4].reshape(len(ext), 4, 4)
            dUi[ext] += out[:, 4:].reshape(len(ext), 4, 4)
        nn = ob.NN
        X = np.zeros(8 * nn, complex)
        U, dU = bvs[m][0]["U"], bvs[m][0]["dU"]
        for s in range(1, len(ob.sids[0])):
            e = abs(ob.sids[0][s])
            for l in range(4 if ob.etype[e] else 3):
                c = ob.eni[e, l]
                X[nn * np.arange(4) + c] = U[s, l]
                X[nn * (np.arange(4) + 4) + c] = dU[s, l]
        GH, rows_of = {}, {}
        for d in range(ob.MN + 1):
            valid = port.domain_rows(ob, d)
            rows = valid[np.unique(np.linspace(0, len(valid) - 1, 40).astype(int))]
            G, H, _, _, _ = ob.rows(d, rows)
            GH[d] = (G, H)
            rows_of[d] = rows
        A = port.build_A_rows(ob, GH, rows_of)
        B = port.build_B(ob, GH, Ui, dUi, rows_of)
        res = np.linalg.norm(A @ X - B) / np.linalg.norm(B)
        print("object %d (%s, %d elements): oracle residual %.2e" % (m, objs[m]["kind"], ob.Ne, res))
        assert res <= 1e-9, (m, res)
