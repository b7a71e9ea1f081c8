"""GPU: the learned near-singular quadrature -- training on the GPU and its
gain, with and without the network, inside the chosen form's assembly.

Training: 4M fallback quadrangle pairs collected from seeded cubes and
cuboids (bem3_emf_b2_gb300.lq.train), labelled by both rules in FP64 and
fitted by the project's MLP kernels.  Then on a cube of side 3 with 12 x 12
quadrangles per face (n = 1.6 in 1.33; the 38,400-element cube's generator)
and a cuboid (the same cube stretched by 1.25 and 0.8 along y and z,
n = 1.5), neither of them in the training set:

  * matrices of the chosen form's assembly (precision 3) without the
    network and with it (correction kept: judge tolerance 1e-3), each
    against the FP64 assembly (64 x 64 fallback rule): relative Frobenius
    error and assembly time; the judge's figures (RMS error of the
    corrected sample against the 64 x 64 rule, and of the 12 x 12 rule alone
    on the same pairs);
  * force and torque of the chosen form with the kept correction against
    the FP64 form;
  * at the chosen form's judge tolerance (1e-7) a correction that misses it
    is reverted to the 64 x 64 rule: the matrices are then bit for bit those
    of the assembly without the network, and the force and torque stay
    within 1e-6 of the FP64 form.
The test reports the gain (or loss); it does not require one.
"""
import ctypes
import os
import time

import numpy as np
import pytest

from bem3_emf_b2_gb300 import meshgen


def _setup(wd, kind):
    if kind == "cube":
        nodes, elems = meshgen.cube(12, 3.0)
        n_in = 1.6
    else:
        nodes, elems = meshgen.cube(10, 2.5)
        nodes = nodes * np.array([1.0, 1.25, 0.8])
        n_in = 1.5
    meshgen.write_mesh(os.path.join(wd, "mesh.msh"), nodes, elems)
    meshgen.write_medium(os.path.join(wd, "medium.txt"), [n_in])
    meshgen.write_ipw(os.path.join(wd, "ipw.txt"), [dict(lambda0=1.0, ni=1.33, power=1.0, e0x=1.0, e0y=0.0)])
    return len(elems)


def _download(L, o, d, ne):
    N = 4 * ne
    m = [np.zeros((N, N), complex), np.zeros((N, N), complex), np.zeros((2 * N, N), complex),
         np.zeros((2 * N, N), complex), np.zeros((N, 3))]
    assert L.gb_cmatrix_download(o, d, *[x.ctypes.data for x in m]) == 0
    return m


def _rel(a, b):
    return max(np.linalg.norm(x - y) / np.linalg.norm(y) for x, y in zip(a, b))


@pytest.mark.gpu
def test_learned_quadrature_gain(gb_build, tmp_path):
    from bem3_emf_b2_gb300 import Scene, lib, lq
    import torch
    L = lib()
    vp, ci = ctypes.c_void_p, ctypes.c_int
    L.gb_cmatrix_download.argtypes = [vp, ci, vp, vp, vp, vp, vp]
    t0 = time.perf_counter()
    info = lq.train(samples=4_000_000, epochs=4, batch=1024, lr=1e-3, seed=1)
    print("training: %s (%.0f s)" % (info, time.perf_counter() - t0))
    assert info["held_out_loss"] < info["held_out_loss_zero"]
    for kind in ("cube", "cuboid"):
        wd = os.path.join(str(tmp_path), kind)
        os.makedirs(wd)
        ne = _setup(wd, kind)
        sc = Scene(os.path.join(wd, "medium.txt"), os.path.join(wd, "mesh.msh"), os.path.join(wd, "ipw.txt"))
        o = sc.obj()
        for d in range(2):
            assert L.gb_assemble2(o, d, 2, 0) == 0
            ref = _download(L, o, d, ne)
            res = {}
            for mode in ("plain", "net", "strict"):
                if mode == "plain":
                    lq.enable(False)
                else:
                    lq.enable(True, 1e-7 if mode == "strict" else 1e-3)
                for _ in range(2):  # the second call is timed
                    torch.cuda.synchronize()
                    t = time.perf_counter()
                    assert L.gb_assemble2(o, d, 2, 3) == 0
                    torch.cuda.synchronize()
                    dt = time.perf_counter() - t
                st = lq.stats() if mode != "plain" else None
                res[mode] = (_download(L, o, d, ne), dt, st)
            lq.enable(False)
            e_plain, e_net = _rel(res["plain"][0], ref), _rel(res["net"][0], ref)
            st = res["net"][2]
            print("%s domain %d: %d fallback pairs; error vs FP64 without the network %.2e (%.3f s), with it %.2e "
                  "(%.3f s); judged %d: RMS corrected %.2e, RMS 12x12 %.2e, reverted %d" % (
                      kind, d, st["pairs"], e_plain, res["plain"][1], e_net, res["net"][1], st["judged"],
                      st["rms_corrected"], st["rms_12x12"], st["reverted"]))
            assert st["pairs"] > 0 and st["reverted"] == 0.0
            assert st["rms_corrected"] < st["rms_12x12"]  # the network moves the 12 x 12 values toward the 64 x 64 rule
            strict = res["strict"][2]
            if strict["rms_corrected"] > 1e-7:
                assert strict["reverted"] == 1.0
                for a, b in zip(res["strict"][0], res["plain"][0]):
                    assert np.array_equal(a, b)
        # the chosen form's force with the network against the FP64 form
        F0, N0 = sc.step(form=0)
        v0 = np.concatenate([F0, N0])
        for tol in (1e-3, 1e-7):
            lq.enable(True, tol)
            try:
                F1, N1 = sc.step(form=1)
            finally:
                lq.enable(False)
            df = np.linalg.norm(np.concatenate([F1, N1]) - v0) / np.linalg.norm(v0)
            print("%s: force/torque with the network (judge tolerance %g) vs FP64 form %.2e" % (kind, tol, df))
            if tol == 1e-7:
                assert df <= 1e-6
        sc.close()
