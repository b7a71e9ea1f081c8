"""Learned near-singular quadrature: training driver (the kernels and the
network are in libbem3gb.so: gb_lq_* in include/gb_bem.h).

The reference integrates a (collocation node, quadrangle) pair whose
|Re dF| exceeds 0.5 by a 64 x 64 Gauss-Legendre rule (d3b1_elem.c:503-504,
bil_dcoef_v2.c:235-326).  The network predicts the difference between that
rule and the 12 x 12 rule from the pair's geometry; the assembly adds it to
the 12 x 12 values and checks a sample of every assembly's corrected pairs
against the 64 x 64 rule, keeping the correction only if the sample's RMS
error is within the tolerance.

train() collects such pairs from a seeded family of quadrangle meshes --
cubes and cuboids of random size, resolution and index, both domains of
each -- labels them on the GPU (both rules in FP64) and trains the network
there.
"""
import ctypes
import os
import tempfile

import numpy as np

from . import Scene, last_error, lib, meshgen


def _api():
    L = lib()
    vp, ci = ctypes.c_void_p, ctypes.c_int
    L.gb_lq_collect.argtypes = [ci]
    L.gb_lq_train.argtypes = [ci, ci, ctypes.c_float, ctypes.c_uint, vp]
    L.gb_lq_enable.argtypes = [ci, ctypes.c_double]
    L.gb_lq_stats.argtypes = [vp]
    L.gb_assemble2.argtypes = [vp, ci, ci, ci]
    L.gb_assemble2.restype = ci
    return L


def stats():
    """Figures of the last assembly that listed pairs: dict of pairs
    corrected, beyond capacity, judged, rms_corrected, rms_12x12,
    max_corrected, reverted, ms."""
    s = np.zeros(8)
    _api().gb_lq_stats(s.ctypes.data)
    keys = ("pairs", "beyond_capacity", "judged", "rms_corrected", "rms_12x12", "max_corrected", "reverted", "ms")
    return dict(zip(keys, s.tolist()))


def enable(on=True, tol=1e-7):
    if _api().gb_lq_enable(1 if on else 0, tol) != 0:
        raise RuntimeError(last_error())


def training_meshes(seed):
    """An endless seeded sequence of (nodes, elems, n_inside, lambda0): cubes
    and mildly stretched cuboids of random size, resolution and refractive
    index -- the pairs that need the fallback rule sit at their edges (the
    smooth cubed spheres of this size range have none)."""
    rng = np.random.default_rng(seed)
    while True:
        size = float(np.exp(rng.uniform(np.log(0.5), np.log(6.0))))
        nodes, elems = meshgen.cube(int(rng.integers(4, 17)), size)
        if rng.random() < 0.5:
            nodes = nodes * rng.uniform(0.75, 1.3, 3)
        n_in = complex(rng.uniform(1.1, 2.6), rng.uniform(0.0, 0.05))
        yield nodes, elems, n_in, 1.0


def collect(target, seed=1, max_meshes=4000, log=None):
    """List fallback quadrangle pairs from training meshes until `target`
    pairs are held; returns the count."""
    L = _api()
    if L.gb_lq_collect(1) != 0:
        raise RuntimeError(last_error())
    total = 0
    try:
        with tempfile.TemporaryDirectory() as wd:
            for i, (nodes, elems, n_in, lam) in enumerate(training_meshes(seed)):
                if total >= target or i >= max_meshes:
                    break
                meshgen.write_mesh(os.path.join(wd, "m.msh"), nodes, elems)
                meshgen.write_medium(os.path.join(wd, "n.txt"), [n_in])
                meshgen.write_ipw(os.path.join(wd, "w.txt"),
                                  [dict(lambda0=lam, ni=1.33, power=1.0, e0x=1.0, e0y=0.0)])
                sc = Scene(os.path.join(wd, "n.txt"), os.path.join(wd, "m.msh"), os.path.join(wd, "w.txt"))
                try:
                    for d in range(2):
                        if L.gb_assemble2(sc.obj(), d, 2, 3) != 0:
                            raise RuntimeError(last_error())
                        total += int(stats()["pairs"])
                finally:
                    sc.close()
                if log:
                    log("mesh %d (%d elements): %d pairs" % (i, len(elems), total))
    finally:
        L.gb_lq_collect(0)
    return total


def train(samples=4_000_000, epochs=4, batch=1024, lr=1e-3, seed=1, log=None):
    """Collect `samples` pairs, train; returns the training figures."""
    n = collect(samples, seed, log=log)
    info = np.zeros(5)
    if _api().gb_lq_train(epochs, batch, lr, seed, info.ctypes.data) != 0:
        raise RuntimeError(last_error())
    return dict(collected=n, trained=int(info[0]), held_out=int(info[1]), train_loss=float(info[2]),
                held_out_loss=float(info[3]), held_out_loss_zero=float(info[4]))
