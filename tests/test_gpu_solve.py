"""GPU parity of the multi-object iteration, boundary values, fields, forces.

The repository's d3b2_create_matrix and d3b2_bv_solver run on the GPU on the
golden scenes; the boundary values in the .dat file, the convergence history
and the fields / radiation force and torque / absorbed power printed by
bem3_analysis are compared with the reference's own outputs (golden
fixtures).  Tolerances: 1e-10 relative Frobenius on boundary values (plain
FP64 form), 1e-9 relative (vector norm) on fields, force and torque."""
import os
import re

import numpy as np
import pytest

from bem3_emf_b2_gb300 import formats, meshgen
from tests._scenes import load_case, parse_analysis, run, write_inputs

BV_TOL = 1e-10
OUT_TOL = 1e-9


def _solve(meta, gb_build, wd):
    write_inputs(meta, wd)
    run([os.path.join(gb_build, "d3b2_create_matrix"), "medium.txt", "mesh.msh", "obj.obj"], wd)
    meshgen.write_object_settings(os.path.join(wd, "objs.txt"), [(o[0], o[1]) for o in meta["objects"]])
    out = run([os.path.join(gb_build, "d3b2_bv_solver"), "objs.txt", "res.dat"], wd)
    ana = run([os.path.join(gb_build, "bem3_analysis"), "res.dat"], wd)
    return out, ana


def _check(meta, gold, wd, out, ana):
    dat = formats.read_dat(os.path.join(wd, "res.dat"))
    errs = {}
    for m, o in enumerate(dat):
        for d, sb in enumerate(o["sb"]):
            for k in ("U", "dU", "E", "dE", "H", "dH"):
                errs["o%d_d%d_%s" % (m, d, k)] = formats.rel_fro(sb[k], gold["o%d_d%d_%s" % (m, d, k)])
    bad = {k: v for k, v in errs.items() if not v <= BV_TOL}
    assert not bad, "boundary values above %g: %s" % (BV_TOL, bad)
    mine = parse_analysis([l for l in ana.splitlines() if l.startswith(("EH_", "force", "absorb"))])
    ref = parse_analysis(meta["analysis"])
    assert set(mine) == set(ref)
    for k, v in ref.items():
        if isinstance(v, int):
            assert mine[k] == v, k
            continue
        den = max(np.linalg.norm(v), 1e-300)
        err = np.linalg.norm(mine[k] - v) / den
        assert err <= OUT_TOL, "%s: relative error %g" % (k, err)
    cc = [float(x) for x in re.findall(r"cc = ([0-9.eE+-]+)", out)]
    assert len(cc) == len(meta["cc"]), "iteration count %d vs reference %d" % (len(cc), len(meta["cc"]))
    for a, b in zip(cc, meta["cc"]):
        if b > 1e-12:
            assert abs(a - b) <= 1e-5 * b, "cc history %s vs %s" % (cc, meta["cc"])


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["cube1", "sphere2", "cone_mix", "cone_tri", "pair"])
def test_bv_solver_parity(case, gb_build, tmp_path):
    meta, gold = load_case(case)
    wd = str(tmp_path)
    out, ana = _solve(meta, gb_build, wd)
    _check(meta, gold, wd, out, ana)


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["cube1", "sphere2", "cone_mix", "cone_tri", "pair"])
def test_tools_with_block_factor_files(case, gb_build, tmp_path):
    """d3b2_create_matrix with GB_CMAT_FORMAT=block writes the versioned
    <prefix>_blk.cmat (header + the five FP64 node-sized factors) in place of
    the dense <prefix>_invA.cmat, records it in the .obj, and d3b2_bv_solver
    solves from it: the same boundary values, convergence history, fields,
    forces and absorbed powers as the reference's golden outputs."""
    import struct
    meta, gold = load_case(case)
    wd = str(tmp_path)
    write_inputs(meta, wd)
    env = {"GB_CMAT_FORMAT": "block"}
    run([os.path.join(gb_build, "d3b2_create_matrix"), "medium.txt", "mesh.msh", "obj.obj"], wd, env)
    obj = formats.read_obj(os.path.join(wd, "obj.obj"))
    assert obj["invA"] == "obj_blk.cmat", obj["invA"]
    assert not os.path.exists(os.path.join(wd, "obj_invA.cmat"))
    with open(os.path.join(wd, "obj_blk.cmat"), "rb") as f:
        hdr = f.read(64)
    assert hdr[:8] == b"GBBLKF64"
    ver, nn, nmat, esz = struct.unpack("<4i", hdr[8:24])
    assert (ver, nn, nmat, esz) == (1, meta["NN"], 5, 16)
    assert os.path.getsize(os.path.join(wd, "obj_blk.cmat")) == 64 + 5 * nn * nn * 16
    meshgen.write_object_settings(os.path.join(wd, "objs.txt"), [(o[0], o[1]) for o in meta["objects"]])
    out = run([os.path.join(gb_build, "d3b2_bv_solver"), "objs.txt", "res.dat"], wd)
    ana = run([os.path.join(gb_build, "bem3_analysis"), "res.dat"], wd)
    _check(meta, gold, wd, out, ana)
