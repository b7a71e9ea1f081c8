"""GPU parity of the coefficient-matrix assembly and of the inverse of A.

The repository's d3b2_create_matrix runs on the GPU on the small scenes of
tests/golden; the .cmat files it writes are compared with those written by
the reference's own d3b2_create_matrix (golden fixtures).  Tolerance: relative
Frobenius error <= 1e-10 per matrix (plain FP64 form)."""
import os

import numpy as np
import pytest

from bem3_emf_b2_gb300 import formats
from tests._scenes import load_case, run, write_inputs

TOL = 1e-10
CASES = ["cube1", "sphere2", "cone_mix", "cone_tri"]


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES)
def test_create_matrix_parity(case, gb_build, tmp_path):
    meta, gold = load_case(case)
    wd = str(tmp_path)
    write_inputs(meta, wd)
    run([os.path.join(gb_build, "d3b2_create_matrix"), "medium.txt", "mesh.msh", "obj.obj"], wd)
    obj = formats.read_obj(os.path.join(wd, "obj.obj"))
    assert obj["NN"] == meta["NN"] and obj["Ne"] == meta["Ne"]
    worst = {}
    for d in range(obj["MN"] + 1):
        mats = formats.read_domain_cmats(obj, d, wd)
        for k, v in mats.items():
            err = formats.rel_fro(v, gold["%s_%d" % (k, d)])
            worst["%s_%d" % (k, d)] = err
    bad = {k: v for k, v in worst.items() if not v <= TOL}
    assert not bad, "relative Frobenius errors above %g: %s (all: %s)" % (TOL, bad, worst)
    if "invA" in gold.files:
        na = 8 * obj["NN"]
        inv = formats.read_cmat(os.path.join(wd, obj["invA"]), (na, na))
        err = formats.rel_fro(inv, gold["invA"])
        assert err <= TOL, "invA relative Frobenius error %g" % err
