"""GPU: the reference's focused-beam known-answer case (analysis_sample3: a
hemisphere n = 1.515 and an absorbing cone n = 0.06 + 4i lit by a focused
plane wave, NA = 0.35; inputs and printed values committed under
tests/golden/sample3 by make_sample3.py), run through the reference-facing
tools: d3b2_create_matrix (FP64; the block-elimination .cmat variant, since
the dense inverse of na = 32,256 would take minutes), d3b2_bv_solver,
bem3_analysis.

  * two objects (ex3): the convergence history to the log's 6 digits and its
    length; total field at (0.3, 0, 1.1), forces and torques, the cone's
    absorbed power to 1e-9 relative (the hemisphere's absorbed power is a
    cancellation the reference itself flags: 1e-7);
  * the hemisphere alone (ex30): the same quantities.
"""
import json
import os
import re
import shutil

import numpy as np
import pytest

from tests._scenes import parse_analysis, run

CASE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "sample3")


def _rel(a, b):
    a, b = np.asarray(a, float).ravel(), np.asarray(b, float).ravel()
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _check(mine, exp, tag):
    worst = 0.0
    for t in ("0", "1"):
        ref = np.array(exp["fields"][t]).ravel()
        e = _rel(mine["EH_t_" + t], ref)
        worst = max(worst, e)
        assert e <= 1e-9, (tag, "field type", t, e)
    for key, ref in exp["force"].items():
        oid, t = key.split("_")
        got = mine["force_%s_%s" % (oid, t)]
        ef, en = _rel(got[:3], ref[:3]), _rel(got[3:], ref[3:])
        worst = max(worst, ef, en)
        assert ef <= 1e-9 and en <= 1e-9, (tag, key, ef, en)
    for key, ref in exp["absorb"].items():
        oid, t = key.split("_")
        got = mine["absorb_%s_%s" % (oid, t)][0]
        tol = 1e-7 if oid == "0" else 1e-9
        assert abs(got - ref) <= tol * abs(ref), (tag, "absorbed power", key, got, ref)
    return worst


@pytest.mark.gpu
def test_sample3_focused_beam_tools(gb_build, tmp_path):
    exp = json.load(open(os.path.join(CASE, "expected.json")))
    wd = str(tmp_path)
    for f in os.listdir(CASE):
        if f != "expected.json":
            shutil.copyfile(os.path.join(CASE, f), os.path.join(wd, f))
    env = {"GB_CMAT_FORMAT": "block"}
    for obj, args in exp["create"].items():
        run([os.path.join(gb_build, "d3b2_create_matrix")] + args[:2] + [obj] + args[2:], wd, env)
    out = run([os.path.join(gb_build, "d3b2_bv_solver"), "object_settings.txt", "ex3.dat"], wd, env)
    assert "focused plane wave" in out
    cc = [float(v) for v in re.findall(r"cc = ([0-9.eE+-]+)", out)]
    assert len(cc) == len(exp["cc_ex3"]), (cc, exp["cc_ex3"])
    for a, b in zip(cc, exp["cc_ex3"]):
        assert abs(a - b) <= 1e-5 * b, (cc, exp["cc_ex3"])
    run([os.path.join(gb_build, "d3b2_bv_solver"), "object_settings0.txt", "ex30.dat"], wd, env)
    worst = 0.0
    for dat, key in (("ex3.dat", "ex3"), ("ex30.dat", "ex30")):
        ana = run([os.path.join(gb_build, "bem3_analysis"), dat, "0.3", "0", "1.1"], wd)
        mine = parse_analysis([l for l in ana.splitlines() if l.startswith(("EH_", "force", "absorb"))])
        worst = max(worst, _check(mine, exp[key], key))
    print("analysis_sample3 (focused beam): largest relative difference %.2e" % worst)
