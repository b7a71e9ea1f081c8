"""GPU: the reference's own end-to-end known-answer case (verification1: two
absorbing cones n = 0.06 + 4i, mesh cone_m1_p5.msh shifted +-0.2 along z,
plane wave at theta = 0.3; inputs and the values its example1 printed are
committed under tests/golden/verification1 by make_verification1.py).

- Plain FP64 form through the reference-facing tools (d3b2_create_matrix,
  d3b2_bv_solver, then the fields, forces and absorbed power of
  bem3_analysis): the printed values (15 significant digits) to 1e-10
  relative, the convergence history to the log's 6 digits and its length.
- Chosen form through the multi-object scene API (double-float quadrature,
  butterfly-randomised FP32 LU, FP64 refinement): force and torque about the
  origin, quadrature type 0, to 1e-6 relative (the chosen form's tolerance).
"""
import json
import os
import re
import shutil

import numpy as np
import pytest

from tests._scenes import parse_analysis, run

CASE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "verification1")


def _expected():
    return json.load(open(os.path.join(CASE, "expected.json")))


def _copy_inputs(wd):
    for f in ("cone_m1_p5.msh", "medium_data.txt", "ipw.txt", "object_settings_v.txt"):
        shutil.copyfile(os.path.join(CASE, f), os.path.join(wd, f))


def _rel(a, b):
    a, b = np.asarray(a, float).ravel(), np.asarray(b, float).ravel()
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.gpu
def test_verification1_fp64_tools(gb_build, tmp_path):
    exp = _expected()
    wd = str(tmp_path)
    _copy_inputs(wd)
    run([os.path.join(gb_build, "d3b2_create_matrix"), "medium_data.txt", "cone_m1_p5.msh", "cone_m1_p5_md_x00.obj"], wd)
    out = run([os.path.join(gb_build, "d3b2_bv_solver"), "object_settings_v.txt", "v1.dat"], wd)
    x, y, z = exp["point"]
    ana = run([os.path.join(gb_build, "bem3_analysis"), "v1.dat", repr(x), repr(y), repr(z)], wd)
    mine = parse_analysis([l for l in ana.splitlines() if l.startswith(("EH_", "force", "absorb"))])
    worst = 0.0
    for t in ("0", "1"):
        ref = np.array(exp["fields"][t]).ravel()  # Ex..Hz as (re, im)
        worst = max(worst, _rel(mine["EH_t_" + t], ref))
        assert _rel(mine["EH_t_" + t], ref) <= 1e-10, ("field type", t, _rel(mine["EH_t_" + t], ref))
    for key, ref in exp["force"].items():
        oid, t = key.split("_")
        got = mine["force_%s_%s" % (oid, t)]
        worst = max(worst, _rel(got[:3], ref[:3]), _rel(got[3:], ref[3:]))
        assert _rel(got[:3], ref[:3]) <= 1e-10, ("force", key, _rel(got[:3], ref[:3]))
        assert _rel(got[3:], ref[3:]) <= 1e-10, ("torque", key, _rel(got[3:], ref[3:]))
    for key, ref in exp["absorb"].items():
        oid, t = key.split("_")
        got = mine["absorb_%s_%s" % (oid, t)][0]
        worst = max(worst, abs(got - ref) / abs(ref))
        assert abs(got - ref) <= 1e-10 * abs(ref), ("absorbed power", key, got, ref)
    print("verification1 FP64 tools: largest relative difference %.2e" % worst)
    cc = [float(v) for v in re.findall(r"cc = ([0-9.eE+-]+)", out)]
    assert len(cc) == len(exp["cc"]), (cc, exp["cc"])
    for a, b in zip(cc, exp["cc"]):
        assert abs(a - b) <= 1e-5 * b, (cc, exp["cc"])


@pytest.mark.gpu
def test_verification1_chosen_form(gb_build, tmp_path):
    from bem3_emf_b2_gb300 import MultiScene
    exp = _expected()
    wd = str(tmp_path)
    _copy_inputs(wd)
    med = os.path.join(wd, "medium_data.txt")
    msh = os.path.join(wd, "cone_m1_p5.msh")
    tv = np.array([0.0, 0.0, 0.2, 0.0, 0.0, -0.2])
    sc = MultiScene([med, med], [msh, msh], os.path.join(wd, "ipw.txt"), tv=tv, quiet=True)
    F, N = sc.step(form=1, rc=np.zeros((2, 3)))
    sc.close()
    print("verification1 chosen form: force %s torque %s" % (
        [_rel(F[o], exp["force"]["%d_0" % o][:3]) for o in range(2)],
        [_rel(N[o], exp["force"]["%d_0" % o][3:]) for o in range(2)]))
    for oid in range(2):
        ref = exp["force"]["%d_0" % oid]
        assert _rel(F[oid], ref[:3]) <= 1e-6, ("force", oid, _rel(F[oid], ref[:3]))
        assert _rel(N[oid], ref[3:]) <= 1e-6, ("torque", oid, _rel(N[oid], ref[3:]))
