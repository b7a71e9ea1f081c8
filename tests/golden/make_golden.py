"""Generates the golden fixtures of tests/golden from the reference itself.

The reference (akohta/bem3_emf_b2) is built unmodified by oracle/build_ref.sh
into oracle/_ref (MKL replaced by numpy's ILP64 OpenBLAS).  This script runs
its d3b2_create_matrix, d3b2_bv_solver and the repository's bem3_analysis
driver (compiled against the reference API) on small synthetic scenes and
stores the outputs:
  <case>.npz   G,H,dG,dH,dF of every domain (.cmat contents), invA (cube only),
               boundary values U,dU,E,dE,H,dH of every object and domain
  <case>.json  inputs, field/force/absorption lines of bem3_analysis, the
               convergence history printed by d3b2_bv_solver
Run from anywhere: python tests/golden/make_golden.py
"""
import json
import os
import re
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from bem3_emf_b2_gb300 import formats, meshgen  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref")

WAVE = dict(lambda0=1.0, ni=1.33, power=1.0, e0x=1.0, e0y=0.0, theta=0.0, phi=0.0)

CASES = {
    # planar quadrangles (inscribed cube): singular H, F vanish
    "cube1": dict(mesh=("sphere", 1, 0.3), n=[1.5], save_inv=True),
    # curved bilinear quadrangles
    "sphere2": dict(mesh=("sphere", 2, 0.35), n=[1.5], save_inv=False),
    # mixed triangles and quadrangles, absorbing medium (complex wave number)
    "cone_mix": dict(mesh=("cone_mixed", 6, 2, 0.3, 0.5), n=[1.5 + 0.05j], save_inv=False),
    # linear triangles only
    "cone_tri": dict(mesh=("cone_tri", 1, 0.3, 0.5), n=[1.59 + 0.0j], save_inv=False),
}
PAIR = dict(mesh=("sphere", 2, 0.25), n=[1.5], shifts=[(0.0, 0.0, 0.45), (0.0, 0.0, -0.45)])


def make_mesh(spec, path):
    if spec[0] == "sphere":
        nodes, elems = meshgen.cubed_sphere(spec[1], spec[2])
    elif spec[0] == "cone_mixed":
        nodes, elems = meshgen.cone_mixed(spec[1], spec[2], spec[3], spec[4])
    else:
        nodes, elems = meshgen.cone_tri(spec[1], spec[2], spec[3], jitter=0.0)
    meshgen.write_mesh(path, nodes, elems)


def run(cmd, cwd):
    r = subprocess.run(cmd, cwd=cwd, capture_output=True, text=True, env=dict(os.environ, OMP_NUM_THREADS="4"))
    if r.returncode != 0:
        raise RuntimeError("%s failed:\n%s%s" % (cmd, r.stdout, r.stderr))
    return r.stdout


def analysis_lines(out):
    return [l for l in out.splitlines() if l.startswith(("EH_", "force", "absorb"))]


def cc_history(out):
    return [float(x) for x in re.findall(r"cc = ([0-9.eE+-]+)", out)]


def solve_case(name, spec, wd, objs):
    meshgen.write_object_settings(os.path.join(wd, "objs.txt"), objs)
    out = run([os.path.join(REF, "d3b2_bv_solver"), "objs.txt", "res.dat"], wd)
    dat = formats.read_dat(os.path.join(wd, "res.dat"))
    ana = run([os.path.join(REF, "bem3_analysis"), "res.dat"], wd)
    arrays = {}
    for m, o in enumerate(dat):
        for d, sb in enumerate(o["sb"]):
            for k in ("U", "dU", "E", "dE", "H", "dH"):
                arrays["o%d_d%d_%s" % (m, d, k)] = sb[k]
    return arrays, analysis_lines(ana), cc_history(out)


def main():
    if not os.path.exists(os.path.join(REF, "d3b2_create_matrix")):
        sys.exit("oracle/_ref is not built (run oracle/build_ref.sh)")
    for name, spec in list(CASES.items()) + [("pair", PAIR)]:
        wd = tempfile.mkdtemp(prefix="golden_")
        try:
            make_mesh(spec["mesh"], os.path.join(wd, "mesh.msh"))
            meshgen.write_medium(os.path.join(wd, "medium.txt"), spec["n"])
            meshgen.write_ipw(os.path.join(wd, "ipw.txt"), [WAVE])
            run([os.path.join(REF, "d3b2_create_matrix"), "medium.txt", "mesh.msh", "obj.obj"], wd)
            obj = formats.read_obj(os.path.join(wd, "obj.obj"))
            arrays = {}
            if name != "pair":
                for d in range(obj["MN"] + 1):
                    for k, v in formats.read_domain_cmats(obj, d, wd).items():
                        arrays["%s_%d" % (k, d)] = v
                if spec.get("save_inv"):
                    na = 8 * obj["NN"]
                    arrays["invA"] = formats.read_cmat(os.path.join(wd, obj["invA"]), (na, na))
                objs = [("obj.obj", (0.0, 0.0, 0.0))]
            else:
                objs = [("obj.obj", s) for s in spec["shifts"]]
            vals, lines, cc = solve_case(name, spec, wd, objs)
            arrays.update(vals)
            np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrays)
            meta = dict(case=name, mesh=list(spec["mesh"]), n=[[complex(x).real, complex(x).imag] for x in spec["n"]],
                        wave=WAVE, objects=[[o[0], list(o[1])] for o in objs], analysis=lines, cc=cc,
                        NN=obj["NN"], Ne=obj["Ne"], sb_Ne=[sb["Ne"] for sb in obj["sb"]])
            with open(os.path.join(HERE, name + ".json"), "w") as f:
                json.dump(meta, f, indent=1)
            print(name, "ok", obj["Ne"], "elements")
        finally:
            shutil.rmtree(wd, ignore_errors=True)


if __name__ == "__main__":
    main()
