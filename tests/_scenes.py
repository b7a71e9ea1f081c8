"""Shared helpers of the tests: write a golden case's inputs into a directory
and run tools there."""
import json
import os
import subprocess

import numpy as np

from bem3_emf_b2_gb300 import meshgen

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_case(name):
    with open(os.path.join(GOLDEN, name + ".json")) as f:
        meta = json.load(f)
    arrays = np.load(os.path.join(GOLDEN, name + ".npz"))
    return meta, arrays


def write_inputs(meta, wd):
    spec = meta["mesh"]
    if spec[0] == "sphere":
        nodes, elems = meshgen.cubed_sphere(spec[1], spec[2])
    elif spec[0] == "cone_mixed":
        nodes, elems = meshgen.cone_mixed(spec[1], spec[2], spec[3], spec[4])
    else:
        nodes, elems = meshgen.cone_tri(spec[1], spec[2], spec[3], jitter=0.0)
    meshgen.write_mesh(os.path.join(wd, "mesh.msh"), nodes, elems)
    meshgen.write_medium(os.path.join(wd, "medium.txt"), [complex(a, b) for a, b in meta["n"]])
    meshgen.write_ipw(os.path.join(wd, "ipw.txt"), [meta["wave"]])


def run(cmd, cwd, env=None):
    e = dict(os.environ)
    if env:
        e.update(env)
    r = subprocess.run(cmd, cwd=cwd, capture_output=True, text=True, env=e)
    if r.returncode != 0:
        raise AssertionError("%s failed (%d):\n%s%s" % (cmd, r.returncode, r.stdout[-4000:], r.stderr[-4000:]))
    return r.stdout


def parse_analysis(lines):
    """bem3_analysis output -> {key: np.array of numbers}"""
    out = {}
    for l in lines:
        t = l.split()
        if t[0].startswith("EH"):
            out["%s_%s" % (t[0], t[2])] = np.array([float(x) for x in t[5:]])
            out["%s_%s_oid" % (t[0], t[2])] = int(t[4])
        elif t[0] == "force":
            out["force_%s_%s" % (t[2], t[4])] = np.array([float(x) for x in t[7:]])
        elif t[0] == "absorb":
            out["absorb_%s_%s" % (t[2], t[4])] = np.array([float(t[7])])
            out["absorb_%s_%s_ret" % (t[2], t[4])] = int(t[6])
    return out
