"""CPU: the drop-in tools fail on bad input the way the reference's do.

The reference's error convention is a message on stdout and exit(1)
(`printf` + `exit(1)`), or its usage text and exit(0) without arguments.  For
input errors that stop a tool before any device work, d3b2_create_matrix and
d3b2_bv_solver built from this repository print the same message with the
same exit code as the reference's own tools built from its sources
(oracle/_ref, present where the reference is).  The message's leading
"<source file>, " names the file that raised it, and is compared without it."""
import os
import re
import subprocess

import pytest

from bem3_emf_b2_gb300 import meshgen

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.path.join(ROOT, "oracle", "_ref")


def _norm(out, tool_path):
    out = out.replace(tool_path, "TOOL")
    return [re.sub(r"^\w+\.c, ", "", l) for l in out.splitlines()]


def _run(path, args, cwd):
    r = subprocess.run([path] + args, cwd=cwd, capture_output=True, text=True, timeout=60)
    return r.returncode, _norm(r.stdout + r.stderr, path)


def _files(wd, names):
    if "ipw" in names:
        meshgen.write_ipw(os.path.join(wd, "ipw.txt"), [dict(lambda0=1.0, ni=1.33, power=1.0)])
    if "bad_medium" in names:
        with open(os.path.join(wd, "med.txt"), "w") as f:
            f.write("1\n")
    if "bad_settings" in names:
        with open(os.path.join(wd, "os.txt"), "w") as f:
            f.write("# settings\n1\nnone.obj\n")


CASES = [
    ("d3b2_create_matrix", [], []),
    ("d3b2_create_matrix", ["nomed.txt", "nomesh.msh", "out.obj"], []),
    ("d3b2_create_matrix", ["nomed.txt", "nomesh.msh", "out.obj"], ["ipw"]),
    ("d3b2_create_matrix", ["med.txt", "nomesh.msh", "out.obj"], ["ipw", "bad_medium"]),
    ("d3b2_bv_solver", [], []),
    ("d3b2_bv_solver", ["nofile.txt", "out.dat"], []),
    ("d3b2_bv_solver", ["os.txt", "out.dat"], ["bad_settings"]),
]


@pytest.mark.parametrize("tool,args,files", CASES)
def test_tool_error_matches_reference(tool, args, files, gb_build, tmp_path):
    ref = os.path.join(REF, tool)
    if not os.path.exists(ref):
        pytest.skip("the reference's tools are not built here (oracle/build_ref.sh needs the reference sources)")
    mine = os.path.join(gb_build, tool)
    out = []
    for path in (ref, mine):
        wd = tmp_path / os.path.basename(os.path.dirname(path))
        wd.mkdir()
        _files(str(wd), files)
        out.append(_run(path, args, str(wd)))
    assert out[1] == out[0], (out[0], out[1])
