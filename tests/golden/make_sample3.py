"""Known-answer case with a focused beam, from the reference's own
analysis_sample3 directory: a hemisphere (hemisphere_m1.msh, n = 1.515) and
an absorbing cone (cone_m2.msh, n = 0.06 + 4i, rotated by pi about x and
shifted +0.13 along z) in air, lit by a focused plane wave (fpw.txt:
lambda0 = 0.6328, NA = 0.35, 64 Gauss-Legendre nodes).  Copies the shipped
inputs next to this script and extracts what the reference printed:
example1_ex3.log (both objects) and example1_ex30.log (the hemisphere alone):
total field at r = (0.3, 0, 1.1), radiation force and torque, absorbed power;
d3b2_bv_solver.log: the two-object convergence history.

Run where the reference is present:
    python3 tests/golden/make_sample3.py [reference_dir]
"""
import importlib.util
import json
import os
import re
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
DST = os.path.join(HERE, "sample3")
FILES = ["hemisphere_m1.msh", "cone_m2.msh", "medium_data1.txt", "medium_data2.txt", "fpw.txt", "object_settings.txt",
         "object_settings0.txt"]


def _extract_log(path):
    """fields / force / absorb blocks of one example1 log (the verification1
    extractor, applied to a log file of another name)"""
    spec = importlib.util.spec_from_file_location("mv1", os.path.join(HERE, "make_verification1.py"))
    mv1 = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mv1)
    tmp = os.path.join(DST, "_tmp")
    os.makedirs(tmp, exist_ok=True)
    shutil.copyfile(path, os.path.join(tmp, "example1.log"))
    open(os.path.join(tmp, "d3b2_bv_solver.log"), "w").close()
    out = mv1.extract(tmp)
    shutil.rmtree(tmp)
    out.pop("cc")
    return out


def main():
    if len(sys.argv) > 1:
        ref = sys.argv[1]
    else:
        ref = subprocess.run(["bash", os.path.join(HERE, "..", "..", "oracle", "build_ref.sh"), "--where"],
                             capture_output=True, text=True).stdout.strip()
    if not ref:
        sys.exit("the reference's sources were not found (give their directory as the argument)")
    src = os.path.join(ref, "analysis_sample3")
    os.makedirs(DST, exist_ok=True)
    for f in FILES:
        shutil.copyfile(os.path.join(src, f), os.path.join(DST, f))
    bv = open(os.path.join(src, "d3b2_bv_solver.log")).read()
    first = bv.split("d3b2_bv_solver object_settings0.txt")[0]
    exp = {"ex3": _extract_log(os.path.join(src, "example1_ex3.log")),
           "ex30": _extract_log(os.path.join(src, "example1_ex30.log")),
           "cc_ex3": [float(x) for x in re.findall(r"cc = ([0-9.eE+-]+)", first)],
           "create": {"hemisphere_m1_md1.obj": ["medium_data1.txt", "hemisphere_m1.msh"],
                      "cone_m2_md2_xpi.obj": ["medium_data2.txt", "cone_m2.msh", "1", "0", "0", "3.1415926535", "0",
                                              "0", "0"]}}
    json.dump(exp, open(os.path.join(DST, "expected.json"), "w"), indent=1)
    print("wrote", DST)


if __name__ == "__main__":
    main()
