"""Known-answer case from the reference's own verification1 directory: two
absorbing cones (n = 0.06 + 4i in n = 1.33, mesh cone_m1_p5.msh shifted
+-0.2 along z), a plane wave at theta = 0.3.  Copies the shipped inputs next
to this script and extracts the values the reference printed (example1.log:
total field at r = (0.3, 0, 1.1) for quadrature types 0 and 1, radiation
force and torque about the origin and absorbed power of both objects;
d3b2_bv_solver.log: the convergence history) into expected.json.

Run where the reference is present:
    python3 tests/golden/make_verification1.py [reference_dir]
(default: the directory oracle/build_ref.sh --where reports).
"""
import json
import os
import re
import shutil

DST = os.path.join(os.path.dirname(os.path.abspath(__file__)), "verification1")
FILES = ["cone_m1_p5.msh", "medium_data.txt", "ipw.txt", "object_settings_v.txt"]


def cnum(re_s, im_s):
    return [float(re_s), float(im_s)]


def extract(src):
    """the values printed by the reference's verification1 run"""
    log = open(os.path.join(src, "example1.log")).read()
    exp = {"point": [0.3, 0.0, 1.1], "fields": {}, "force": {}, "absorb": {}}
    # total field blocks: one per type, Ex..Hz
    blocks = re.split(r"type=(\d) setting", log.split("Total electromagnetic field")[1].split("Radiation force")[0])
    for i in range(1, len(blocks), 2):
        t = int(blocks[i])
        vals = re.findall(r"([EH][xyz]) =\s*([-+0-9.e]+)\s*([-+0-9.e]+) I", blocks[i + 1])
        exp["fields"][str(t)] = [cnum(a, b) for _, a, b in vals]
    force_part = log.split("Radiation force and torque")[1].split("Absorbed energy")[0]
    parts = re.split(r"type=(\d) setting", force_part)
    for i in range(1, len(parts), 2):
        t = int(parts[i])
        objs = re.findall(r"obj[ec]+t id = (\d)\s*\nF = \(([^)]*)\)\s*\nN = \(([^)]*)\)", parts[i + 1])
        for oid, F, N in objs:
            exp["force"]["%s_%d" % (oid, t)] = [float(x) for x in F.split(",")] + [float(x) for x in N.split(",")]
    abs_part = log.split("Absorbed energy")[1]
    parts = re.split(r"type=(\d) setting", abs_part)
    for i in range(1, len(parts), 2):
        t = int(parts[i])
        for oid, P in re.findall(r"object id = (\d)\s*\nP = ([-+0-9.e]+)", parts[i + 1]):
            exp["absorb"]["%s_%d" % (oid, t)] = float(P)
    bv = open(os.path.join(src, "d3b2_bv_solver.log")).read()
    exp["cc"] = [float(x) for x in re.findall(r"cc = ([0-9.eE+-]+)", bv)]
    return exp


def main():
    import subprocess
    import sys
    if len(sys.argv) > 1:
        ref = sys.argv[1]
    else:
        here = os.path.dirname(os.path.abspath(__file__))
        ref = subprocess.run([os.path.join(here, "..", "..", "oracle", "build_ref.sh"), "--where"], capture_output=True,
                             text=True).stdout.strip()
    if not ref:
        sys.exit("the reference's sources were not found (give their directory as the argument)")
    src = os.path.join(ref, "verification1")
    os.makedirs(DST, exist_ok=True)
    for f in FILES:
        shutil.copyfile(os.path.join(src, f), os.path.join(DST, f))
    json.dump(extract(src), open(os.path.join(DST, "expected.json"), "w"), indent=1)


if __name__ == "__main__":
    main()
