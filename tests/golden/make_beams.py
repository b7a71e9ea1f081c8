"""Golden incident fields of the reference's beam families.

For each beam file of the reference's beam_sample directory (ipw, fpw, lgb,
bsb, blg, rab: the reference's own sample parameters) alone, and for all six
together (summed in the reference's order), the unmodified reference
(oracle/_ref/ref_beam: init_mfb, read_data_mfb, setup_mfb, calc_mfb_EH_dv,
mfb_src/multi_fbeam.c) evaluates E, H, dE/dv, dH/dv at seeded points around
the foci (a 3 x 3 x 3 lambda box about the origin, plus a few points 5 to
20 lambda out) along seeded unit directions.  Writes beams/<name>.txt (the
sample files) and beams/expected.json next to this script.

Run where the reference is present (after oracle/build_ref.sh):
    python3 tests/golden/make_beams.py [reference_dir]
"""
import json
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
DST = os.path.join(HERE, "beams")
FAMILIES = ["ipw", "fpw", "lgb", "bsb", "blg", "rab"]


def points(seed=11):
    rng = np.random.default_rng(seed)
    box = rng.uniform(-1.5, 1.5, (40, 3))
    far_dir = rng.normal(size=(8, 3))
    far = far_dir / np.linalg.norm(far_dir, axis=1)[:, None] * rng.uniform(5.0, 20.0, (8, 1))
    x = np.concatenate([[[0.0, 0.0, 0.0]], box, far])
    v = rng.normal(size=x.shape)
    v /= np.linalg.norm(v, axis=1)[:, None]
    return x, v


def run_ref(files, x, v):
    exe = os.path.join(ROOT, "oracle", "_ref", "ref_beam")
    with tempfile.TemporaryDirectory() as wd:
        for f in files:
            shutil.copyfile(os.path.join(DST, f + ".txt"), os.path.join(wd, f + ".txt"))
        inp = "".join("%.17e %.17e %.17e %.17e %.17e %.17e\n" % (tuple(a) + tuple(b)) for a, b in zip(x, v))
        out = subprocess.run([exe], input=inp, capture_output=True, text=True, cwd=wd, check=True).stdout
    rows = [list(map(float, l.split())) for l in out.strip().splitlines()]
    assert len(rows) == len(x) and all(len(r) == 24 for r in rows)
    return rows


def main():
    if len(sys.argv) > 1:
        ref = sys.argv[1]
    else:
        ref = subprocess.run(["bash", os.path.join(ROOT, "oracle", "build_ref.sh"), "--where"], capture_output=True,
                             text=True, check=True).stdout.strip()
    os.makedirs(DST, exist_ok=True)
    for f in FAMILIES:
        shutil.copyfile(os.path.join(ref, "beam_sample", f + ".txt"), os.path.join(DST, f + ".txt"))
    x, v = points()
    exp = {"x": x.tolist(), "v": v.tolist(), "cases": {}}
    for f in FAMILIES:
        exp["cases"][f] = {"files": [f], "EHdEdH": run_ref([f], x, v)}
    exp["cases"]["all"] = {"files": FAMILIES, "EHdEdH": run_ref(FAMILIES, x, v)}
    json.dump(exp, open(os.path.join(DST, "expected.json"), "w"))
    print("wrote", DST)


if __name__ == "__main__":
    main()
