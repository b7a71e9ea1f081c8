"""The reference build used as the oracle (oracle/_ref) against the
reference's own shipped results: the total field that its example1 printed in
verification1/example1.log and analysis_sample3/example1_ex30.log for the
shipped .dat files.  Runs only where the reference sources are present (the
container that generates the golden fixtures)."""
import os
import re
import subprocess

import numpy as np
import pytest

import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REFSRC = oracle.reference_dir() or ""
REF = os.path.join(ROOT, "oracle", "_ref")

CASES = [("verification1/v1.dat", "verification1/example1.log"),
         ("verification1/combined_object/vc.dat", "verification1/combined_object/example1.log"),
         ("analysis_sample3/ex30.dat", "analysis_sample3/example1_ex30.log")]


def _log_fields(path):
    txt = open(path).read()
    vals = re.findall(r"^[EH][xyz] =\s*([-+0-9.e]+)\s*([-+0-9.e]+) I", txt, re.M)
    v = np.array([[float(a), float(b)] for a, b in vals[:12]]).reshape(2, 6, 2)
    return v


@pytest.mark.skipif(not REFSRC, reason="reference sources not present")
@pytest.mark.parametrize("dat,log", CASES)
def test_ref_reproduces_shipped_logs(dat, log, tmp_path):
    if not os.path.exists(os.path.join(REF, "ref_point")):
        subprocess.check_call([os.path.join(ROOT, "oracle", "build_ref.sh"), REFSRC], stdout=subprocess.DEVNULL)
    out = subprocess.run([os.path.join(REF, "ref_point"), os.path.join(REFSRC, dat), "0.3", "0.0", "1.1"],
                         capture_output=True, text=True, check=True, cwd=str(tmp_path)).stdout
    mine = np.array([[float(x) for x in l.split()[2:]] for l in out.splitlines()]).reshape(2, 6, 2)
    ref = _log_fields(os.path.join(REFSRC, log))
    for t in range(2):
        err = np.linalg.norm(mine[t] - ref[t]) / np.linalg.norm(ref[t])
        assert err < 1e-13, "type %d relative difference %g" % (t, err)


@pytest.mark.skipif(not REFSRC, reason="reference sources not present")
def test_verification1_fixture_matches_reference():
    """The committed verification1 fixture (inputs and the printed values)
    is what make_verification1.py extracts from the reference's own files."""
    import filecmp
    import importlib.util
    import json
    spec = importlib.util.spec_from_file_location("mkv1", os.path.join(ROOT, "tests", "golden", "make_verification1.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    committed = json.load(open(os.path.join(ROOT, "tests", "golden", "verification1", "expected.json")))
    assert mod.extract(os.path.join(REFSRC, "verification1")) == committed
    assert len(committed["fields"]) == 2 and len(committed["force"]) == 4 and len(committed["absorb"]) == 4
    assert len(committed["cc"]) == 10
    for f in mod.FILES:
        assert filecmp.cmp(os.path.join(REFSRC, "verification1", f), os.path.join(ROOT, "tests", "golden", "verification1", f),
                           shallow=False), f
