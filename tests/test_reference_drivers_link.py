"""CPU: the reference's own drivers and example programs compile unchanged
against this repository's headers (include/) and link against libbem3gb.so.

The reference's d3b2_create_matrix.c, d3b2_bv_solver.c (d3b2_src/) and
example1.c, example2.c, example4.c are compiled with no edit, no extra define
and no shim; every symbol they call must resolve in libbem3gb.so (undefined
symbols fail the link).  Each source is copied byte for byte into a scratch
directory first: a quoted #include searches the including file's own
directory before -I, so in d3b2_src/ the reference's headers would shadow
these.  example3.c
needs libpng, which this image lacks.  Runs only where the reference's sources
are present (the GPU machine has none); running the programs needs a GPU and is
covered by the tools' own GPU tests."""
import os
import subprocess

import pytest

import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REFSRC = oracle.reference_dir()
PROGRAMS = ["d3b2_src/d3b2_create_matrix.c", "d3b2_src/d3b2_bv_solver.c", "example1.c", "example2.c", "example4.c"]


@pytest.mark.skipif(not REFSRC, reason="reference sources not present")
@pytest.mark.parametrize("src", PROGRAMS)
def test_reference_program_links_against_library(src, gb_build, tmp_path):
    import shutil
    exe = os.path.join(str(tmp_path), os.path.basename(src)[:-2])
    copy = os.path.join(str(tmp_path), os.path.basename(src))
    shutil.copyfile(os.path.join(REFSRC, src), copy)
    cmd = ["gcc", "-O2", "-std=gnu11", "-fopenmp", "-I", os.path.join(ROOT, "include"), "-o", exe,
           copy, "-L", gb_build, "-lbem3gb", "-Wl,-rpath," + gb_build, "-Wl,--no-undefined", "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert os.path.exists(exe)
    # every symbol the program needs from the library is defined there
    und = subprocess.run(["nm", "-u", exe], capture_output=True, text=True).stdout.split()
    lib = subprocess.run(["nm", "-D", "--defined-only", os.path.join(gb_build, "libbem3gb.so")], capture_output=True,
                         text=True).stdout.split()
    defined = set(lib[2::3])
    ours = [s for s in und if s in defined]
    assert ours, "the program uses nothing from libbem3gb.so"
