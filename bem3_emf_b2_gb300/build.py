"""Build of the GB300 BEM library (sm_103a) and its command-line tools.

Everything is compiled in-tree into ``bem3_emf_b2_gb300/_build``:
  libbem3gb.so           host C library (the reference API) + CUDA kernels + C ABI
  d3b2_create_matrix     drop-in for the reference's tool of the same name
  d3b2_bv_solver         drop-in for the reference's tool of the same name
  bem3_analysis          prints fields, forces and absorbed power of a .dat
Translation units are compiled in parallel; one -gencode (sm_103a).
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
INCLUDE = os.path.join(ROOT, "include")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SRCS = ["gb_api.cu", "gb_assemble.cu", "gb_linalg.cu", "gb_tc.cu", "gb_field.cu", "gb_solve.cu", "gb_schur.cu", "gb_mlp.cu",
           "gb_gmres.cu", "gb_beam.cu"]
LIB = os.path.join(BUILD, "libbem3gb.so")
APPS = ["d3b2_create_matrix", "d3b2_bv_solver", "bem3_analysis"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r


def _newer(target, deps):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def build(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    host_dir = os.path.join(CSRC, "host")
    headers += [os.path.join(host_dir, f) for f in os.listdir(host_dir) if f.endswith(".h")]
    jobs = []
    objs = []
    for f in CU_SRCS:
        src = os.path.join(CSRC, f)
        obj = os.path.join(BUILD, f.replace(".cu", ".o"))
        objs.append(obj)
        if force or not _newer(obj, [src] + headers):
            jobs.append([NVCC] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                                         "-I", INCLUDE, "-I", CSRC, "-c", src, "-o", obj])
    for f in sorted(os.listdir(host_dir)):
        if not f.endswith(".c"):
            continue
        src = os.path.join(host_dir, f)
        obj = os.path.join(BUILD, "host_" + f.replace(".c", ".o"))
        objs.append(obj)
        if force or not _newer(obj, [src] + headers):
            jobs.append(["gcc", "-O2", "-fPIC", "-std=gnu11", "-Wall", "-Wno-unused-result", "-fopenmp",
                         "-I", INCLUDE, "-I", host_dir, "-c", src, "-o", obj])
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        for r in ex.map(_run, jobs):
            if verbose and (r.stdout or r.stderr):
                print(r.stdout + r.stderr)
    if force or jobs or not os.path.exists(LIB):
        _run([NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-Xcompiler", "-fopenmp", "-lpthread", "-lm"])
    for app in APPS:
        src = os.path.join(PKG, "apps", app + ".c")
        exe = os.path.join(BUILD, app)
        if force or not _newer(exe, [src, LIB] + headers):
            _run(["gcc", "-O2", "-std=gnu11", "-fopenmp", "-I", INCLUDE, "-o", exe, src, "-L", BUILD, "-lbem3gb",
                  "-Wl,-rpath," + BUILD, "-lm"])
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
