"""Host-side pieces that need no GPU: scene generator, struct layouts of the
drop-in headers, the C ABI exports of the built library, host setup."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from bem3_emf_b2_gb300 import meshgen

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("n", [1, 2, 8])
def test_cubed_sphere_counts_and_orientation(n):
    nodes, elems = meshgen.cubed_sphere(n, 1.0)
    assert len(nodes) == 6 * n * n + 2 and len(elems) == 6 * n * n
    assert np.allclose(np.linalg.norm(nodes, axis=1), 1.0)
    for e in elems:
        p = nodes[list(e)]
        assert np.dot(np.cross(p[1] - p[0], p[3] - p[0]), p.mean(0)) > 0


def test_cone_meshes():
    nodes, elems = meshgen.cone_tri(16, 0.5, 1.0, jitter=0.05, seed=3)
    assert len(elems) == 12 * 16 * 16   # 3072 triangles: the two-cone scene's size
    nodes, elems = meshgen.cone_mixed(6, 2, 0.3, 0.5)
    assert sum(len(e) == 3 for e in elems) == 12 and sum(len(e) == 4 for e in elems) == 12


def test_struct_layouts_match_the_reference_lp64_sizes(tmp_path):
    src = tmp_path / "sz.c"
    src.write_text('#include "bem3_emf_b2.h"\n#include <stddef.h>\nint main(){printf("%zu %zu %zu %zu %zu %zu %zu\\n",'
                   'sizeof(Bobj),sizeof(Ipw),sizeof(DOMD),sizeof(BOUD),sizeof(CMD),sizeof(SUBD),offsetof(Bobj,bd));return 0;}\n')
    exe = tmp_path / "sz"
    subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    out = subprocess.check_output([str(exe)], text=True).split()
    # the reference's own headers give 264 240 2648 1936 112 64 216 (LP64): raw struct dumps in .obj/.dat depend on it
    assert out == ["264", "240", "2648", "1936", "112", "64", "216"]


def test_beam_struct_layouts_match_the_reference(tmp_path):
    """The five angular-spectrum beam structs are stored as raw bytes after
    Bobj in .obj/.dat files (reference mo_setup.c:170-176): sizes and member
    offsets of the reference's mfb_src headers (LP64)."""
    src = tmp_path / "sz.c"
    src.write_text('#include "multi_fbeam.h"\n#include <stddef.h>\nint main(){printf("' + "%zu " * 16 + '\\n",'
                   'sizeof(Fpw),sizeof(LGb),sizeof(Bsb),sizeof(BsLGb),sizeof(RAb),offsetof(Fpw,nn),offsetof(Fpw,data),'
                   'offsetof(FpwD,nt),offsetof(LGb,lg_m),offsetof(LGbD,ph_p),offsetof(Bsb,data),offsetof(BsbD,ct),'
                   'offsetof(BsLGb,lg_m),offsetof(BsLGbD,ph_p),offsetof(RAb,nn),offsetof(RAbD,sp));return 0;}\n')
    exe = tmp_path / "sz"
    subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    out = subprocess.check_output([str(exe)], text=True).split()
    assert out == "272 280 248 264 272 104 112 112 104 160 104 112 104 144 104 152".split()


def _declared(header):
    txt = open(os.path.join(ROOT, "include", header)).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    names = re.findall(r"^[A-Za-z_][\w \t\*]*?\b([A-Za-z_]\w*)\s*\([^;{]*\)\s*;", txt, re.M)
    return [n for n in names if n not in ("if", "for", "while")]


def test_library_exports_every_declared_entry_point(gb_build):
    lib = ctypes.CDLL(os.path.join(gb_build, "libbem3gb.so"))
    missing = []
    for h in ("gb_bem.h", "gb_scene.h", "gb_mlp.h", "bem3_emf_b2.h", "d3b1_elem.h", "multi_fbeam.h", "ipw.h", "my_utils.h",
              "gauleg.h", "osu_mksa.h"):
        for name in _declared(h):
            if not hasattr(lib, name):
                missing.append((h, name))
    assert not missing, missing


def test_host_setup_without_gpu(gb_build, tmp_path):
    """gbh_scene_open performs only host work (files, geometry, incident
    field); counts must match the oracle's independent setup."""
    from bem3_emf_b2_gb300 import Scene
    from oracle import port
    wd = str(tmp_path)
    nodes, elems = meshgen.cone_mixed(6, 2, 0.3, 0.5)
    meshgen.write_mesh(os.path.join(wd, "m.msh"), nodes, elems)
    meshgen.write_medium(os.path.join(wd, "med.txt"), [1.5 + 0.05j])
    meshgen.write_ipw(os.path.join(wd, "ipw.txt"), [dict(lambda0=1.0, ni=1.33, power=1.0)])
    sc = Scene(os.path.join(wd, "med.txt"), os.path.join(wd, "m.msh"), os.path.join(wd, "ipw.txt"))
    sc.close()
    o = port.Obj(os.path.join(wd, "m.msh"), [1.5 + 0.05j], 1.0, 1.33)
    assert o.NN == 12 * 3 + 12 * 4 and o.Ne == 24


def test_butterfly_parameters(gb_build):
    """gbi_rbt_params (host code of the library, no GPU needed): 4 n
    parameters e^{rho/10}, rho in [-1/2, 1/2), reproducible for an order and
    different across orders (the factorisations are reproducible)."""
    import numpy as np
    lib = ctypes.CDLL(os.path.join(gb_build, "libbem3gb.so"))
    lib.gbi_rbt_params.argtypes = [ctypes.c_int, ctypes.c_void_p]
    lib.gbi_rbt_params.restype = None

    def params(n):
        h = np.zeros(4 * n, np.float32)
        lib.gbi_rbt_params(n, h.ctypes.data)
        return h
    a, b, c = params(1024), params(1024), params(2048)
    assert np.array_equal(a, b)
    assert not np.array_equal(a, c[:4096])
    lo, hi = np.float32(np.exp(-0.05)), np.float32(np.exp(0.05))
    assert a.min() >= lo * (1 - 1e-6) and a.max() <= hi * (1 + 1e-6)
    rho = 10.0 * np.log(a.astype(np.float64))
    assert abs(rho.mean()) < 0.03 and 0.25 < rho.std() < 0.32  # uniform on [-1/2, 1/2): std 0.289
