"""GPU: incident fields of the reference's beam families (plane wave, focused
plane wave, Laguerre-Gaussian, Bessel, Bessel with spiral phase,
radial/azimuthal), evaluated by gb_beam.cu behind the reference's beam API.

Golden values: the unmodified reference (oracle/_ref/ref_beam,
calc_mfb_EH_dv of mfb_src/multi_fbeam.c) on the reference's own beam_sample
files, at seeded points in a 3 lambda box about the foci and 5..20 lambda
out (tests/golden/make_beams.py).

  * each family alone and all six summed: E, H, dE/dv, dH/dv within 1e-11 of
    the largest golden magnitude of the case;
  * the per-family single-point functions (calc_fpw_EH_dv, ...) give the
    batched values;
  * a .dat round trip (gb_mfb_write / gb_mfb_read) keeps every beam.
"""
import ctypes
import json
import os
import shutil

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "beams")
BOBJ = 264           # sizeof(Bobj), LP64
BD = 216             # offsetof(Bobj, bd): six pointers ipw, fpw, lgb, bsb, blg, rab


def _lib():
    from bem3_emf_b2_gb300 import lib
    L = lib()
    vp, ci = ctypes.c_void_p, ctypes.c_int
    L.init_mfb.argtypes = [vp]
    L.setup_mfb.argtypes = [vp]
    L.free_mfb.argtypes = [vp]
    for f in ("ipw", "fpw", "lgb", "bsb", "blg", "rab"):
        getattr(L, "read_data_mfb_" + f).argtypes = [ctypes.c_char_p, vp]
        getattr(L, "read_data_mfb_" + f).restype = ci
    L.calc_mfb_EH_dv_points.argtypes = [vp, ci, vp, vp, vp, vp, vp, vp]
    L.calc_mfb_EH_points.argtypes = [vp, ci, vp, vp, vp]
    return L


def _beams(L, wd, files):
    obj = ctypes.create_string_buffer(BOBJ)
    L.init_mfb(obj)
    for f in files:
        p = os.path.join(wd, f + ".txt")
        shutil.copyfile(os.path.join(GOLD, f + ".txt"), p)
        assert getattr(L, "read_data_mfb_" + f)(p.encode(), obj) > 0
    L.setup_mfb(obj)
    return obj


def _eval(L, obj, x, v):
    n = len(x)
    out = [np.zeros((n, 3), complex) for _ in range(4)]
    L.calc_mfb_EH_dv_points(obj, n, x.ctypes.data, v.ctypes.data, *[o.ctypes.data for o in out])
    return np.concatenate([np.stack([o.real, o.imag], -1).reshape(n, 6) for o in out], 1)


def _golden():
    g = json.load(open(os.path.join(GOLD, "expected.json")))
    return np.ascontiguousarray(g["x"]), np.ascontiguousarray(g["v"]), g["cases"]


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["ipw", "fpw", "lgb", "bsb", "blg", "rab", "all"])
def test_beam_family_matches_reference(case, gb_build, tmp_path):
    L = _lib()
    x, v, cases = _golden()
    c = cases[case]
    obj = _beams(L, str(tmp_path), c["files"])
    got = _eval(L, obj, x, v)
    ref = np.array(c["EHdEdH"])
    for g, name in enumerate(("E", "H", "dE", "dH")):
        a, b = got[:, 6 * g:6 * g + 6], ref[:, 6 * g:6 * g + 6]
        err = np.abs(a - b).max() / np.abs(b).max()
        print("%s %s: %.2e" % (case, name, err))
        assert err <= 1e-11, (case, name, err)
    # E and H alone (no derivative) are the same numbers
    n = len(x)
    E = np.zeros((n, 3), complex)
    H = np.zeros((n, 3), complex)
    L.calc_mfb_EH_points(obj, n, x.ctypes.data, E.ctypes.data, H.ctypes.data)
    assert np.allclose(np.stack([E.real, E.imag], -1).reshape(n, 6), got[:, :6], rtol=0, atol=1e-13 * np.abs(ref).max())
    L.free_mfb(obj)


@pytest.mark.gpu
def test_single_beam_functions_and_storage(gb_build, tmp_path):
    """calc_<family>_EH_dv on the first beam of each file equals the batched
    sum of that beam alone; gb_mfb_write / gb_mfb_read keep all beams."""
    L = _lib()
    vp = ctypes.c_void_p
    x, v, cases = _golden()
    wd = str(tmp_path)
    obj = _beams(L, wd, ["ipw", "fpw", "lgb", "bsb", "blg", "rab"])
    ptrs = np.frombuffer(obj.raw[BD:BD + 48], dtype=np.uint64)
    names = {"fpw": ("calc_fpw_EH_dv", 1), "lgb": ("calc_lgb_EH_dv", 2), "bsb": ("calc_bsb_EH_dv", 3),
             "blg": ("calc_bslgb_EH_dv", 4), "rab": ("calc_rab_EH_dv", 5)}
    for fam, (fn, slot) in names.items():
        f = getattr(L, fn)
        f.argtypes = [vp] * 7
        # a file holding only its first beam
        lines = open(os.path.join(GOLD, fam + ".txt")).read().splitlines()
        first = os.path.join(wd, "first_" + fam + ".txt")
        open(first, "w").write("\n".join(lines[:2] + ["1"] + lines[3:5]) + "\n")
        o1 = ctypes.create_string_buffer(BOBJ)
        L.init_mfb(o1)
        assert getattr(L, "read_data_mfb_" + fam)(first.encode(), o1) == 1
        L.setup_mfb(o1)
        want = _eval(L, o1, x[:6], v[:6])
        for p in range(6):
            out = [np.zeros(3, complex) for _ in range(4)]
            xp, vp_ = np.ascontiguousarray(x[p]), np.ascontiguousarray(v[p])
            f(*[o.ctypes.data for o in out], xp.ctypes.data, vp_.ctypes.data, int(ptrs[slot]))
            got = np.concatenate([np.stack([o.real, o.imag], -1).ravel() for o in out])
            assert np.array_equal(got, want[p]), (fam, p)
        L.free_mfb(o1)
    # storage round trip
    libc = ctypes.CDLL(None)
    libc.fopen.restype = vp
    libc.fopen.argtypes = [ctypes.c_char_p, ctypes.c_char_p]
    libc.fclose.argtypes = [vp]
    L.gb_mfb_write.argtypes = [vp, vp]
    L.gb_mfb_read.argtypes = [vp, vp]
    path = os.path.join(wd, "beams.bin").encode()
    fp = libc.fopen(path, b"wb")
    L.gb_mfb_write(fp, obj)
    libc.fclose(fp)
    back = ctypes.create_string_buffer(BOBJ)
    fp = libc.fopen(path, b"rb")
    L.gb_mfb_read(fp, back)
    libc.fclose(fp)
    assert back.raw[:BD] == obj.raw[:BD]  # counts, names, n_0, lambda_0, omega
    assert np.array_equal(_eval(L, back, x, v), _eval(L, obj, x, v))
    L.free_mfb(back)
    L.free_mfb(obj)
