"""Readers of the reference's binary files (.obj, .dat, .cmat).

Layouts follow the reference's writers: dat_write2 (solve_bieq2.c:439-502)
for the single-object .obj file, mo_dat_write (mo_setup.c:147-203) for the
multi-object .dat file, and the headerless row-major .cmat matrices
(solve_bieq2.c:168-183,403).  Structs stored as raw bytes have the LP64
sizes of the reference: Bobj 264 bytes, Ipw 240 bytes.
"""
import numpy as np

SIZEOF_BOBJ = 264
SIZEOF_IPW = 240
FNLGTH = 256


class _Reader:
    def __init__(self, data):
        self.b = data
        self.p = 0

    def take(self, n):
        v = self.b[self.p:self.p + n]
        if len(v) != n:
            raise ValueError("truncated file at byte %d" % self.p)
        self.p += n
        return v

    def arr(self, dtype, n):
        dt = np.dtype(dtype)
        return np.frombuffer(self.take(dt.itemsize * n), dtype=dt).copy()

    def i32(self):
        return int(self.arr("<i4", 1)[0])

    def cstr(self, n):
        s = self.take(n)
        return s.split(b"\0", 1)[0].decode("latin-1")


def _read_object_body(r, with_values):
    o = {}
    o["med_fn"] = r.cstr(128)
    o["msh_fn"] = r.cstr(128)
    o["rv"] = r.arr("<f8", 3)
    o["th"] = float(r.arr("<f8", 1)[0])
    o["tv"] = r.arr("<f8", 3)
    MN = r.i32()
    o["MN"] = MN
    o["n"] = r.arr("<c16", MN + 1)
    o["kn"] = r.arr("<c16", MN + 1)
    bobj = r.take(SIZEOF_BOBJ)
    counts = [int(np.frombuffer(bobj[32 * i:32 * i + 4], "<i4")[0]) for i in range(6)]
    o["n_ipw"] = counts[0]
    if any(counts[1:]):
        raise ValueError("beam types other than plane waves are not supported")
    o["ipw_raw"] = r.take(SIZEOF_IPW * counts[0])
    Nn = r.i32()
    Ne = r.i32()
    o["Nn"], o["Ne"] = Nn, Ne
    o["rn"] = r.arr("<f8", 3 * (Nn + 1)).reshape(Nn + 1, 3)
    o["ed"] = r.arr("<i4", 4 * (Ne + 1)).reshape(Ne + 1, 4)
    o["NN"] = r.i32()
    o["eni"] = r.arr("<i4", 4 * (Ne + 1)).reshape(Ne + 1, 4)
    o["md"] = r.arr("<i4", Ne + 1)
    o["sd"] = r.arr("<i4", Ne + 1)
    o["gd"] = r.arr("<i4", Ne + 1)
    o["ren"] = r.arr("<f8", 12 * (Ne + 1)).reshape(Ne + 1, 4, 3)
    o["wen"] = r.arr("<f8", 12 * (Ne + 1)).reshape(Ne + 1, 4, 3)
    o["sb"] = []
    for _ in range(MN + 1):
        sb = {}
        ne = r.i32()
        sb["Ne"] = ne
        sb["sid"] = r.arr("<i4", ne + 1)
        if with_values:
            sb["U"] = r.arr("<c16", 16 * (ne + 1)).reshape(ne + 1, 4, 4)
            sb["dU"] = r.arr("<c16", 16 * (ne + 1)).reshape(ne + 1, 4, 4)
            for k in ("E", "dE", "H", "dH"):
                sb[k] = r.arr("<c16", 12 * (ne + 1)).reshape(ne + 1, 4, 3)
        o["sb"].append(sb)
    return o


def read_obj(path):
    """Single-object file written by d3b2_create_matrix."""
    with open(path, "rb") as f:
        r = _Reader(f.read())
    o = _read_object_body(r, with_values=False)
    o["cmat"] = []
    for _ in range(o["MN"] + 1):
        o["cmat"].append({k: r.cstr(128) for k in ("G", "H", "dG", "dH", "dF")})
    o["invA"] = r.cstr(128)
    return o


def read_dat(path):
    """Multi-object result file written by d3b2_bv_solver."""
    with open(path, "rb") as f:
        r = _Reader(f.read())
    N = r.i32()
    objs = []
    for _ in range(N):
        mod_fn = r.cstr(FNLGTH)
        rs = r.arr("<f8", 3)
        o = _read_object_body(r, with_values=True)
        o["mod_fn"], o["rs"] = mod_fn, rs
        objs.append(o)
    return objs


def read_cmat(path, shape, dtype="<c16"):
    a = np.fromfile(path, dtype=dtype)
    n = int(np.prod(shape))
    if a.size != n:
        raise ValueError("%s: %d values, expected %d" % (path, a.size, n))
    return a.reshape(shape)


def read_domain_cmats(obj, did, workdir="."):
    """G, H, dG, dH, dF of domain did of a read_obj() result (files relative to workdir)."""
    import os
    N = 4 * obj["sb"][did]["Ne"]
    names = obj["cmat"][did]
    out = {}
    for k, shape, dt in (("G", (N, N), "<c16"), ("H", (N, N), "<c16"), ("dG", (2 * N, N), "<c16"),
                         ("dH", (2 * N, N), "<c16"), ("dF", (N, 3), "<f8")):
        out[k] = read_cmat(os.path.join(workdir, names[k]), shape, dt)
    return out


def rel_fro(a, b):
    """Relative Frobenius error ||a-b|| / ||b|| (0 if both are zero)."""
    a = np.asarray(a)
    b = np.asarray(b)
    nb = np.linalg.norm(b.ravel())
    d = np.linalg.norm((a - b).ravel())
    if nb == 0.0:
        return float(d)
    return float(d / nb)
