"""CPU oracle of the BEM hot path -- TEST INFRASTRUCTURE ONLY.

Used by tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py
as the checker; the product (bem3_emf_b2_gb300) never imports it.

  * A numpy restatement of the reference's object setup (setup2.c): Gmsh 2.2
    reading with the duplicated-element convention (:205-503), element
    geometry coefficients (:666-745), collocation nodes (:838-869), sub-domain
    lists (:751-835), wave numbers (:99-121), incident plane wave at the
    exterior nodes (mo_setup.c:704-758, ipw.c:3-89).
  * ctypes access to oracle/port/bem_port.c (C restatement of the element
    quadrature, assembly rows, domain test and field sums).
  * numpy restatements of the dense stages: coupled matrix A
    (solve_bieq2.c:209-341), inverse through LAPACK zgetrf/zgetri (the
    reference calls MKL's, solve_bieq2.c:389-395), RHS B (mo_solve.c:150-244),
    boundary values (tmatrix_bd_store :457-545).
Parity of this oracle is pinned against the reference's own outputs in
tests/golden (tests/test_oracle_port.py).
"""
import ctypes
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libbemport.so")

P44 = 0.5773502691896257645091
Z44 = np.array([-P44, P44, P44, -P44]); E44 = np.array([-P44, -P44, P44, P44])
Z34 = np.array([-0.2, 0.4, -0.2, 0.0]); E34 = np.array([-0.3464101615137754587055, 0.0, 0.3464101615137754587055, 0.0])


def build(force=False):
    """Compile the C restatement (gcc, OpenMP) into oracle/_build."""
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "port", "bem_port.c")
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
        subprocess.check_call(["gcc", "-O2", "-fPIC", "-fopenmp", "-shared", "-o", LIB, src, "-lm"])
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(LIB)
    return _lib


class _MeshArgs(ctypes.Structure):
    _fields_ = [("Ne", ctypes.c_int), ("MN", ctypes.c_int),
                ("cr", ctypes.c_void_p), ("cw", ctypes.c_void_p), ("ren", ctypes.c_void_p), ("corner", ctypes.c_void_p),
                ("etype", ctypes.c_void_p), ("sd", ctypes.c_void_p), ("sid", ctypes.c_void_p), ("sb_Ne", ctypes.c_void_p),
                ("sb_off", ctypes.c_void_p), ("kn", ctypes.c_void_p)]


def read_msh(path, MN):
    """Gmsh 2.2 ASCII with each element twice (reference setup2.c:205-503)."""
    with open(path) as f:
        tok = f.read().split()
    i = tok.index("$Nodes") + 1
    nn = int(tok[i]); i += 1
    rn = np.zeros((nn + 1, 3))
    for k in range(1, nn + 1):
        rn[k] = [float(tok[i + 1]), float(tok[i + 2]), float(tok[i + 3])]
        i += 4
    i = tok.index("$Elements") + 1
    ne = int(tok[i]) // 2; i += 1
    ed = np.zeros((ne + 1, 4), np.int32); md = np.zeros(ne + 1, np.int32); sd = np.zeros(ne + 1, np.int32)
    for e in range(1, ne + 1):
        for copy in range(2):
            et, nt = int(tok[i + 1]), int(tok[i + 2])
            tags = [int(x) for x in tok[i + 3:i + 3 + nt]]
            nv = 3 if et == 2 else 4
            nodes = [int(x) for x in tok[i + 3 + nt:i + 3 + nt + nv]]
            i += 3 + nt + nv
            dom = 0 if tags[0] == 99 else tags[0]
            if dom > MN:
                raise ValueError("domain id %d is not defined by the medium data" % dom)
            if copy == 0:
                md[e] = dom
                ed[e, :nv] = nodes
            else:
                sd[e] = dom
        if sd[e] == 0:
            sd[e], md[e] = md[e], 0
            if ed[e, 3] == 0:
                ed[e, 1], ed[e, 2] = ed[e, 2], ed[e, 1]
            else:
                ed[e, 1], ed[e, 3] = ed[e, 3], ed[e, 1]
    return rn, ed, md, sd


class Obj:
    """One BEM object (domains 0..MN), arrays 1-based in the element index."""

    def __init__(self, msh, n_media, lambda0, n_host, shift=(0.0, 0.0, 0.0)):
        MN = len(n_media)
        self.MN = MN
        self.lambda0 = lambda0
        rn, ed, md, sd = read_msh(msh, MN)
        rn = rn.copy()
        rn[1:] += np.asarray(shift, float)
        self.rn, self.ed, self.md, self.sd = rn, ed, md, sd
        ne = ed.shape[0] - 1
        self.Ne = ne
        self.etype = (ed[:, 3] != 0).astype(np.int32)
        self.etype[0] = 1
        self.n = np.array([n_host] + list(n_media), complex)
        self.kn = 2.0 * math.pi / lambda0 * self.n
        cr = np.zeros((ne + 1, 3, 4)); cw = np.zeros((ne + 1, 3, 3))
        for e in range(1, ne + 1):
            rc = rn[ed[e]].T  # [xyz][corner]
            if self.etype[e]:
                cr[e, :, 0] = 0.25 * (rc[:, 0] + rc[:, 1] + rc[:, 2] + rc[:, 3])
                cr[e, :, 1] = 0.25 * (-rc[:, 0] + rc[:, 1] + rc[:, 2] - rc[:, 3])
                cr[e, :, 2] = 0.25 * (-rc[:, 0] - rc[:, 1] + rc[:, 2] + rc[:, 3])
                cr[e, :, 3] = 0.25 * (rc[:, 0] - rc[:, 1] + rc[:, 2] - rc[:, 3])
                for d in range(3):
                    a, b = (d + 1) % 3, (d + 2) % 3
                    cw[e, d, 0] = 0.125 * ((rc[a, 0] - rc[a, 2]) * (rc[b, 1] - rc[b, 3]) - (rc[a, 1] - rc[a, 3]) * (rc[b, 0] - rc[b, 2]))
                    cw[e, d, 1] = 0.125 * ((rc[a, 2] - rc[a, 3]) * (rc[b, 0] - rc[b, 1]) - (rc[a, 0] - rc[a, 1]) * (rc[b, 2] - rc[b, 3]))
                    cw[e, d, 2] = 0.125 * ((rc[a, 1] - rc[a, 2]) * (rc[b, 0] - rc[b, 3]) - (rc[a, 0] - rc[a, 3]) * (rc[b, 1] - rc[b, 2]))
            else:
                cr[e, :, 0] = (rc[:, 0] + rc[:, 1] + rc[:, 2]) / 3.0
                cr[e, :, 1] = (-rc[:, 0] + 2.0 * rc[:, 1] - rc[:, 2]) / 3.0
                cr[e, :, 2] = (rc[:, 2] - rc[:, 0]) / math.sqrt(3.0)
                for d in range(3):
                    a, b = (d + 1) % 3, (d + 2) % 3
                    cw[e, d, 0] = (rc[a, 1] - rc[a, 0]) * (rc[b, 2] - rc[b, 0]) - (rc[b, 1] - rc[b, 0]) * (rc[a, 2] - rc[a, 0])
        self.cr, self.cw = cr, cw
        ren = np.zeros((ne + 1, 4, 3)); wen = np.zeros((ne + 1, 4, 3))
        for e in range(1, ne + 1):
            zt, et = (Z44, E44) if self.etype[e] else (Z34, E34)
            for j in range(4):
                z, h = zt[j], et[j]
                if self.etype[e]:
                    ren[e, j] = cr[e, :, 0] + cr[e, :, 1] * z + cr[e, :, 2] * h + cr[e, :, 3] * z * h
                    wen[e, j] = cw[e, :, 0] + cw[e, :, 1] * z + cw[e, :, 2] * h
                else:
                    ren[e, j] = cr[e, :, 0] + cr[e, :, 1] * z + cr[e, :, 2] * h
                    wen[e, j] = cw[e, :, 0]
        self.ren, self.wen = ren, wen
        self.corner = rn[ed]  # (ne+1, 4, 3)
        eni = -np.ones((ne + 1, 4), np.int32)
        c = 0
        for e in range(1, ne + 1):
            for j in range(4 if self.etype[e] else 3):
                eni[e, j] = c
                c += 1
        self.eni, self.NN = eni, c
        self.sids = []
        for d in range(MN + 1):
            l = [0]
            for e in range(1, ne + 1):
                if md[e] == d:
                    l.append(e)
                elif sd[e] == d:
                    l.append(-e)
            self.sids.append(np.array(l, np.int32))
        self._keep = None

    def args(self):
        sid = np.concatenate(self.sids).astype(np.int32)
        sb_ne = np.array([len(s) - 1 for s in self.sids], np.int32)
        off = np.concatenate([[0], np.cumsum([len(s) for s in self.sids])]).astype(np.int32)
        arrs = dict(cr=np.ascontiguousarray(self.cr), cw=np.ascontiguousarray(self.cw), ren=np.ascontiguousarray(self.ren),
                    corner=np.ascontiguousarray(self.corner), etype=self.etype.astype(np.int32), sd=self.sd.astype(np.int32),
                    sid=sid, sb_Ne=sb_ne, sb_off=off,
                    kn=np.ascontiguousarray(np.stack([self.kn.real, self.kn.imag], 1).ravel()))
        self._keep = arrs
        a = _MeshArgs()
        a.Ne, a.MN = self.Ne, self.MN
        for k, v in arrs.items():
            setattr(a, k, v.ctypes.data)
        return a

    # ---- assembly rows (C restatement) ----
    def rows(self, did, rows=None, type_=2):
        N = 4 * (len(self.sids[did]) - 1)
        rows = np.arange(N, dtype=np.int32) if rows is None else np.asarray(rows, np.int32)
        nr = len(rows)
        G = np.zeros((nr, N), complex); H = np.zeros((nr, N), complex)
        dG = np.zeros((nr, 2, N), complex); dH = np.zeros((nr, 2, N), complex); dF = np.zeros((nr, 3))
        a = self.args()
        lib().port_rows_c(ctypes.byref(a), did, type_, nr, rows.ctypes.data_as(ctypes.c_void_p),
                          G.ctypes.data_as(ctypes.c_void_p), H.ctypes.data_as(ctypes.c_void_p),
                          dG.ctypes.data_as(ctypes.c_void_p), dH.ctypes.data_as(ctypes.c_void_p),
                          dF.ctypes.data_as(ctypes.c_void_p))
        return G, H, dG.reshape(2 * nr, N), dH.reshape(2 * nr, N), dF

    def domain_id(self, pts):
        pts = np.ascontiguousarray(pts, float).reshape(-1, 3)
        out = np.zeros(len(pts), np.int32)
        a = self.args()
        lib().port_domain_id_c(ctypes.byref(a), len(pts), pts.ctypes.data_as(ctypes.c_void_p), out.ctypes.data_as(ctypes.c_void_p))
        return out

    def field(self, mode, type_, pts, bv, v=None):
        """bv: list over domains of dicts U,dU,E,dE,H,dH (reference layout)."""
        pts = np.ascontiguousarray(pts, float).reshape(-1, 3)
        n = len(pts)
        nout = 4 if mode == 0 else (8 if mode == 3 else 6)
        out = np.zeros((n, nout), complex)
        ret = np.zeros(n, np.int32)
        keep = []
        ptrs = (ctypes.c_void_p * (6 * (self.MN + 1)))()
        for d in range(self.MN + 1):
            for j, k in enumerate(("U", "dU", "E", "dE", "H", "dH")):
                arr = np.ascontiguousarray(bv[d][k], complex)
                keep.append(arr)
                ptrs[6 * d + j] = arr.ctypes.data
        vv = None if v is None else np.ascontiguousarray(v, float).reshape(-1, 3)
        a = self.args()
        lib().port_field_c(ctypes.byref(a), mode, type_, n, pts.ctypes.data_as(ctypes.c_void_p),
                           None if vv is None else vv.ctypes.data_as(ctypes.c_void_p), ctypes.c_double(self.lambda0), ptrs,
                           out.ctypes.data_as(ctypes.c_void_p), ret.ctypes.data_as(ctypes.c_void_p))
        return out, ret

    # ---- dense stages (numpy) ----
    def build_A(self, GH):
        """Coupled matrix from {did: (G, H)} (reference solve_bieq2.c:209-341)."""
        nn = self.NN
        na = 8 * nn
        A = np.zeros((na, na), complex)
        j = 0
        for did in range(self.MN + 1):
            G, H = GH[did]
            sid = self.sids[did]
            for cid in range(4):
                for t in range(1, len(sid)):
                    td = sid[t]
                    for tn in range(4):
                        if tn == 3 and not self.etype[abs(td)]:
                            continue
                        row = (t - 1) * 4 + tn
                        for s in range(1, len(sid)):
                            sd = sid[s]
                            asd = abs(sd)
                            mdid, sdid = self.md[asd], self.sd[asd]
                            nl = 4 if self.etype[asd] else 3
                            for l in range(nl):
                                c = self.eni[asd, l]
                                g, h = G[row, (s - 1) * 4 + l], H[row, (s - 1) * 4 + l]
                                if did == mdid:
                                    A[j, nn * cid + c] = h
                                    A[j, nn * (cid + 4) + c] = -g
                                    continue
                                k1, k2 = self.kn[mdid], self.kn[sdid]
                                delt, beps = k1 * k1 - k2 * k2, k1 * k1 / (k2 * k2)
                                sigm = 1.0 - beps
                                vn = self.wen[asd, l] / np.linalg.norm(self.wen[asd, l])
                                if cid < 3:
                                    A[j, nn * cid + c] = h
                                    A[j, nn * 3 + c] = delt * vn[cid] * g
                                    A[j, nn * (cid + 4) + c] = g
                                else:
                                    A[j, nn * 0 + c] = sigm * vn[0] * g
                                    A[j, nn * 1 + c] = sigm * vn[1] * g
                                    A[j, nn * 2 + c] = sigm * vn[2] * g
                                    A[j, nn * 3 + c] = h
                                    A[j, nn * 7 + c] = beps * g
                        j += 1
        return A


def lapack_inverse(A):
    """zgetrf + zgetri (LAPACK through scipy), as the reference's lu_dec_A."""
    from scipy.linalg import lapack
    lu, piv, info = lapack.zgetrf(A)
    if info != 0:
        raise np.linalg.LinAlgError("zgetrf info=%d" % info)
    inv, info = lapack.zgetri(lu, piv)
    if info != 0:
        raise np.linalg.LinAlgError("zgetri info=%d" % info)
    return inv


# ---- incident plane waves, coupled system and boundary values (numpy) ----
def ipw_setup(w):
    """Polarisation and wave vector of one plane wave (restates setup_ipw,
    reference mfb_src/ipw.c:65-89): dict with ki, E0, (ex, ey, ez), (hx, hy,
    hz), propagation direction and translation f."""
    ni, lam, power = float(w.get("ni", 1.0)), float(w.get("lambda0", 1.0)), float(w.get("power", 1.0))
    e0x, e0y = complex(w.get("e0x", 1.0)), complex(w.get("e0y", 0.0))
    cs = 1.0 / math.sqrt(abs(e0x) ** 2 + abs(e0y) ** 2)
    ex, ey = e0x * cs, e0y * cs
    hx, hy = -ey * ni, ex * ni
    th, ph = float(w.get("theta", 0.0)), float(w.get("phi", 0.0))
    st, ct, sp, cp = math.sin(th), math.cos(th), math.sin(ph), math.cos(ph)

    def rot(ax, ay):
        return np.array([ax * (sp * sp + cp * cp * ct) + ay * (sp * cp * ct - sp * cp),
                         ax * (sp * cp * ct - sp * cp) + ay * (sp * sp * ct + cp * cp),
                         -(ax * cp + ay * sp) * st])
    return dict(ki=2.0 * math.pi * ni / lam, E0=math.sqrt(power * 2.0 / ni), e=rot(ex, ey), h=rot(hx, hy),
                k=np.array([st * cp, st * sp, ct]), f=np.asarray(w.get("f", (0.0, 0.0, 0.0)), float))


def incident(obj, waves):
    """Incident potential Ui, dUi [(Ne+1)][4][4] at the collocation nodes of
    the exterior elements (md == 0): E and dE/dn of the summed plane waves,
    phi = 0 (restates init_boundary_data_u2, reference mo_setup.c:704-758, with
    calc_ipw_EH_dv, mfb_src/ipw.c:15-33, summed as calc_mfb_EH_dv,
    multi_fbeam.c:817-833)."""
    ne = obj.Ne
    Ui = np.zeros((ne + 1, 4, 4), complex)
    dUi = np.zeros((ne + 1, 4, 4), complex)
    ext = np.nonzero(obj.md[1:] == 0)[0] + 1
    r = obj.ren[ext]                       # (m, 4, 3)
    v = obj.wen[ext] / np.linalg.norm(obj.wen[ext], axis=2)[..., None]
    for w in waves:
        p = ipw_setup(w)
        te = p["ki"] * ((r - p["f"]) @ p["k"])
        Ee = (np.cos(te) + 1j * np.sin(te)) * p["E0"]
        gcf = 1j * p["ki"] * (v @ p["k"])
        Ui[ext, :, :3] += Ee[..., None] * p["e"]
        dUi[ext, :, :3] += (Ee * gcf)[..., None] * p["e"]
    return Ui, dUi


def _domain_columns(obj, did):
    """Per column (s, l) of domain did's matrices: valid mask, node c, main /
    sub domain of the source element, its node normal (n_bd_node,
    d3b1_elem.c:38-44), coupling constants delta, beta, sigma
    (solve_bieq2.c:270-275)."""
    sid = obj.sids[did][1:]
    asd = np.abs(sid)
    N = 4 * len(sid)
    l = np.tile(np.arange(4), len(sid))
    e = np.repeat(asd, 4)
    valid = ~((l == 3) & (obj.etype[e] == 0))
    c = obj.eni[e, l]
    mdid, sdid = obj.md[e], obj.sd[e]
    vn = obj.wen[e, l] / np.linalg.norm(obj.wen[e, l], axis=1)[:, None]
    k1, k2 = obj.kn[mdid], obj.kn[sdid]
    delt = k1 * k1 - k2 * k2
    beps = k1 * k1 / (k2 * k2)
    return dict(N=N, valid=valid, c=c, e=e, l=l, mdid=mdid, sdid=sdid, vn=vn, delt=delt, beps=beps, sigm=1.0 - beps)


def domain_rows(obj, did):
    """The rows (t - 1) * 4 + tn of domain did's matrices that become rows of
    A, in order: the fourth node of triangles is skipped
    (solve_bieq2.c:228-239)"""
    sid = obj.sids[did][1:]
    tn = np.tile(np.arange(4), len(sid))
    e = np.repeat(np.abs(sid), 4)
    return np.nonzero(~((tn == 3) & (obj.etype[e] == 0)))[0]


def build_A_rows(obj, GH, rows_of=None):
    """Rows of the coupled matrix A (8 NN columns), vectorised restatement of
    create_Amatrix_csr_dac (reference solve_bieq2.c:209-341).  rows_of None:
    GH = {did: (G, H)} full domain matrices and every row of A, in A's order;
    else GH[did] holds only the rows rows_of[did] of domain did's G and H
    (positions in the domain's N rows, fourth nodes of triangles excluded)
    and the result has, per domain and component cid = 0..3, those rows."""
    nn = obj.NN
    blocks = []
    for did in range(obj.MN + 1):
        G, H = GH[did]
        if rows_of is None:
            rows = domain_rows(obj, did)
            Gr, Hr = G[rows], H[rows]
        else:
            Gr, Hr = G, H
        nr = Gr.shape[0]
        col = _domain_columns(obj, did)
        m_main = col["valid"] & (col["mdid"] == did)
        m_sub = col["valid"] & (col["mdid"] != did)
        cm, cs = np.nonzero(m_main)[0], np.nonzero(m_sub)[0]
        for cid in range(4):
            A = np.zeros((nr, 8 * nn), complex)
            A[:, nn * cid + col["c"][cm]] = Hr[:, cm]
            A[:, nn * (cid + 4) + col["c"][cm]] = -Gr[:, cm]
            c = col["c"][cs]
            g, h = Gr[:, cs], Hr[:, cs]
            vn = col["vn"][cs]
            if cid < 3:
                A[:, nn * cid + c] = h
                A[:, nn * 3 + c] = g * (col["delt"][cs] * vn[:, cid])
                A[:, nn * (cid + 4) + c] = g
            else:
                for k in range(3):
                    A[:, nn * k + c] = g * (col["sigm"][cs] * vn[:, k])
                A[:, nn * 3 + c] = h
                A[:, nn * 7 + c] = g * col["beps"][cs]
            blocks.append(A)
    return np.concatenate(blocks)


def build_A_dense(obj, GH):
    """Coupled matrix A (na x na) from {did: (G, H)} (all rows of build_A_rows;
    same entries as Obj.build_A)."""
    return build_A_rows(obj, GH)


def build_B(obj, GH, Ui, dUi, rows_of=None):
    """Right-hand side B from the incident potential, vectorised restatement
    of create_Bmatrix_dac (reference mo_solve.c:150-244): rows of domain did
    take, over the source elements whose sub domain is did and whose main
    domain is 0, -H Ui - G dUi - G Ui_phi delta n_c (c < 3) and
    -H Ui_phi - sigma G (n . Ui) - beta G dUi_phi (c = 3).  rows_of as in
    build_A_rows (None: GH full matrices, all of B)."""
    out = []
    for did in range(obj.MN + 1):
        G, H = GH[did]
        if rows_of is None:
            rows = domain_rows(obj, did)
            G, H = G[rows], H[rows]
        col = _domain_columns(obj, did)
        m = col["valid"] & (col["mdid"] != did) & (col["mdid"] == 0)
        cs = np.nonzero(m)[0]
        e, l = col["e"][cs], col["l"][cs]
        vn = col["vn"][cs]
        Gr, Hr = G[:, cs], H[:, cs]
        u, du = Ui[e, l], dUi[e, l]
        for cid in range(4):
            if cid < 3:
                b = -Hr @ u[:, cid] - Gr @ du[:, cid] - Gr @ (u[:, 3] * col["delt"][cs] * vn[:, cid])
            else:
                b = (-Hr @ u[:, 3] - Gr @ (col["sigm"][cs] * (vn * u[:, :3]).sum(1))
                     - Gr @ (col["beps"][cs] * du[:, 3]))
            out.append(b)
    return np.concatenate(out)


def store_bv(obj, X, Ui, dUi):
    """Boundary values U, dU [(Ne_d+1)][4][4] of every domain from the solution
    X (restates tmatrix_bd_store, reference mo_solve.c:457-545)."""
    nn = obj.NN
    res = []
    for d in range(obj.MN + 1):
        sid = obj.sids[d]
        U = np.zeros((len(sid), 4, 4), complex)
        dU = np.zeros((len(sid), 4, 4), complex)
        for s in range(1, len(sid)):
            asd = abs(sid[s])
            mdid, sdid = obj.md[asd], obj.sd[asd]
            for l in range(4 if obj.etype[asd] else 3):
                c = obj.eni[asd, l]
                if d == mdid:
                    for i in range(4):
                        U[s, l, i] = X[nn * i + c]
                        dU[s, l, i] = X[nn * (i + 4) + c]
                    continue
                k1, k2 = obj.kn[mdid], obj.kn[sdid]
                delt, beps = k1 * k1 - k2 * k2, k1 * k1 / (k2 * k2)
                sigm = 1.0 - beps
                n = obj.wen[asd, l] / np.linalg.norm(obj.wen[asd, l])
                tU = np.array([X[nn * i + c] for i in range(4)])
                for i in range(3):
                    U[s, l, i] = tU[i]
                    dU[s, l, i] = -(X[nn * (i + 4) + c] + delt * tU[3] * n[i])
                    if mdid == 0:
                        U[s, l, i] += Ui[asd, l, i]
                        dU[s, l, i] += -dUi[asd, l, i]
                U[s, l, 3] = tU[3]
                dU[s, l, 3] = -(beps * X[nn * 7 + c] + sigm * np.dot(n, tU[:3]))
                if mdid == 0:
                    dU[s, l, 3] += -sigm * np.dot(n, Ui[asd, l, :3])
        res.append(dict(U=U, dU=dU))
    return res


def solve_single(obj, waves, type_=2):
    """The reference's single-object solve on the CPU: all rows of every
    domain (C restatement), A and B, X = A^-1 B through LAPACK's LU solve
    (the reference applies the zgetrf/zgetri inverse, solve_bieq2.c:343-408,
    mo_solve.c:246-274), boundary values.  Returns (bv, GH, X)."""
    from scipy.linalg import lu_factor, lu_solve
    GH = {}
    for d in range(obj.MN + 1):
        G, H, _, _, _ = obj.rows(d, type_=type_)
        GH[d] = (G, H)
    Ui, dUi = incident(obj, waves)
    A = build_A_dense(obj, GH)
    B = build_B(obj, GH, Ui, dUi)
    X = lu_solve(lu_factor(A, overwrite_a=True, check_finite=False), B, check_finite=False)
    return store_bv(obj, X, Ui, dUi), GH, X
