"""Synthetic scenes for the BEM hot path, written in the reference's input formats.

Meshes are Gmsh 2.2 ASCII files in the reference's convention (reference
setup2.c:205-503): every surface element appears twice, id 2i-1 with the
physical tag of the object's medium and the nodes counter-clockwise seen from
outside, id 2i with tag 99 (the open region) and the reversed node order.

  cubed_sphere   sphere of radius r, n x n bilinear quadrangles per cube face
                 (6 n^2 elements, 6 n^2 + 2 nodes)
  cube           cube of a given side, n x n planar quadrangles per face
  cone_tri       right circular cone meshed with linear triangles on rings of
                 6k nodes (12 m^2 triangles), seeded tangential node jitter
  cone_mixed     cone with quadrangle rings and triangle fans at apex and base
                 centre (mixed ELT3/ELT4 mesh)
Medium (medium_data.txt), plane wave (ipw.txt) and object-settings files use
the reference's text layouts.
"""
import math

import numpy as np


def _write_msh(path, nodes, elems, phys=1):
    """nodes: (Nn,3); elems: list of node-index tuples (0-based), outward CCW."""
    with open(path, "w") as f:
        f.write("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$Nodes\n%d\n" % len(nodes))
        for i, p in enumerate(nodes):
            f.write("%d %.17g %.17g %.17g\n" % (i + 1, p[0], p[1], p[2]))
        f.write("$EndNodes\n$Elements\n%d\n" % (2 * len(elems)))
        for i, e in enumerate(elems):
            et = 3 if len(e) == 4 else 2
            ids = [v + 1 for v in e]
            rev = [ids[0]] + ids[:0:-1]
            f.write("%d %d 2 %d 1 %s\n" % (2 * i + 1, et, phys, " ".join(map(str, ids))))
            f.write("%d %d 2 99 1 %s\n" % (2 * i + 2, et, " ".join(map(str, rev))))


def _orient(nodes, elems, center):
    out = []
    for e in elems:
        p = np.array([nodes[v] for v in e])
        n = np.cross(p[1] - p[0], p[-1] - p[0])
        c = p.mean(axis=0) - center
        out.append(tuple(e) if np.dot(n, c) > 0 else (e[0],) + tuple(e[:0:-1]))
    return out


def cubed_sphere(n, radius=1.0, center=(0.0, 0.0, 0.0)):
    """Nodes and quadrangles of a cubed sphere (gnomonic-free: cube lattice
    points projected radially)."""
    key = {}
    nodes = []

    def node(i, j, k):
        t = (i, j, k)
        if t not in key:
            p = np.array([2.0 * i / n - 1.0, 2.0 * j / n - 1.0, 2.0 * k / n - 1.0])
            key[t] = len(nodes)
            nodes.append(p / np.linalg.norm(p) * radius + np.asarray(center, float))
        return key[t]

    elems = []
    for axis in range(3):
        for side in (0, n):
            for u in range(n):
                for v in range(n):
                    q = []
                    for du, dv in ((0, 0), (1, 0), (1, 1), (0, 1)):
                        c = [0, 0, 0]
                        c[axis] = side
                        c[(axis + 1) % 3] = u + du
                        c[(axis + 2) % 3] = v + dv
                        q.append(node(*c))
                    elems.append(tuple(q))
    nodes = np.array(nodes)
    return nodes, _orient(nodes, elems, np.asarray(center, float))


def cube(n, side=1.0, center=(0.0, 0.0, 0.0)):
    """Nodes and planar quadrangles of a cube of the given side, n x n per
    face (6 n^2 elements, 6 n^2 + 2 nodes), outward orientation."""
    key = {}
    nodes = []
    h = 0.5 * side

    def node(i, j, k):
        t = (i, j, k)
        if t not in key:
            key[t] = len(nodes)
            nodes.append(np.array([(2.0 * i / n - 1.0) * h, (2.0 * j / n - 1.0) * h, (2.0 * k / n - 1.0) * h])
                         + np.asarray(center, float))
        return key[t]

    elems = []
    for axis in range(3):
        for s in (0, n):
            for u in range(n):
                for v in range(n):
                    q = []
                    for du, dv in ((0, 0), (1, 0), (1, 1), (0, 1)):
                        c = [0, 0, 0]
                        c[axis] = s
                        c[(axis + 1) % 3] = u + du
                        c[(axis + 2) % 3] = v + dv
                        q.append(node(*c))
                    elems.append(tuple(q))
    nodes = np.array(nodes)
    return nodes, _orient(nodes, elems, np.asarray(center, float))


def cone_tri(m, radius=0.5, height=1.0, jitter=0.05, seed=0):
    """Cone with apex (0,0,height), base at z=0: lateral surface and base disk,
    each with rings of 6k nodes (k = 1..m) and 6(2k-1) triangles between
    rings; interior nodes jittered tangentially by <= jitter x local edge."""
    rng = np.random.default_rng(seed)
    nodes = []
    elems = []

    def ring_tri(inner, outer, k):
        # inner: 6(k-1) node ids (or [apex]), outer: 6k node ids
        if k == 1:
            for j in range(6):
                elems.append((inner[0], outer[j], outer[(j + 1) % 6]))
            return
        ni, no = len(inner), len(outer)
        i = j = 0
        while i < ni or j < no:
            # advance along the ring whose next angle is smaller
            ai = (i + 1) / ni if i < ni else 2.0
            ao = (j + 1) / no if j < no else 2.0
            if ao <= ai:
                elems.append((inner[i % ni], outer[j % no], outer[(j + 1) % no]))
                j += 1
            else:
                elems.append((inner[i % ni], outer[j % no], inner[(i + 1) % ni]))
                i += 1

    def surf(zfun, rfun, apex_pt, jit_scale):
        rings = [[len(nodes)]]
        nodes.append(np.array(apex_pt, float))
        for k in range(1, m + 1):
            ids = []
            rk = rfun(k)
            for j in range(6 * k):
                th = 2.0 * math.pi * j / (6 * k)
                if k < m and jitter > 0:
                    th += rng.uniform(-1, 1) * jitter * (2.0 * math.pi / (6 * k))
                    rr = rk + rng.uniform(-1, 1) * jitter * jit_scale
                else:
                    rr = rk
                ids.append(len(nodes))
                nodes.append(np.array([rr * math.cos(th), rr * math.sin(th), zfun(rr)]))
            rings.append(ids)
        return rings

    # lateral surface: z = height (1 - rho/radius)
    lat = surf(lambda rr: height * (1.0 - rr / radius), lambda k: radius * k / m, (0.0, 0.0, height), radius / m)
    for k in range(1, m + 1):
        ring_tri(lat[k - 1], lat[k], k)
    rim = lat[m]
    # base disk: shares the rim
    base_rings = [[len(nodes)]]
    nodes.append(np.array([0.0, 0.0, 0.0]))
    for k in range(1, m):
        ids = []
        for j in range(6 * k):
            th = 2.0 * math.pi * j / (6 * k)
            rr = radius * k / m
            if jitter > 0:
                th += rng.uniform(-1, 1) * jitter * (2.0 * math.pi / (6 * k))
                rr += rng.uniform(-1, 1) * jitter * radius / m
            ids.append(len(nodes))
            nodes.append(np.array([rr * math.cos(th), rr * math.sin(th), 0.0]))
        base_rings.append(ids)
    base_rings.append(rim)
    for k in range(1, m + 1):
        ring_tri(base_rings[k - 1], base_rings[k], k)
    nodes = np.array(nodes)
    center = np.array([0.0, 0.0, height / 4.0])
    return nodes, _orient(nodes, elems, center)


def cone_mixed(nth, nr, radius=0.5, height=1.0):
    """Cone with quadrangle rings (nth nodes per ring) and triangle fans at the
    apex and at the base centre: 2 nth triangles, 2 nth (nr-1) quadrangles."""
    nodes = [np.array([0.0, 0.0, height])]
    lat = [[0]]
    for k in range(1, nr + 1):
        rr = radius * k / nr
        ids = []
        for j in range(nth):
            th = 2.0 * math.pi * (j + 0.5 * (k % 2)) / nth
            ids.append(len(nodes))
            nodes.append(np.array([rr * math.cos(th), rr * math.sin(th), height * (1.0 - k / nr)]))
        lat.append(ids)
    base = [[len(nodes)]]
    nodes.append(np.array([0.0, 0.0, 0.0]))
    for k in range(1, nr):
        rr = radius * k / nr
        ids = []
        for j in range(nth):
            th = 2.0 * math.pi * (j + 0.5 * (nr % 2)) / nth
            ids.append(len(nodes))
            nodes.append(np.array([rr * math.cos(th), rr * math.sin(th), 0.0]))
        base.append(ids)
    base.append(lat[nr])
    elems = []
    for rings in (lat, base):
        for j in range(nth):
            elems.append((rings[0][0], rings[1][j], rings[1][(j + 1) % nth]))
        for k in range(1, nr):
            a, b = rings[k], rings[k + 1]
            for j in range(nth):
                elems.append((a[j], b[j], b[(j + 1) % nth], a[(j + 1) % nth]))
    nodes = np.array(nodes)
    return nodes, _orient(nodes, elems, np.array([0.0, 0.0, height / 4.0]))


def batch_scene(seed, n_obj, box=20.0, size=(0.3, 1.5), elems=(200, 6000), n_range=(1.33, 2.0)):
    """Seeded multi-object scene: n_obj non-overlapping spheres, cubes and
    cones in a cube of side box centred at the origin, characteristic size
    uniform in size, element count uniform in elems (the nearest the
    generators allow), real refractive index uniform in n_range, random
    orientation.  Returns a list of dicts: kind, nodes (already rotated and
    placed), elems, n, centre, radius (bounding)."""
    rng = np.random.default_rng(seed)
    out = []
    kinds = ("sphere", "cube", "cone")
    tries = 0
    while len(out) < n_obj:
        tries += 1
        if tries > 10000:
            raise RuntimeError("batch_scene: the objects do not fit in the box")
        kind = kinds[rng.integers(3)]
        s = rng.uniform(*size)
        ne = rng.uniform(*elems)
        if kind == "sphere":
            k = max(2, int(round(math.sqrt(ne / 6.0))))
            nodes, el = cubed_sphere(k, 0.5 * s)
            rad = 0.5 * s
        elif kind == "cube":
            k = max(2, int(round(math.sqrt(ne / 6.0))))
            nodes, el = cube(k, s)
            rad = 0.5 * math.sqrt(3.0) * s
        else:
            k = max(2, int(round(math.sqrt(ne / 12.0))))
            nodes, el = cone_tri(k, 0.5 * s, s, jitter=0.05, seed=int(rng.integers(1 << 30)))
            nodes = nodes - np.array([0.0, 0.0, 0.25 * s])
            rad = math.sqrt((0.5 * s) ** 2 + (0.75 * s) ** 2)
        axis = rng.normal(size=3)
        nodes = transform(nodes, axis / np.linalg.norm(axis), rng.uniform(0.0, 2.0 * math.pi))
        c = rng.uniform(-0.5 * box + rad, 0.5 * box - rad, 3)
        if any(np.linalg.norm(c - o["centre"]) < 1.05 * (rad + o["radius"]) for o in out):
            continue
        out.append(dict(kind=kind, nodes=nodes + c, elems=el, n=float(rng.uniform(*n_range)), centre=c, radius=rad))
    return out


def random_waves(seed, n, lambda0=1.0, ni=1.33, power=1.0):
    """n plane waves with directions uniform on the sphere and uniformly
    random linear polarisation angles (ipw.txt parameters)"""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        th = math.acos(1.0 - 2.0 * rng.uniform())
        ph = rng.uniform(0.0, 2.0 * math.pi)
        psi = rng.uniform(0.0, math.pi)
        out.append(dict(lambda0=lambda0, ni=ni, power=power, e0x=math.cos(psi), e0y=math.sin(psi), theta=th, phi=ph))
    return out


def transform(nodes, axis=(1.0, 0.0, 0.0), angle=0.0, shift=(0.0, 0.0, 0.0)):
    """Rodrigues rotation then translation (the reference's convention)."""
    a = np.asarray(axis, float)
    a = a / np.linalg.norm(a)
    c, s = math.cos(angle), math.sin(angle)
    K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
    R = c * np.eye(3) + s * K + (1 - c) * np.outer(a, a)
    return nodes @ R.T + np.asarray(shift, float)


def write_mesh(path, nodes, elems, phys=1):
    _write_msh(path, nodes, elems, phys)


def write_medium(path, indices):
    """indices: refractive index of media 1..MN (complex)."""
    with open(path, "w") as f:
        f.write("## medium data file for bem3_emf_b2\n# number of medium\n%d\n" % len(indices))
        f.write("# real(refractive_index) imag(refractive_index)\n")
        for n in indices:
            n = complex(n)
            f.write("%.17g %.17g\n" % (n.real, n.imag))


def write_ipw(path, waves):
    """waves: list of dicts lambda0, ni, power, e0x, e0y, f=(fx,fy,fz), theta, phi."""
    with open(path, "w") as f:
        f.write("## plane wave\n# number of waves\n%d\n" % len(waves))
        f.write("#lambda0 ni power real(e0x) imag(e0x) real(e0y) imag(e0y) fx fy fz theta phi\n")
        for w in waves:
            e0x, e0y = complex(w.get("e0x", 1.0)), complex(w.get("e0y", 0.0))
            fx, fy, fz = w.get("f", (0.0, 0.0, 0.0))
            f.write("%.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g\n" % (
                w.get("lambda0", 1.0), w.get("ni", 1.0), w.get("power", 1.0), e0x.real, e0x.imag, e0y.real,
                e0y.imag, fx, fy, fz, w.get("theta", 0.0), w.get("phi", 0.0)))


def write_object_settings(path, objs, reset=0):
    """objs: list of (obj_file, (sx, sy, sz))."""
    with open(path, "w") as f:
        f.write("# number_of_objects reset_flag_of_incident_field(0:no reset, 1:reset)\n")
        f.write("%d %d\n" % (len(objs), reset))
        f.write("# object_data_file_name shitf_x shift_y shit_z\n")
        for fn, s in objs:
            f.write("%s %.17g %.17g %.17g\n" % (fn, s[0], s[1], s[2]))
