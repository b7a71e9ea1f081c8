"""Benchmark of the GB300 BEM hot path: seconds per scene.

One step = one scene solved on the GPU: coefficient-matrix assembly of every
domain of every object (GLN x GLN quadrature, GHN fallback, singular self
terms), the factorisation of each object's coupled system, the multiple-
scattering iteration (reference mo_solve_bv: scattered potentials of the other
objects, right-hand sides, refined solves, the reference's convergence rule),
the E/H boundary values and normal derivatives, and the radiation force and
torque of every object.

Default workload (--workload cones): two right circular cones (base radius
0.5, height 1, n = 1.59 in n = 1.33, lengths in vacuum wavelengths), 3,072
linear triangles each (na = 73,728 unknowns per cone), cone 2 rotated pi about
x and shifted 1.5 along x, right-circularly polarised plane wave along +z.
This is the largest of the reference-defined configurations that fits one
GPU.  --workload sphere: the 384-element dielectric sphere (single object).

  value        chosen form: double-float quadrature on the FP32 pipes, block
               elimination with complex-FP32 node inverses (butterfly-
               randomised LUs, tensor-core updates), FP64 refinement; inputs
               resident in HBM; CUDA events with a device-wide synchronise on
               both sides of each step (the step spans several streams)
  e2e          same step through the C ABI from host memory: device copies
               re-created from host arrays (H2D) and boundary values read back
               (D2H) every step
  fp64_form    the plain FP64 form (FP64 quadrature; FP64 block elimination
               for one-interface objects, else FP64 LU + explicit inverse)
               timed the same way, and the relative force/torque difference
  roofline     the tensor-core update kernel of the factorisation, timed per
               launch in a separate instrumented step (not inside the timed
               steps), against the measured bf16 peak and the TF32 rate
               cuBLAS reaches in the same run
  roofline_assembly
               the double-float assembly kernel (the step's largest): pairs
               per second from the same instrumented step, issue and FP32-pipe
               fractions from its committed per-pair instruction counts
  cpu_baseline the CPU oracle (oracle/port: C restatement of the quadrature,
               LAPACK for the dense LU/inverse) on this host's cores: a
               bounded sample scaled to one scene ("estimated": true)
With torchrun (N > 1) every rank solves its own copy of the scene (replicas;
the path has no exchange step): value = max-over-ranks time / scenes.
`--impl reference` times the CPU implementation of the path on the host cores
when it can finish a scene inside the run, else prints its `unavailable` line.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "assembly+LU+solve s per scene; chosen vs FP64 GPU at 1e-6 force/torque rel err"
SPHERE = dict(name="sphere r=1, cubed 8x8 quads/face (384 elements, na=12288), n=1.5 in 1.33, lambda0=1, "
                   "x-pol plane wave +z, single object",
              faces_n=8, radius=1.0, n_obj=1.5, n_host=1.33, lambda0=1.0)
CONES = dict(name="two cones (base radius 0.5, height 1, n = 1.59 in 1.33, lambda0 = 1), 12 m^2 linear triangles "
                  "each (m = 16: 3,072 triangles, na = 73,728 per cone, node jitter 5 % of the ring spacing, "
                  "seed 7); cone 2 rotated pi about x and shifted 1.5 along x; right-circularly polarised plane "
                  "wave along +z; multiple-scattering iteration to the reference's convergence rule",
             m=16, radius=0.5, height=1.0, n_obj=1.59, n_host=1.33, lambda0=1.0, seed=7)
VS_BASELINE_NOTE = "no published number for this metric: the reference publishes no benchmark"


def write_sphere(wd, n_face=8):
    from bem3_emf_b2_gb300 import meshgen
    nodes, elems = meshgen.cubed_sphere(n_face, SPHERE["radius"])
    meshgen.write_mesh(os.path.join(wd, "mesh.msh"), nodes, elems)
    meshgen.write_medium(os.path.join(wd, "medium.txt"), [SPHERE["n_obj"]])
    meshgen.write_ipw(os.path.join(wd, "ipw.txt"), [dict(lambda0=SPHERE["lambda0"], ni=SPHERE["n_host"], power=1.0,
                                                          e0x=1.0, e0y=0.0)])
    return len(elems)


def write_cones(wd, m=None):
    from bem3_emf_b2_gb300 import meshgen
    m = m or CONES["m"]
    nodes, elems = meshgen.cone_tri(m, CONES["radius"], CONES["height"], jitter=0.05, seed=CONES["seed"])
    meshgen.write_mesh(os.path.join(wd, "cone.msh"), nodes, elems)
    meshgen.write_medium(os.path.join(wd, "medium.txt"), [CONES["n_obj"]])
    meshgen.write_ipw(os.path.join(wd, "ipw.txt"), [dict(lambda0=CONES["lambda0"], ni=CONES["n_host"], power=1.0,
                                                          e0x=1.0, e0y=1j)])
    return len(elems)


CONE_RV = np.array([[1.0, 0.0, 0.0], [1.0, 0.0, 0.0]])
CONE_TH = np.array([0.0, np.pi])
CONE_TV = np.array([[0.0, 0.0, 0.0], [1.5, 0.0, 0.0]])


def write_sphere3(wd, nf):
    from bem3_emf_b2_gb300 import meshgen
    nodes, elems = meshgen.cubed_sphere(nf, SPHERE3["radius"])
    meshgen.write_mesh(os.path.join(wd, "mesh.msh"), nodes, elems)
    meshgen.write_medium(os.path.join(wd, "medium.txt"), [SPHERE3["n_obj"]])
    meshgen.write_ipw(os.path.join(wd, "ipw.txt"), [dict(lambda0=SPHERE3["lambda0"], ni=SPHERE3["n_host"], power=1.0,
                                                          e0x=1.0, e0y=0.0)])
    return len(elems)


def open_workload(args, wd):
    """(scene, description dict) of the chosen workload, set up from its input files"""
    from bem3_emf_b2_gb300 import MultiScene, Scene, meshgen
    if args.workload == "beams":
        objs = meshgen.batch_scene(BATCH["seed"], BATCH["n_obj"], box=BATCH["box"], elems=BATCH["elems"])
        med, msh = [], []
        for i, o in enumerate(objs):
            meshgen.write_mesh(os.path.join(wd, "o%d.msh" % i), o["nodes"], o["elems"])
            meshgen.write_medium(os.path.join(wd, "m%d.txt" % i), [o["n"]])
            med.append(os.path.join(wd, "m%d.txt" % i))
            msh.append(os.path.join(wd, "o%d.msh" % i))
        meshgen.write_ipw(os.path.join(wd, "beams.txt"), meshgen.random_waves(BATCH["seed"], BATCH["n_beam"]))
        sc = MultiScene(med, msh, os.path.join(wd, "beams.txt"))
        ne = [len(o["elems"]) for o in objs]
        return _Beams(sc, os.path.join(wd, "beams.txt")), dict(
            workload=BATCH["name"], objects=len(objs), elements_per_object=ne, beams=BATCH["n_beam"],
            na_per_object=[8 * (3 if o["kind"] == "cone" else 4) * len(o["elems"]) for o in objs])
    if args.workload == "cones":
        ne = write_cones(wd, args.cone_m)
        med = [os.path.join(wd, "medium.txt")] * 2
        msh = [os.path.join(wd, "cone.msh")] * 2
        sc = MultiScene(med, msh, os.path.join(wd, "ipw.txt"), rv=CONE_RV, th=CONE_TH, tv=CONE_TV)
        m = args.cone_m or CONES["m"]
        name = CONES["name"] if m == CONES["m"] else CONES["name"].replace("m = 16: 3,072", "m = %d: %d" % (m, ne))
        return sc, dict(workload=name, objects=2, elements_per_object=ne, na_per_object=8 * 3 * ne)
    if args.workload == "sphere3":
        nf = args.faces3
        ne = write_sphere3(wd, nf)
        sc = Scene(os.path.join(wd, "medium.txt"), os.path.join(wd, "mesh.msh"), os.path.join(wd, "ipw.txt"))
        return sc, dict(workload=SPHERE3["name"] % (nf, nf, ne), objects=1, elements_per_object=ne,
                        na_per_object=8 * 4 * ne)
    ne = write_sphere(wd, args.faces)
    sc = Scene(os.path.join(wd, "medium.txt"), os.path.join(wd, "mesh.msh"), os.path.join(wd, "ipw.txt"))
    name = SPHERE["name"] if args.faces == 8 else "sphere r=1, cubed %dx%d quads/face (%d elements)" % (
        args.faces, args.faces, ne)
    return sc, dict(workload=name, objects=1, elements_per_object=ne, na_per_object=8 * 4 * ne)


SPHERE3 = dict(name="sphere r=3, cubed %dx%d quads/face (%d elements), n = 1.5+0.01i in 1.33, lambda0 = 1, x-pol "
                    "plane wave +z: the 64x64-per-face sphere's geometry and media at a size whose FP64 form fits "
                    "one GPU", radius=3.0, n_obj=complex(1.5, 0.01), n_host=1.33, lambda0=1.0)

BATCH = dict(name="seeded multi-object scene (seed 11): 8 spheres, cubes and cones in a 20^3 box, characteristic size "
                  "U[0.3, 1.5], element counts U[200, 600], n U[1.33, 2.0] in 1.33, random orientation; 32 plane "
                  "waves of random direction and linear polarisation, each its own right-hand side",
             seed=11, n_obj=8, n_beam=32, box=20.0, elems=(200, 600))


class _Beams:
    """a multi-object scene whose step solves every beam (gbh_mscene_beams)"""

    def __init__(self, sc, beams_file):
        self.sc, self.beams_file = sc, beams_file

    def step(self, form=1):
        return self.sc.beams(self.beams_file, form=form)

    def __getattr__(self, k):
        return getattr(self.sc, k)


def force_vec(F, N):
    return np.concatenate([np.asarray(F, float).ravel(), np.asarray(N, float).ravel()])


# ---------------------------------------------------------------- distributed
def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return None, 0, 1
    import torch.distributed as dist
    backend = os.environ.get("BENCH_BACKEND", "nccl")
    dist.init_process_group(backend=backend)
    return dist, dist.get_rank(), dist.get_world_size()


def dist_barrier(dist):
    if dist is not None:
        dist.barrier()


def dist_max(dist, v):
    if dist is None:
        return v
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi samples (200 ms) during the timed region."""

    def __init__(self, gpu):
        self.gpu = gpu
        self.p = None
        self.out = tempfile.NamedTemporaryFile(prefix="clk", suffix=".csv", delete=False).name

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.out, "w")
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + q, "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p is not None:
            self.p.terminate()
            self.p.wait()
            self.f.close()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            for line in open(self.out):
                f = [x.strip() for x in line.split(",")]
                if len(f) < 9:
                    continue
                try:
                    sm.append(float(f[1]))
                    mx = float(f[2])
                except ValueError:
                    continue
                for n, v in zip(names, f[5:9]):
                    if v.lower() == "active":
                        reasons.add(n)
        except OSError:
            pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def flush_l2():
    import torch
    buf = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    buf.fill_(1.0)
    del buf


# ---------------------------------------------------------------- CPU baseline
def _lapack_rate(ns=3072):
    """seconds of LAPACK zgetrf + zgetri at order ns on this host"""
    from scipy.linalg import lapack
    rng = np.random.default_rng(0)
    A = rng.standard_normal((ns, ns)) + 1j * rng.standard_normal((ns, ns))
    t0 = time.perf_counter()
    lu, piv, info = lapack.zgetrf(A)
    lapack.zgetri(lu, piv)
    return time.perf_counter() - t0


def cpu_baseline(args, wd, iterations=11):
    """Oracle port on the host cores, a bounded sample scaled to one scene
    (an estimate, not a timing of a whole scene):
      assembly   sampled rows of every domain, scaled by rows;
      LU+inverse LAPACK zgetrf + zgetri at order 3,072, scaled by (na/3072)^3
                 (the reference inverts A densely, solve_bieq2.c:343-408);
      iteration  (multi-object scenes) sampled scattered-potential points of
                 add_scattered_mEMP (oracle field mode 3) scaled to every
                 exterior node of every object, times the GPU run's iteration
                 count, plus one invA b product (8 na^2 flop) per object and
                 iteration at the host's measured LAPACK rate."""
    from oracle import port
    ncpu = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(ncpu))
    if args.workload == "cones":
        objs = [port.Obj(os.path.join(wd, "cone.msh"), [CONES["n_obj"]], CONES["lambda0"], CONES["n_host"])]
        nobj = 2
    else:
        S = SPHERE3 if args.workload == "sphere3" else SPHERE
        objs = [port.Obj(os.path.join(wd, "mesh.msh"), [S["n_obj"]], S["lambda0"], S["n_host"])]
        nobj = 1
    o = objs[0]
    t_asm = 0.0
    sample_rows = max(4 * ncpu, 64)
    for d in range(o.MN + 1):
        N = 4 * (len(o.sids[d]) - 1)
        rows = np.linspace(0, N - 1, sample_rows).astype(np.int32)
        t0 = time.perf_counter()
        o.rows(d, rows)
        t_asm += (time.perf_counter() - t0) * N / len(rows)
    t_asm *= nobj
    na = 8 * o.NN
    ns = 3072
    t_ns = _lapack_rate(ns)
    t_lu = nobj * t_ns * (na / ns) ** 3
    t_it = 0.0
    if nobj > 1:
        # scattered potential of one object at sampled exterior nodes of the other
        ext = o.ren[1:, :3, :].reshape(-1, 3) + np.array([1.5, 0.0, 0.0])
        npts = max(2 * ncpu, 32)
        pts = ext[np.linspace(0, len(ext) - 1, npts).astype(int)]
        v = np.tile([0.0, 0.0, 1.0], (npts, 1))
        bv = [dict(U=np.zeros((len(o.sids[d]), 4, 4), complex), dU=np.zeros((len(o.sids[d]), 4, 4), complex),
                   E=np.zeros((len(o.sids[d]), 4, 3), complex), dE=np.zeros((len(o.sids[d]), 4, 3), complex),
                   H=np.zeros((len(o.sids[d]), 4, 3), complex), dH=np.zeros((len(o.sids[d]), 4, 3), complex))
              for d in range(o.MN + 1)]
        t0 = time.perf_counter()
        o.field(3, 2, pts, bv, v)
        t_pt = (time.perf_counter() - t0) / npts
        matvec = t_ns / (8.0 * ns ** 3) * 8.0 * na * na  # invA b at the LAPACK flop rate
        t_it = iterations * nobj * (t_pt * o.NN + matvec)
    total = t_asm + t_lu + t_it
    return dict(value=total, unit="s/scene", cores=ncpu, kind="port", estimated=True,
                sample="oracle port on %d cores: %d assembly rows per domain (scaled by rows), LAPACK zgetrf+zgetri at "
                       "n=%d scaled by (%d/%d)^3 per object%s; estimate %.1f s assembly + %.1f s LU/inverse + %.1f s "
                       "iteration (E/H stage and force not included)" % (
                           ncpu, sample_rows, ns, na, ns,
                           (", %d add_scattered points scaled to %d nodes x %d iterations" % (npts, o.NN, iterations))
                           if nobj > 1 else "", t_asm, t_lu, t_it))


# ---------------------------------------------------------------- GPU arm
def rel_vec(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300))


def timed_steps(sc, form, steps, warmup, dist=None):
    """warm-up steps, then `steps` steps each bracketed by a device-wide
    synchronise and CUDA events on the current stream (the step spans several
    streams and host threads); L2 flushed before each step"""
    import torch
    for _ in range(warmup):
        sc.step(form=form)
    st = torch.cuda.current_stream()
    times = []
    F = N = None
    torch.cuda.synchronize()
    dist_barrier(dist)
    for _ in range(steps):
        flush_l2()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(st)
        F, N = sc.step(form=form)
        torch.cuda.synchronize()
        e1.record(st)
        e1.synchronize()
        times.append(e0.elapsed_time(e1) / 1000.0)
    dist_barrier(dist)
    return times, F, N


def run_gpu(args):
    import torch
    dist, rank, ws = dist_init()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    from bem3_emf_b2_gb300 import build, ktime_list, ktime_read, lib
    build.build()
    L = lib()
    L.gb_set_tc_passes.argtypes = [ctypes.c_int]
    if L.gb_set_tc_passes(args.tc_passes) != 0:
        raise RuntimeError("gb_set_tc_passes(%d) refused" % args.tc_passes)
    wd = tempfile.mkdtemp(prefix="bench_")
    sc, desc = open_workload(args, wd)
    cones = args.workload in ("cones", "beams")
    # outer block of the node-matrix LUs and inverses, tuned on the
    # workload's node count before any timed step
    tune = None
    if args.workload in ("cones", "sphere", "sphere3") and not args.no_tune:
        nn = desc["na_per_object"] // 8
        best = ctypes.c_int(0)
        ms = (ctypes.c_double * 4)()
        L.gb_tune_lu_outer_block.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
        if L.gb_tune_lu_outer_block(nn, ctypes.byref(best), ms) != 0:
            raise RuntimeError("gb_tune_lu_outer_block failed")
        tune = {"lu_outer_block": best.value, "order": nn,
                "lu_plus_inverse_ms": dict(zip(("128", "256", "512", "1024"), [round(v, 3) for v in ms]))}

    # chosen form: warm-up, then exactly K timed steps (launch count over them)
    for _ in range(args.warmup):
        sc.step(form=1)
    l0 = L.gb_launch_count()
    with ClockSampler(local) as clk:
        t32, F32, N32 = timed_steps(sc, 1, args.steps, 0, dist)
    launches = (L.gb_launch_count() - l0) / args.steps
    tsum = sum(t32)
    tmax = dist_max(dist, tsum)
    value = tmax / (args.steps * ws)
    phases = sc.phase_times() if cones else None
    iters = sc.iteration() if cones else None
    # plain FP64 form (after the chosen form: its allocations are not in the line's steps)
    n64 = 1 if cones else max(1, min(args.steps, 2))
    if args.no_fp64:  # a comparison run of the chosen form alone
        t64, F64, N64 = [float("nan")], F32, N32
    else:
        t64, F64, N64 = timed_steps(sc, 0, n64, 0, dist)
    # e2e: device copies rebuilt from host memory every step (H2D), results read back (D2H)
    h2d, d2h = sc.h2d_bytes(), sc.d2h_bytes()
    te = []
    for _ in range(max(1, min(args.steps, 2 if cones else 3))):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sc.drop_device()
        sc.step(form=1)
        torch.cuda.synchronize()
        te.append(time.perf_counter() - t0)
    e2e = dist_max(dist, sum(te)) / (len(te) * ws)
    # far field of the solved scene on the 91 x 180 angular grid at r = 2000
    # lambda0 (reference example4.c:32-66) through the batched field map
    far = None
    if args.workload == "cones":
        th = np.linspace(0.0, np.pi, 91)
        ph = np.arange(180) * (2.0 * np.pi / 180)
        T, P = np.meshgrid(th, ph, indexing="ij")
        pts = 2000.0 * np.stack([np.sin(T) * np.cos(P), np.sin(T) * np.sin(P), np.cos(T)], -1).reshape(-1, 3)
        sc.field_map(pts[:64])
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        Ef, Hf, _ = sc.field_map(pts)
        far = {"points": len(pts), "s": time.perf_counter() - t0, "r": 2000.0,
               "form": "mo_EH_mEMP_s (scattered, potential-derivative formula), quadrature type 2",
               "max_abs_E": float(np.abs(Ef).max())}
    # instrumented step for the roofline (per-launch events), outside the timed steps
    L.gb_ktime_enable(1)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sc.step(form=1)
    torch.cuda.synchronize()
    t_instr = time.perf_counter() - t0
    kt = ktime_list()
    ktime_read()
    asm_t = (ctypes.c_double(), ctypes.c_double(), ctypes.c_long())
    if L.gb_ktime_asm(*[ctypes.byref(x) for x in asm_t]) != 0:
        asm_t = None
    L.gb_ktime_enable(0)
    force_err = rel_vec(force_vec(F32, N32), force_vec(F64, N64))
    out = None
    if rank == 0:
        roof = roofline_live(kt, t_instr, 1, tf32_peak())
        cpu = cpu_baseline(args, wd, iters[0] if iters else 11) if (ws == 1 and not args.no_cpu and
                                                                    args.workload != "beams") else None
        cfg = {"workload": desc["workload"], "objects": desc["objects"],
               "elements_per_object": desc["elements_per_object"], "na_per_object": desc["na_per_object"],
               "form": "chosen (double-float quadrature, FP32 block elimination (tensor-core passes: %d) + FP64 "
                       "GMRES refinement)" % args.tc_passes,
               "parallelism": "replicas x%d" % ws,
               "l2": "working set larger than L2 (coefficient matrices %s) and a 256 MB L2 flush before each step" % (
                   {"cones": "2 x 29 GB", "beams": "8 x 0.1-0.4 GB"}.get(args.workload, "0.45 GB")),
               "timing": "CUDA events on the current stream with a device-wide synchronise on both sides of each step"}
        out = {"metric": METRIC, "value": value, "unit": "s/scene", "n_gpus": ws, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": 1000.0 * tmax / args.steps, "higher_is_better": False,
               "scaling": "weak", "vs_baseline": None, "vs_baseline_note": VS_BASELINE_NOTE,
               "dtype": "double-float (f32 pairs) quadrature, c64 block LU + c128 refinement",
               "data": "synthetic (meshgen %s)" % {"cones": "cones, seed 7", "beams": "batch_scene seed 11, random_waves seed 11"}.get(
                   args.workload, "cubed sphere, seeded by construction"),
               "config": cfg,
               "fp64_form": None if args.no_fp64 else {
                   "s_per_scene": sum(t64) / len(t64), "steps": len(t64),
                   "force_torque_rel_diff_vs_chosen": force_err,
                   "form": "FP64 quadrature, FP64 block elimination (node LUs + inverses), FP64 E/H"},
               "force": np.asarray(F32).tolist(), "torque": np.asarray(N32).tolist(),
               "e2e": {"value": e2e, "unit": "s/scene", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
               "gpu_launches": int(round(launches)), "clocks": clk.summary()}
        if tune:
            out["autotune"] = tune
        if phases:
            out["phases_s_last_step"] = phases
        if far:
            out["far_field_91x180"] = far
        if iters:
            out["iterations"] = {"count": iters[0], "cc": iters[1]}
        if roof:
            out["roofline"] = roof
        roof_asm = roofline_assembly(asm_t, clk.summary()) if asm_t else None
        if roof_asm:
            out["roofline_assembly"] = roof_asm
        if cpu:
            out["cpu_baseline"] = {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample", "estimated")}
    sc.close()
    if dist is not None:
        dist.destroy_process_group()
    return out


TRAFFIC_FILE = os.path.join(ROOT, "profiles", "tc_cgemm_traffic.json")


def gb_tc_passes():
    """tensor-core passes of the library's FP32 factorisations"""
    from bem3_emf_b2_gb300 import lib
    return int(lib().gb_get_tc_passes())


def tf32_peak(n=8192, reps=10):
    """Dense TF32 GEMM rate of this GPU through cuBLAS (torch matmul of two
    n x n FP32 matrices with TF32 allowed; CUDA events, after warm-up): the
    ceiling of the single-pass TF32 tensor-core kernel, measured in the run
    instead of taken from a data-sheet ratio.  TFLOP/s (2 n^3 per product)."""
    import torch
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = True
    try:
        g = torch.Generator(device="cuda").manual_seed(5)
        a = torch.randn(n, n, device="cuda", generator=g)
        b = torch.randn(n, n, device="cuda", generator=g)
        c = torch.empty(n, n, device="cuda")
        for _ in range(3):
            torch.matmul(a, b, out=c)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(reps):
            torch.matmul(a, b, out=c)
        e1.record()
        torch.cuda.synchronize()
        t = e0.elapsed_time(e1) / 1000.0 / reps
        del a, b, c
        return 2.0 * n ** 3 / t / 1e12
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev


def roofline_live(klist, step_seconds, steps, tf32=None):
    """Roofline of the factorisation's tensor-core update kernel
    k_tc_cgemm_sub (tcgen05 kind::tf32; one pass by default, three split
    passes for FP32-accurate products) from CUDA events around each of its
    launches on the library's streams in one instrumented step.  Per launch
    M x N x K (complex): algorithmic flops 8 M N K (complex-equivalent),
    algorithmic HBM bytes 16 M N (C read and written) + the split operands
    4 (M + 2N) Kp per plane (two planes for three passes, one for one).
    Two classes: launches with K >= 128 (outer-block updates and the block
    elimination's products: >= 64 complex flop per byte, tensor-bound) and
    the inner-panel updates (K <= 64, HBM-bound).  `traffic` scales the
    measured DRAM bytes per algorithmic byte of one ncu capture
    (profiles/tc_cgemm_traffic.json, taken on the three-pass kernel) to
    these launches.
    The tensor figures are against the measured dense bf16 peak and, beside
    it, the TF32 rate cuBLAS reaches on the same GPU in the same run (tf32)."""
    if not klist:
        return None
    peaks = {}
    pf = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pf):
        peaks = json.load(open(pf))
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    bf16 = float(peaks.get("bf16_tflops", 1900.0))
    src = "MEASURED_PEAKS.json (measured)" if "hbm_gbs" in peaks else "fallback 6.8 TB/s, 1.9 PFLOP/s"
    ceil3 = bf16 * 1.1 / 2.25 / 3.0
    tr = json.load(open(TRAFFIC_FILE)) if os.path.exists(TRAFFIC_FILE) else {}
    cls = {"outer": [0, 0.0, 0.0, 0.0], "inner": [0, 0.0, 0.0, 0.0]}
    planes = 2.0 if gb_tc_passes() == 3 else 1.0  # split operand planes read (hi, lo) or (hi)
    for ms, M, N, K in klist:
        Kp = ((2 * int(K) + 31) // 32) * 32
        c = cls["outer" if K >= 128 else "inner"]
        c[0] += 1
        c[1] += ms
        c[2] += 8.0 * M * N * K
        c[3] += 16.0 * M * N + planes * 4.0 * (M + 2.0 * N) * Kp
    out = None
    o = cls["outer"]
    if o[0]:
        dt = o[1] / 1000.0
        ach = o[2] / dt / 1e12
        ratio = tr.get("outer", {}).get("dram_bytes_per_algorithmic_byte")
        out = {"kernel": "k_tc_cgemm_sub (tcgen05 TF32 complex update, passes %d), launches with K >= 128" % gb_tc_passes(),
               "bound": "tensor", "achieved": ach, "peak": bf16, "unit": "TFLOP/s", "frac": ach / bf16,
               "peak_source": src + " bf16_tflops",
               "traffic": ratio * o[3] / o[0] if ratio else None,
               "algorithmic_bytes_per_launch": o[3] / o[0], "algorithmic_flops_per_launch": o[2] / o[0],
               "tf32x3_ceiling_tflops": ceil3, "frac_of_tf32x3_ceiling": ach / ceil3,
               "tf32_cublas_tflops_measured": tf32, "frac_of_tf32_measured": ach / tf32 if tf32 else None,
               "launches_per_step": o[0] / steps, "kernel_ms_total": o[1],
               "kernel_share_of_timed_steps": dt / step_seconds}
    i = cls["inner"]
    if i[0]:
        dt = i[1] / 1000.0
        ach = i[3] / dt / 1e9
        ratio = tr.get("inner", {}).get("dram_bytes_per_algorithmic_byte")
        inner = {"kernel": "k_tc_cgemm_sub, inner-panel launches (K <= 64)", "bound": "hbm", "achieved": ach,
                 "peak": hbm, "unit": "GB/s", "frac": ach / hbm, "peak_source": src + " hbm_gbs",
                 "traffic": ratio * i[3] / i[0] if ratio else None, "launches_per_step": i[0] / steps,
                 "kernel_ms_total": i[1], "kernel_share_of_timed_steps": dt / step_seconds}
        if out is None:
            out = inner
        else:
            out["inner_launches"] = inner
    return out


ASM_ISSUE_FILE = os.path.join(ROOT, "profiles", "asm_regular_df_issue.json")


def roofline_assembly(rec, clocks):
    """Issue-rate roofline of the double-float regular assembly
    (k_asm_regular_df_list), the step's largest kernel: bound by the SM
    sub-partitions' instruction issue (one warp instruction per clock each,
    4 per SM) and within that by the FP32 pipe.  Live: device time and pairs
    of its launches in the instrumented step (CUDA events on its stream).
    Instructions per pair: an ncu count of the same launch on the same
    workload (profiles/asm_regular_df_issue.json).  Peaks at the median SM
    clock sampled during the timed steps."""
    import torch
    ms, pairs, n = rec[0].value, rec[1].value, rec[2].value
    if n <= 0 or ms <= 0.0:
        return None
    rate = pairs / (ms / 1000.0)
    out = {"kernel": "k_asm_regular_df_list (double-float regular pairs, all (object, domain) items)",
           "bound": "fp32-issue", "launches_per_step": n, "kernel_ms_total": ms, "pairs_per_launch": pairs / n,
           "pairs_per_s": rate}
    iss = json.load(open(ASM_ISSUE_FILE)) if os.path.exists(ASM_ISSUE_FILE) else None
    mhz = (clocks or {}).get("sm_mhz") or (clocks or {}).get("sm_max_mhz") or 2070.0
    nsm = torch.cuda.get_device_properties(0).multi_processor_count if torch.cuda.is_available() else 152
    if iss:
        slots = nsm * 4 * float(mhz) * 1e6  # warp instructions per second, all sub-partitions
        ach = iss["inst_per_pair"] * rate
        fma = iss["fma_pipe_inst_per_pair"] * rate
        out.update({"achieved": fma / 1e9, "peak": slots / 1e9, "unit": "G warp-inst/s (FP32 pipe)",
                    "frac": fma / slots, "issue_achieved": ach / 1e9, "issue_frac": ach / slots,
                    "peak_source": "%d SMs x 4 sub-partitions x 1 warp instruction per clock at %.0f MHz" % (nsm, mhz),
                    "inst_counts": "ncu smsp__inst_executed.sum and smsp__inst_executed_pipe_fma.sum per pair, %s" %
                                   iss.get("source", "")})
    return out


# ---------------------------------------------------------------- reference arm
def run_reference(args):
    """The reference's CPU path on this host.  Its dense inverse of each
    object's coupled matrix (zgetrf + zgetri of na = 8 NN, solve_bieq2.c:343-408)
    is what bounds a CPU scene: for the two-cone scene that is two inverses of
    order 73,728 (87 GB of complex128 each, ~3.2e15 flop each), hours on the
    host's cores -- it cannot finish inside this run, so the arm prints its
    `unavailable` line with the sampled estimate of cpu_baseline beside it."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return None
    if args.workload in ("beams", "cube"):
        return {"impl": "reference", "unavailable": "the CPU restatement of the path has no multi-object iteration "
                "or row-block assembly timing for this workload"}
    wd = tempfile.mkdtemp(prefix="bench_ref_")
    if args.workload == "cones":
        write_cones(wd, args.cone_m)
    elif args.workload == "sphere3":
        write_sphere3(wd, args.faces3)
    else:
        write_sphere(wd, args.faces)
    cpu = cpu_baseline(args, wd)
    reason = ("the reference CPU path inverts each object's coupled matrix densely (zgetrf+zgetri, "
              "solve_bieq2.c:343-408); for this workload that is %s and cannot finish a scene inside this run; "
              "sampled estimate %.0f s/scene on %d cores" % (
                  "2 x order 73,728 (87 GB c128 each, ~3.2e15 flop each)" if args.workload == "cones"
                  else "order %d plus the E/H stage and force that the CPU restatement does not cover" % (
                      8 * 4 * 6 * (args.faces3 if args.workload == "sphere3" else args.faces) ** 2),
                  cpu["value"], cpu["cores"]))
    return {"impl": "reference", "unavailable": reason,
            "cpu_baseline": {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample", "estimated")}}


CUBE = dict(name="cube of side 6 (lambda0 = 1), 80 x 80 planar quadrangles per face (38,400 elements, N = 153,600 "
                 "rows per domain), n = 1.6 in 1.33; coefficient-matrix assembly of both domains streamed in row "
                 "blocks (gb_assemble_rows), the 377 GB per-domain matrices never stored",
            n=80, side=6.0, n_obj=1.6, n_host=1.33, lambda0=1.0)


def run_cube(args):
    """Assembly throughput of the 38,400-element cube (pairs of a collocation
    node and a source element per second): each step assembles one block of
    --rows rows of G, H, dG, dH, dF (blocks spread over both domains) in the
    chosen form's precision; the FP64 form's rate is measured the same way
    on two blocks."""
    import torch
    from bem3_emf_b2_gb300 import Scene, build, lib, meshgen
    import ctypes
    build.build()
    L = lib()
    vp, ci = ctypes.c_void_p, ctypes.c_int
    L.gb_assemble_rows.argtypes = [vp, ci, ci, ci, ci, ci, vp, vp, vp, vp, vp]
    L.gb_assemble_rows.restype = ci
    L.gb_obj_stream.argtypes = [vp]
    L.gb_obj_stream.restype = vp
    wd = tempfile.mkdtemp(prefix="cube_")
    n = args.cube_n or CUBE["n"]
    nodes, elems = meshgen.cube(n, CUBE["side"])
    meshgen.write_mesh(os.path.join(wd, "mesh.msh"), nodes, elems)
    meshgen.write_medium(os.path.join(wd, "medium.txt"), [CUBE["n_obj"]])
    meshgen.write_ipw(os.path.join(wd, "ipw.txt"), [dict(lambda0=1.0, ni=CUBE["n_host"], power=1.0, e0x=1.0, e0y=0.0)])
    sc = Scene(os.path.join(wd, "medium.txt"), os.path.join(wd, "mesh.msh"), os.path.join(wd, "ipw.txt"))
    o = sc.obj()
    ne = len(elems)
    N = 4 * ne
    B = min(args.rows, N)
    G = torch.empty((B, N), dtype=torch.complex128, device="cuda")
    H = torch.empty_like(G)
    dG = torch.empty((2 * B, N), dtype=torch.complex128, device="cuda")
    dH = torch.empty_like(dG)
    dF = torch.empty((B, 3), dtype=torch.float64, device="cuda")
    st = torch.cuda.ExternalStream(L.gb_obj_stream(o))
    nblk = N // B

    def block(i, prec):
        d = i % 2
        r0 = ((i // 2) * 7919 % max(nblk, 1)) * B  # blocks spread over the domain
        if L.gb_assemble_rows(o, d, r0, B, 2, prec, G.data_ptr(), H.data_ptr(), dG.data_ptr(), dH.data_ptr(),
                              dF.data_ptr()) != 0:
            raise RuntimeError(L.gb_last_error().decode())

    def timed(prec, steps, warmup):
        for i in range(warmup):
            block(i, prec)
        st.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for i in range(steps):
            block(warmup + i, prec)
        e1.record(st)
        e1.synchronize()
        return e0.elapsed_time(e1) / 1000.0
    l0 = L.gb_launch_count()
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        t = timed(3, args.steps, args.warmup)
    launches = (L.gb_launch_count() - l0) / (args.steps + args.warmup)
    t64 = timed(0, 2, 0)
    pairs = float(B) * ne
    sc.close()
    rate = pairs * args.steps / t
    return {"metric": "assembly pairs/s (collocation node x source element), 38,400-element cube",
            "value": rate, "unit": "pairs/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * t / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "vs_baseline_note": VS_BASELINE_NOTE,
            "dtype": "double-float quadrature, adaptive order (precision 3)", "data": "synthetic (meshgen cube)",
            "config": {"workload": CUBE["name"] if n == CUBE["n"] else "cube %d x %d per face" % (n, n),
                       "elements": ne, "rows_per_step": B, "pairs_per_step": pairs,
                       "full_assembly_s_estimate": 2.0 * N * ne / rate},
            "fp64_form": {"pairs_per_s": pairs * 2 / t64},
            "gpu_launches": int(round(launches)), "clocks": clk.summary()}


def profile_step(args):
    """Warm-up steps then exactly one chosen-form step (for ncu launch lists)."""
    import torch
    from bem3_emf_b2_gb300 import build
    build.build()
    wd = tempfile.mkdtemp(prefix="prof_")
    sc, desc = open_workload(args, wd)
    for _ in range(args.warmup):
        sc.step(form=1)
    torch.cuda.synchronize()
    F, N = sc.step(form=1)
    torch.cuda.synchronize()
    print("profile step done: %s force=%s" % (desc["workload"][:40], np.asarray(F).ravel()))
    sc.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb", choices=["gb", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline sample")
    ap.add_argument("--profile-step", action="store_true",
                    help="profiling run: one chosen-form scene step after --warmup steps, nothing else, no JSON line")
    ap.add_argument("--faces3", type=int, default=24, help="quadrangles per cube face of the sphere3 workload")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 form (comparison runs of the chosen form)")
    ap.add_argument("--no-tune", action="store_true", help="keep the default LU outer block (no tuning run)")
    ap.add_argument("--tc-passes", type=int, default=1, choices=[1, 3],
                    help="tensor-core passes of the FP32 factorisations (gb_set_tc_passes)")
    ap.add_argument("--workload", choices=["cones", "sphere", "sphere3", "cube", "beams"], default="cones",
                    help="cones: the two-cone scene (default); sphere: the 384-element sphere; cube: assembly "
                         "throughput of the 38,400-element cube")
    ap.add_argument("--cube-n", type=int, default=None, help="quadrangles per cube edge (cube workload)")
    ap.add_argument("--rows", type=int, default=1024, help="rows per step of the cube workload")
    ap.add_argument("--faces", type=int, default=8, help="quadrangles per cube face of the sphere workload")
    ap.add_argument("--cone-m", type=int, default=None, help="rings per cone surface (12 m^2 triangles per cone)")
    args = ap.parse_args()
    if args.profile_step:
        profile_step(args)
        return
    if args.workload == "cube" and args.impl != "reference":
        out = run_cube(args)
    else:
        out = run_reference(args) if args.impl == "reference" else run_gpu(args)
    if out is not None:
        print(json.dumps(out))


if __name__ == "__main__":
    main()
