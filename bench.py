"""Benchmark of the GB300 BEM hot path: seconds per scene.

One step = one scene solved on the GPU: coefficient-matrix assembly of both
domains (GLN x GLN quadrature, GHN fallback, singular self terms), the coupled
matrix A and its factorisation, the boundary values (potentials, E, H and
normal derivatives), and the radiation force and torque.  Workload: dielectric
sphere of radius 1 (lengths in vacuum wavelengths), n = 1.5 in n = 1.33,
cubed sphere with 8 x 8 bilinear quadrangles per face (384 elements,
na = 12,288 unknowns), x-polarised plane wave along +z.

  value        chosen form (double-float quadrature on the FP32 pipes; A
               randomised by recursive butterflies, complex-FP32 LU without
               interchanges with tensor-core trailing updates, FP64
               iterative refinement to a relative residual of 1e-13), inputs
               resident in HBM, CUDA events on the library's stream
  e2e          same step through the C ABI from host memory: device copy
               re-created from host arrays (H2D) and boundary values read back
               (D2H) every step
  fp64_form    the plain FP64 form (FP64 quadrature, FP64 LU + explicit
               inverse, as the reference) timed the same way, and the
               relative force/torque difference between the two forms
  roofline     the tensor-core trailing update of the LU, timed live per
               launch: its outer-block launches (tensor-bound) and, nested,
               its inner-panel launches (HBM-bound)
  cpu_baseline the CPU oracle (oracle/port: C restatement of the quadrature,
               LAPACK for the LU) on this host, on a bounded sample scaled to
               one scene
With torchrun (N > 1) every rank solves its own copy of the scene (replicas;
the path has no exchange step): value = max-over-ranks time / scenes.
`--impl reference` times the CPU implementation of the path (oracle port) on
the host cores and prints the same line with "impl": "reference".
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "assembly+LU+solve s per scene; chosen vs FP64 GPU at 1e-6 force/torque rel err"
WORKLOAD = dict(name="sphere r=1, cubed 8x8 quads/face (384 elements, na=12288), n=1.5 in 1.33, lambda0=1, "
                     "x-pol plane wave +z, single object",
                faces_n=8, radius=1.0, n_obj=1.5, n_host=1.33, lambda0=1.0)


def write_scene(wd, n_face=8):
    from bem3_emf_b2_gb300 import meshgen
    nodes, elems = meshgen.cubed_sphere(n_face, WORKLOAD["radius"])
    meshgen.write_mesh(os.path.join(wd, "mesh.msh"), nodes, elems)
    meshgen.write_medium(os.path.join(wd, "medium.txt"), [WORKLOAD["n_obj"]])
    meshgen.write_ipw(os.path.join(wd, "ipw.txt"), [dict(lambda0=WORKLOAD["lambda0"], ni=WORKLOAD["n_host"], power=1.0,
                                                          e0x=1.0, e0y=0.0)])


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
def cpu_baseline(wd, seconds_budget=20.0):
    """Oracle port on the host cores: a sample of assembly rows of both
    domains and a LAPACK zgetrf+zgetri at a reduced order, scaled to one
    scene (rows x N, and (na / n_sample)^3)."""
    from oracle import port
    ncpu = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(ncpu))
    o = port.Obj(os.path.join(wd, "mesh.msh"), [WORKLOAD["n_obj"]], WORKLOAD["lambda0"], WORKLOAD["n_host"])
    t_asm = 0.0
    nrows_total = 0
    sample_rows = max(8 * ncpu, 128)
    for d in range(o.MN + 1):
        N = 4 * (len(o.sids[d]) - 1)
        rows = np.linspace(0, N - 1, sample_rows).astype(np.int32)
        t0 = time.perf_counter()
        o.rows(d, rows)
        t_asm += (time.perf_counter() - t0) * N / len(rows)
        nrows_total += N
    from scipy.linalg import lapack
    na = 8 * o.NN
    ns = 3072
    A = (np.random.default_rng(0).standard_normal((ns, ns)) + 1j * np.random.default_rng(1).standard_normal((ns, ns)))
    t0 = time.perf_counter()
    lu, piv, info = lapack.zgetrf(A)
    inv, info = lapack.zgetri(lu, piv)
    t_lu = (time.perf_counter() - t0) * (na / ns) ** 3
    total = t_asm + t_lu
    return dict(value=total, unit="s/scene", cores=ncpu, kind="port",
                sample="assembly: %d rows per domain of %d (scaled by N/rows), LU+inverse: LAPACK zgetrf+zgetri at "
                       "n=%d scaled by (%d/%d)^3; estimate %.1f s assembly + %.1f s LU" % (
                           sample_rows, nrows_total // (o.MN + 1), ns, na, ns, t_asm, t_lu),
                assembly_s=t_asm, lu_s=t_lu)


# ---------------------------------------------------------------- GPU arm
def rel_vec(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300))


def run_gpu(args):
    import torch
    dist, rank, ws = dist_init()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    from bem3_emf_b2_gb300 import Scene, build, lib, ktime_list, ktime_read
    build.build()
    wd = tempfile.mkdtemp(prefix="bench_")
    write_scene(wd)
    sc = Scene(os.path.join(wd, "medium.txt"), os.path.join(wd, "mesh.msh"), os.path.join(wd, "ipw.txt"))
    L = lib()

    def timed(form, steps, warmup, ktime=False):
        for _ in range(warmup):
            sc.step(form=form)
        st = torch.cuda.ExternalStream(sc.stream())
        times = []
        F = N = None
        torch.cuda.synchronize()
        dist_barrier(dist)
        l0 = L.gb_launch_count()
        if ktime:
            L.gb_ktime_enable(1)
        for _ in range(steps):
            flush_l2()
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(st)
            F, N = sc.step(form=form)
            e1.record(st)
            e1.synchronize()
            times.append(e0.elapsed_time(e1) / 1000.0)
        torch.cuda.synchronize()
        launches = (L.gb_launch_count() - l0) / steps
        kt = None
        if ktime:
            kt = ktime_list()
            ktime_read()
            L.gb_ktime_enable(0)
        dist_barrier(dist)
        return times, F, N, launches, kt

    # plain FP64 form (reference-equivalent), then the chosen form
    t64, F64, N64, _, _ = timed(0, max(1, min(args.steps, 2)), 1)
    with ClockSampler(local) as clk:
        t32, F32, N32, launches, kt = timed(1, args.steps, args.warmup, ktime=True)
    tsum = sum(t32)
    tmax = dist_max(dist, tsum)
    value = tmax / (args.steps * ws)
    # e2e: device copy rebuilt from host memory every step (H2D), results read back (D2H)
    h2d, d2h = sc.h2d_bytes(), sc.d2h_bytes()
    te = []
    for _ in range(max(1, min(args.steps, 3))):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sc.drop_device()
        sc.step(form=1)
        torch.cuda.synchronize()
        te.append(time.perf_counter() - t0)
    e2e = dist_max(dist, sum(te)) / (len(te) * ws)
    # relative difference of the combined force/torque vector (a component that
    # vanishes by symmetry is rounding noise and is not a meaningful ratio)
    force_err = rel_vec(np.concatenate([F32, N32]), np.concatenate([F64, N64]))
    out = None
    if rank == 0:
        roof = roofline_live(kt, tsum, args.steps)
        cpu = cpu_baseline(wd) if (ws == 1 and not args.no_cpu) else None
        out = {"metric": METRIC, "value": value, "unit": "s/scene", "n_gpus": ws, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": 1000.0 * tmax / args.steps, "higher_is_better": False,
               "scaling": "weak", "vs_baseline": None, "dtype": "double-float (f32 pairs) quadrature, c64 LU + c128 refinement",
               "data": "synthetic (meshgen cubed sphere, seeded by construction)",
               "config": {"workload": WORKLOAD["name"], "elements": 384, "na": 12288, "form": "mixed",
                          "parallelism": "replicas x%d" % ws,
                          "l2": "working set larger than L2 (A: 2.4 GB FP64) and a 256 MB L2 flush before each step"},
               "fp64_form": {"s_per_scene": sum(t64) / len(t64), "force_torque_rel_diff_vs_chosen": force_err},
               "force": list(map(float, F32)), "torque": list(map(float, N32)),
               "e2e": {"value": e2e, "unit": "s/scene", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
               "gpu_launches": int(round(launches)), "clocks": clk.summary()}
        if roof:
            out["roofline"] = roof
        if cpu:
            out["cpu_baseline"] = {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")}
    sc.close()
    if dist is not None:
        dist.destroy_process_group()
    return out


TRAFFIC_FILE = os.path.join(ROOT, "profiles", "tc_cgemm_traffic.json")


def roofline_live(klist, step_seconds, steps):
    """Roofline of the dominant kernel of the complex-FP32 LU -- the tensor-core
    trailing update k_tc_cgemm_sub (tcgen05, TF32 in three passes for FP32
    accuracy) -- from CUDA events around each of its launches on the library's
    stream inside the timed steps.  Per launch M x N x K (complex):
    algorithmic flops 8 M N K (complex-equivalent), algorithmic HBM bytes
    16 M N (C read and written) + the split operands 2 x 4 (M + 2N) Kp.
    Two classes: the outer-block updates (K = 256: 128 complex flop per byte,
    above the ridge, tensor-bound) and the inner-panel updates (K <= 64,
    HBM-bound).  The tensor figures are against the measured dense bf16 peak;
    tcgen05 kind::tf32 issues at 1.1/2.25 of the kind::f16 rate and the FP32-
    accurate split needs three passes, so the ceiling this arithmetic can reach
    is bf16 x (1.1 / 2.25) / 3, reported beside it."""
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
    for ms, M, N, K in klist:
        Kp = ((2 * int(K) + 31) // 32) * 32
        c = cls["outer" if K >= 128 else "inner"]
        c[0] += 1
        c[1] += ms
        c[2] += 8.0 * M * N * K
        c[3] += 16.0 * M * N + 8.0 * (M + 2.0 * N) * Kp
    out = None
    o = cls["outer"]
    if o[0]:
        dt = o[1] / 1000.0
        ach = o[2] / dt / 1e12
        ratio = tr.get("outer", {}).get("dram_bytes_per_algorithmic_byte")
        out = {"kernel": "k_tc_cgemm_sub (tcgen05 TF32 x3 complex trailing update), outer-block launches (K = 256)",
               "bound": "tensor", "achieved": ach, "peak": bf16, "unit": "TFLOP/s", "frac": ach / bf16,
               "peak_source": src + " bf16_tflops",
               "traffic": ratio * o[3] / o[0] if ratio else None,
               "algorithmic_bytes_per_launch": o[3] / o[0], "algorithmic_flops_per_launch": o[2] / o[0],
               "tf32x3_ceiling_tflops": ceil3, "frac_of_tf32x3_ceiling": ach / ceil3,
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


# ---------------------------------------------------------------- reference arm
def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return None
    wd = tempfile.mkdtemp(prefix="bench_ref_")
    write_scene(wd)
    vals = []
    cpu = None
    for _ in range(max(1, args.steps)):
        cpu = cpu_baseline(wd)
        vals.append(cpu["value"])
    v = statistics.median(vals)
    return {"metric": METRIC, "value": v, "unit": "s/scene", "n_gpus": int(os.environ.get("WORLD_SIZE", "1")),
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * v, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64 (complex128)", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": WORKLOAD["name"], "elements": 384, "na": 12288, "form": "CPU oracle port"},
            "cpu_baseline": {"value": v, "unit": "s/scene", "cores": cpu["cores"], "kind": cpu["kind"],
                             "sample": cpu["sample"]},
            "e2e": {"value": v, "unit": "s/scene", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


CONES = dict(name="two cones (base radius 0.5, height 1, n = 1.59 in 1.33, lambda0 = 1), 12 m^2 linear triangles "
                   "each (m = 16: 3,072 triangles, na = 73,728 per cone, node jitter 5 % of the ring spacing, "
                   "seed 7); cone 2 rotated pi about x and shifted 1.5 along x; right-circularly polarised plane "
                   "wave along +z; multiple-scattering iteration to the reference's convergence rule",
             m=16, radius=0.5, height=1.0, n_obj=1.59, n_host=1.33, lambda0=1.0, seed=7)


def write_cones(wd, m=None):
    from bem3_emf_b2_gb300 import meshgen
    m = m or CONES["m"]
    nodes, elems = meshgen.cone_tri(m, CONES["radius"], CONES["height"], jitter=0.05, seed=CONES["seed"])
    meshgen.write_mesh(os.path.join(wd, "cone.msh"), nodes, elems)
    meshgen.write_medium(os.path.join(wd, "medium.txt"), [CONES["n_obj"]])
    meshgen.write_ipw(os.path.join(wd, "ipw.txt"), [dict(lambda0=CONES["lambda0"], ni=CONES["n_host"], power=1.0,
                                                          e0x=1.0, e0y=1j)])
    return len(elems)


def run_cones(args):
    """The two-cone scene in the chosen form (one GPU): seconds per scene and
    force/torque on each cone.  Its plain FP64 form (an FP64 LU and inverse of
    na = 73,728 per cone, ~3e15 flop each) is not timed here."""
    import torch
    from bem3_emf_b2_gb300 import MultiScene, build, lib
    build.build()
    L = lib()
    wd = tempfile.mkdtemp(prefix="cones_")
    ne = write_cones(wd, args.cone_m)
    med = [os.path.join(wd, "medium.txt")] * 2
    msh = [os.path.join(wd, "cone.msh")] * 2
    rv = np.array([[1.0, 0.0, 0.0], [1.0, 0.0, 0.0]])
    th = np.array([0.0, np.pi])
    tv = np.array([[0.0, 0.0, 0.0], [1.5, 0.0, 0.0]])
    sc = MultiScene(med, msh, os.path.join(wd, "ipw.txt"), rv=rv, th=th, tv=tv)
    times = []
    F = N = None
    l0 = L.gb_launch_count()
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        F, N = sc.step(form=1)
        torch.cuda.synchronize()
        if i >= args.warmup:
            times.append(time.perf_counter() - t0)
    it, cc = sc.iteration()
    phases = sc.phase_times()
    launches = (L.gb_launch_count() - l0) / (args.warmup + args.steps)
    sc.close()
    v = sum(times) / len(times)
    return {"metric": METRIC, "value": v, "unit": "s/scene", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * v, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "double-float (f32 pairs) quadrature, c64 LU + c128 refinement", "data": "synthetic (meshgen cones, seed 7)",
            "config": {"workload": CONES["name"], "elements_per_cone": ne, "form": "mixed",
                       "timing": "host wall clock around each scene step (synchronised)"},
            "iterations": it, "cc": cc, "phases_s": phases, "force": F.tolist(), "torque": N.tolist(),
            "gpu_launches": int(round(launches))}


def profile_step(args):
    """Warm-up steps then exactly one chosen-form step (for ncu launch lists)."""
    import torch
    from bem3_emf_b2_gb300 import Scene, build
    build.build()
    wd = tempfile.mkdtemp(prefix="prof_")
    write_scene(wd, args.faces)
    sc = Scene(os.path.join(wd, "medium.txt"), os.path.join(wd, "mesh.msh"), os.path.join(wd, "ipw.txt"))
    for _ in range(args.warmup):
        sc.step(form=1)
    torch.cuda.synchronize()
    F, N = sc.step(form=1)
    torch.cuda.synchronize()
    print("profile step done: faces=%d force=%s" % (args.faces, F))
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
    ap.add_argument("--faces", type=int, default=8, help="quadrangles per cube face of the profiling scene")
    ap.add_argument("--workload", choices=["sphere", "cones"], default="sphere",
                    help="sphere: the bench line (both forms); cones: the two-cone scene, chosen form only")
    ap.add_argument("--cone-m", type=int, default=None, help="rings per cone surface (12 m^2 triangles per cone)")
    args = ap.parse_args()
    if args.profile_step:
        profile_step(args)
        return
    if args.workload == "cones":
        out = run_cones(args)
    else:
        out = run_reference(args) if args.impl == "reference" else run_gpu(args)
    if out is not None:
        print(json.dumps(out))


if __name__ == "__main__":
    main()
