"""Benchmark of the explicit MPM step (USL, linear hat basis) on one GB300.

Workload (default): the 3D Taylor bar -- J2 plasticity with linear hardening,
E=117e9, nu=0.35, rho=8930, sigma_y=400e6, H=100e6, cylinder r=3.2 mm,
L=32.4 mm, 2x2x2 particles per cell at h=0.25 mm (511,784 particles) on a
65x65x161-node grid, -190 m/s against the z=0 wall, dt = 0.2 h/c.
One bench step = one full USL step (P2G, grid update, G2P + F + J2) of all
particles.  Inputs are synthetic (generated from the geometry).  The
particle state (~160 MB) and grid (~70 MB) exceed the 129 MB L2, so no L2
flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--precision f64|f32|dw]
  python bench.py --impl reference ...   # the CPU restatement on the host cores

The default FP64 line also carries "double_word": the MPM_PREC_DW variant of
the same step (FP64 fields and node sums, P2G and G2P arithmetic in
double-word FP32) timed the same way, with its roofline and its largest
relative difference per field from the FP64 run at the same step.

Prints one JSON line on rank 0.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# one process per GPU: pin this rank to its GPU before any CUDA runtime starts
if "LOCAL_RANK" in os.environ and int(os.environ.get("WORLD_SIZE", "1")) > 1:
    os.environ["CUDA_VISIBLE_DEVICES"] = os.environ["LOCAL_RANK"]

import numpy as np  # noqa: E402

METRIC = "particle-updates/s"
# Algorithmic bytes per particle per launch, FP64, 3D J2 (each persistent field
# read once and each updated field written once; symmetric tensors counted as 6):
#   P2G  reads x3 v3 m V sigma6                      = 14 doubles -> 112 B
#   G2P  reads x3 v3 V0 F9 eps6 alpha ep6            = 29 doubles
#        writes x3 v3 V F9 eps6 sigma6 alpha ep6 vm  = 36 doubles -> 520 B
# plus the grid share (8 particles per active node): P2G 7 doubles/node, G2P 6
# doubles/node gathered, grid update 13 doubles/node -> 600 B per particle-update.
# These are the algorithmic bytes: what the step must move.  The FP64 step also
# keeps a hat cache (per axis a cell code, int32, and the lower hat value, double;
# P2G writes 36 B per particle, the G2P of the same step reads them back): that is
# this implementation's own traffic, counted in the measured DRAM bytes
# ("traffic") but not in "achieved".
HAT = 36
BYTES = {
    "f64": {"p2g": 112 + 7, "g2p": 520 + 6, "step": 600},
    "f32": {"p2g": 56 + 7, "g2p": 260 + 3, "step": 330},
}
# the double-word variant keeps the FP64 fields and nodes: the same bytes
BYTES["dw"] = BYTES["f64"]
# MUSL, FP64, 3D J2: P2G as above; the G2P stage is G2P-1 (reads x3 v3 m, writes v3
# = 80 B, + P2G-2 grid share 3 doubles/node) and G2P-2 (reads x3 v3 V0 F9 eps6 alpha
# ep6, writes x3 V F9 eps6 sigma6 alpha ep6 vm = 496 B, + 6 doubles/node gathered)
BYTES_MUSL = {"p2g": 112 + 7, "g2p": 80 + 3 + 496 + 6, "step": 720}
# Johnson-Cook, FP64: G2P reads x3 v3 V0 F9 eps6 sigma6 alpha alphadot (30 doubles)
# and writes x3 v3 V F9 eps6 sigma6 alpha alphadot vm (31 doubles) -> 488 B
BYTES_JC = {"p2g": 112 + 7, "g2p": 488 + 6, "step": 560}
# Johnson-Cook with damage, FP64: as Johnson-Cook plus damage_init, damage and
# temperature read and written and vm read (kept by failed particles) -> 544 B
BYTES_JCD = {"p2g": 112 + 7, "g2p": 544 + 6, "step": 616}


def launches_per_run(args, nbodies, p2g=None):
    """Kernels of the timed steps: USL clear + P2G per body + grid update (which
    lists the node blocks in the same launch) + G2P per body; MUSL: clear, P2G,
    compaction, its grid update, G2P-1 per body and, in 3D, the gradient
    velocity pass (2D: the solve and the node pass in place of the grid update);
    a cell sort is a key pass per body, three scan passes and the scatter.  The
    fused strategy runs all timed steps in one launch."""
    if p2g == "fused":
        return 1
    per_step = 2 + 2 * nbodies if args.algorithm == "usl" else 4 + 3 * nbodies
    sorts = args.steps // args.sort_interval if args.sort_interval > 0 else 0
    return args.steps * per_step + sorts * (nbodies + 4)


def scheme_kw(args):
    """Descriptor arguments of the update scheme and basis under test."""
    kw = {"basis": args.basis} if args.basis != "linear" else {}
    if args.algorithm == "musl":
        kw.update(algorithm="musl", alpha=args.alpha)
    return kw


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class timed_range:
    """NVTX range around the timed region (a no-op where NVTX is unavailable), so an ncu
    launch list can take exactly its kernels (--nvtx --nvtx-include "timed_steps/")."""

    def __init__(self, name):
        self.name = name
        self.nvtx = None

    def __enter__(self):
        try:
            import torch
            self.nvtx = torch.cuda.nvtx
            self.nvtx.range_push(self.name)
        except Exception:
            self.nvtx = None
        return self

    def __exit__(self, *exc):
        if self.nvtx is not None:
            self.nvtx.range_pop()
        return False


def variant_tag(args):
    """Profile-name tag of the update scheme, basis and material under test ("" for
    USL, the linear basis and J2, the default workload)."""
    tag = ""
    if args.algorithm == "musl":
        tag += "_musl"
    if args.basis != "linear":
        tag += f"_{args.basis}"
    if args.material != "j2":
        tag += f"_{args.material}"
    return tag


def ncu_fp64_inst(stage: str, tag: str):
    """FP64-pipe instructions per particle of a stage's kernels (ncu, committed variants
    table; MUSL's g2p stage is G2P-1 + G2P-2), or None when the table has no such row."""
    name = {"": "j2", "_jc": "jc", "_jcdamage": "jcdamage", "_musl": "musl", "_quad": "quad",
            "_cubic": "cubic"}.get(tag)
    path = os.path.join(ROOT, "profiles", "kernels_taylor_bar_variants_f64.txt")
    if name is None or not os.path.exists(path):
        return None
    total = None
    for line in open(path):
        cols = [c.strip() for c in line.split("|")]
        if len(cols) > 8 and cols[0] == name and stage in cols[1]:
            total = (total or 0.0) + float(cols[8])
    return total


def ncu_traffic(kernel: str, precision: str, tag: str = ""):
    """DRAM bytes per launch from the committed ncu summary of this exact variant, if one exists:
    the per-kernel file of the default workload, or the keyed line of the variants table."""
    if not tag:
        path = os.path.join(ROOT, "profiles", f"{kernel}_taylor_bar_{precision}.txt")
        if os.path.exists(path):
            for line in open(path):
                if line.startswith("traffic_bytes_per_launch_full_size:"):
                    return float(line.split(":", 1)[1])
        return None
    path = os.path.join(ROOT, "profiles", f"kernels_taylor_bar_variants_{precision}.txt")
    key = f"traffic[{kernel}{tag}]:"
    if os.path.exists(path):
        for line in open(path):
            if line.startswith(key):
                return float(line.split(":", 1)[1])
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    def __init__(self):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                       "-lms", "100"], stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.15)
        self.p.terminate()
        self.p.wait()
        self.f.seek(0)
        dev = os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0]
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9 or (dev.isdigit() and parts[0] != dev):
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.f.name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# Steps each Taylor-bar variant runs from the impact before the first error
# (det F <= 0 at the crushed corner, or a particle leaving the grid), measured
# on the GPU in steps of 25 (the FP64 J2 bar fails at the same step in the
# oracle).  MUSL and the B-spline bases ran 2200 steps without one.  The late
# window and the end-to-end solve stay within 80% of it.
HEALTHY_STEPS = {("j2", "f64"): 1450, ("j2", "dw"): 1450, ("j2", "f32"): 925, ("jc", "f64"): 1250, ("jc", "f32"): 1250,
                 ("jcdamage", "f64"): 200, ("jcdamage", "f32"): 100}


def healthy_steps(args):
    """Steps the workload runs before its first error, or None if it has no such limit here."""
    if args.workload != "taylor_bar":
        return None
    if args.algorithm != "usl" or args.basis != "linear":
        return 2200
    return HEALTHY_STEPS.get((args.material, args.precision))


def workload(name: str, material: str = "j2"):
    from jump_gb300 import scenarios
    if name == "taylor_bar":
        g, s, alg, data = scenarios.taylor_bar()
        # the J2 copper, or the Johnson-Cook copper / Johnson-Cook steel with damage of
        # the reference's Taylor-bar drivers, on the copper bar's geometry and time step
        label = scenarios.taylor_material(s[0], material, 2.5e-4)
        cfg = {"workload": f"taylor_bar_3d_{material}", "particles": int(s[0].parCount), "grid_nodes": [65, 65, 161],
               "h_m": 2.5e-4, "particles_per_cell": 8, "material": label,
               "dt_s": data["dt"], "l2": "inputs larger than L2 (~230 MB resident)"}
    elif name == "two_disks":
        g, s, alg, data = scenarios.two_disks()
        cfg = {"workload": "two_disks_2d_elastic", "particles": int(sum(x.parCount for x in s)),
               "grid_nodes": [21, 21], "l2": "fits in L2 (latency-bound case)"}
    else:
        raise SystemExit(f"unknown workload {name}")
    scenarios.apply_dirichlet(g, data)
    return g, s, alg, data, cfg


def dist_init(world, backend=None):
    """One process per GPU (torchrun env): NCCL when this rank sees a GPU, else gloo."""
    if world <= 1:
        return None
    import torch.distributed as dist
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    if backend is None:
        backend = "nccl"
        try:
            import torch
            torch.cuda.set_device(0)
        except Exception:
            backend = "gloo"
    dist.init_process_group(backend=backend)
    return dist


def shard(n: int, rank: int, world: int) -> list[int]:
    """Problems of an ensemble that rank runs: every world-th one from rank, so
    ranks get the seeded size mix alike; together the ranks cover 0..n-1 once."""
    return list(range(rank, n, world))


def aggregate(dist, device_s: float, units: float):
    """Whole-job throughput: units summed over ranks / the slowest rank's time."""
    t_max = allreduce_max(dist, device_s)
    total = allreduce_sum(dist, units)
    return t_max, total, total / t_max


def allreduce_max(dist, x: float) -> float:
    if dist is None:
        return x
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def allreduce_sum(dist, x: float) -> float:
    if dist is None:
        return x
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t)
    return float(t.item())


def pinned_like(a: np.ndarray) -> np.ndarray:
    """A copy of a in page-locked host memory with a's strides (so column-major
    matrix views stay column-major)."""
    import torch
    t = torch.empty_strided(a.shape, tuple(x // a.itemsize for x in a.strides),
                            dtype=torch.from_numpy(np.zeros(0, a.dtype)).dtype, pin_memory=True)
    out = t.numpy()  # the array's base keeps the pinned tensor alive
    np.copyto(out, a)
    return out


PARTICLE_ARRAYS = ("pos", "velocity", "mass", "volume", "volumeInitial", "deformationGradient", "strain",
                   "stress", "youngs")
MATERIAL_ARRAYS = ("alpha", "pstrain", "pstrain_3D", "alphadot", "vmStr", "damage_init", "dam")


def pin_solids(solids):
    for sol in solids:
        for k in PARTICLE_ARRAYS:
            if getattr(sol, k, None) is not None:
                setattr(sol, k, pinned_like(getattr(sol, k)))
        for k in MATERIAL_ARRAYS:
            if getattr(sol.mat, k, None) is not None:
                setattr(sol.mat, k, pinned_like(getattr(sol.mat, k)))
    return solids


def pin_state(st):
    for k in st.FIELDS:
        setattr(st, k, pinned_like(getattr(st, k)))
    return st


def cpu_sample(desc_factory, np_total, threads, target_s):
    """Time the CPU oracle on the same workload for about target_s seconds."""
    from oracle.oracle import OracleContext
    ctx = OracleContext(desc_factory(), threads=threads)
    ctx.step(1, check=False)  # first touch
    steps, t0 = 0, time.perf_counter()
    while True:
        ctx.step(1, check=False)
        steps += 1
        el = time.perf_counter() - t0
        if el >= target_s or steps >= 1000:
            break
    ctx.close()
    return np_total * steps / el, steps, el


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from jump_gb300.engine import Descriptors
    from oracle import oracle
    oracle.build()
    g, s, alg, data, cfg = workload(args.workload, args.material)
    npart = sum(x.parCount for x in s)
    mk = lambda: Descriptors(g, s, tolerance=alg.tolerance, body_force=data.get("bodyforce"), dt=data["dt"],
                             **scheme_kw(args))
    threads = oracle.max_threads() if args.algorithm == "usl" else 1  # the oracle's MUSL is single-threaded
    ctx = oracle.OracleContext(mk(), threads=threads)
    for _ in range(args.warmup):
        ctx.step(1, check=False)
    t0 = time.perf_counter()
    ctx.step(args.steps, check=False)
    el = time.perf_counter() - t0
    ctx.close()
    value = npart * args.steps / el
    out = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (geometry-generated particles)",
        "config": dict(cfg, algorithm=args.algorithm if args.algorithm == "usl" else f"musl(alpha={args.alpha})",
                       basis=args.basis),
        "cpu_baseline": {"value": value, "unit": METRIC, "cores": threads, "kind": "port",
                         "sample": f"{args.steps} full {args.algorithm.upper()} steps of the workload after {args.warmup} warm-up "
                                   f"steps; C++ restatement of the Julia loops (Julia is not installed on the "
                                   f"host), OpenMP over {threads} threads"},
        "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))


def import_nvtx():
    """Import torch (for its NVTX ranges) before any clock starts: a first import takes
    seconds and must not land inside a timed region."""
    try:
        import torch  # noqa: F401
        return True
    except Exception:
        return False


def plastic_fraction(ctx) -> float:
    """Share of particles with plastic strain (alpha > 0), all bodies."""
    sts = ctx.download_all()
    n = sum(st.n for st in sts)
    return float(sum(int(np.count_nonzero(st.alpha > 0)) for st in sts)) / max(n, 1)


def late_window(args, ctx, npart, advanced_before):
    """The same step timed again after advancing the bar args.late_steps steps into its
    mushrooming, plastically flowing phase (more active node blocks, more particles on
    the return-mapping branch, disordered particles), with the tuner re-run there.
    The default 1000 steps (about 11 us of the impact) stays inside the run's healthy
    range: with the linear hat basis the crushed impact corner of the J2 bar reaches
    det F <= 0 near step 1450, in the oracle as on the GPU; other variants are capped
    by HEALTHY_STEPS."""
    ctx.step(args.late_steps)  # untimed
    tuning = ctx.tune(3) if args.tune else None
    launch = ctx.launch()
    ctx.step(args.warmup)
    sampler = ClockSampler()
    t0 = time.perf_counter()
    ctx.step(args.steps)
    wall = time.perf_counter() - t0
    clocks = sampler.stop()
    dev = ctx.last_step_ms() / 1e3
    steps_before = advanced_before + args.late_steps + args.warmup
    return {"value": npart * args.steps / dev, "unit": METRIC, "ms_per_step": 1e3 * dev / args.steps,
            "wall_ms_per_step": 1e3 * wall / args.steps, "steps": args.steps,
            "steps_before_window": steps_before, "plastic_particles_frac": plastic_fraction(ctx),
            "launch": launch, "launch_chosen_by": "mpm_tune" if tuning else "defaults",
            "tuning_ms_per_step": tuning["ms_per_step"] if tuning else None, "clocks": clocks,
            "how": f"after {steps_before} steps from the impact (the timed window of the headline starts at step "
                   f"{args.warmup})"}


def e2e_solve(args, g, s, alg, data, launch, precision):
    """End to end through the public API: one solve of max(K, --e2e-steps)
    steps from host arrays.  The caller's particle arrays (inputs) and the
    arrays it downloads into (outputs) sit in pinned host memory before the
    clock starts, like a solver's own Solid arrays.  Timed: packing the
    descriptors, mpm_create (every host->device copy), the steps with the
    EnergiesFix sums of every step (mpm_step_energies, the solver's path when
    no hook reads particle arrays: each step's record formed on the device,
    all of them copied to the host at the end of the call), and the download
    of every field.  Returns (wall s, steps, host->device bytes, device->host
    bytes of the fields, record bytes per step, the parts in ms)."""
    import copy
    from jump_gb300.engine import BodyState, Descriptors, MPMContext
    s_pin = pin_solids(copy.deepcopy(s))
    out_states = [pin_state(BodyState(x.parCount, x.dim)) for x in s]
    t0 = time.perf_counter()
    desc = Descriptors(g, s_pin, tolerance=alg.tolerance, body_force=data.get("bodyforce"), dt=data["dt"],
                       precision=precision, sort_interval=launch["sort_interval"], **scheme_kw(args))
    c2 = MPMContext(desc)
    c2.set_launch(**launch)
    t1 = time.perf_counter()
    limit = healthy_steps(args)
    steps = max(args.steps, min(args.e2e_steps, int(0.8 * limit)) if limit else args.e2e_steps)
    recs, _ = c2.step_energies(steps, 1, 0)
    t2 = time.perf_counter()
    assert recs.shape[0] == steps and np.all(np.isfinite(recs))
    states = c2.download_all(out_states)
    wall = time.perf_counter() - t0
    parts = {"create_ms": 1e3 * (t1 - t0), "steps_ms": 1e3 * (t2 - t1), "download_ms": 1e3 * (t0 + wall - t2)}
    c2.close()
    h2d = sum(a.nbytes for a in desc._keep)
    d2h = sum(sum(getattr(stt, k).nbytes for k in stt.FIELDS) for stt in states)
    return wall, steps, h2d, d2h, recs.itemsize * recs.shape[1], parts


def run_ours(args):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    dist = dist_init(world)
    import_nvtx()
    from jump_gb300 import _capi
    if not os.path.exists(_capi.LIB_PATH):
        from jump_gb300 import build
        build.build()
    from jump_gb300.engine import Descriptors, MPMContext

    g, s, alg, data, cfg = workload(args.workload, args.material)
    npart = sum(x.parCount for x in s)
    mk = lambda: Descriptors(g, s, tolerance=alg.tolerance, body_force=data.get("bodyforce"), dt=data["dt"],
                             precision=args.precision, sort_interval=args.sort_interval, **scheme_kw(args))
    ctx = MPMContext(mk())
    tuning = None
    if args.tune:
        # the context's autotuner picks the P2G strategy, CTA size and sort interval
        # (outside the timed region; the simulation does not advance)
        tuning = ctx.tune(3)
    launch = ctx.launch()
    args.sort_interval = launch["sort_interval"]
    ctx.step(args.warmup)
    sampler = ClockSampler()
    if dist is not None:
        dist.barrier()
    t0 = time.perf_counter()
    with timed_range("timed_steps"):  # NVTX range: launch lists capture exactly these steps
        ctx.step(args.steps)  # synchronizes the context stream before returning
    wall = time.perf_counter() - t0
    dev_ms = ctx.last_step_ms()
    if dist is not None:
        dist.barrier()
    clocks = sampler.stop()
    t_max, total_updates, value = aggregate(dist, dev_ms / 1e3, float(npart * args.steps))

    # per-stage device times (individual launches, CUDA events on the context stream)
    nprof = max(3, min(args.steps, 10))
    st = ctx.profile_stages(nprof)
    per = {k: v / nprof for k, v in st.items()}
    dom = max(("p2g", "g2p"), key=lambda k: per[k])
    peak, peak_kind = load_peaks()
    table = BYTES_MUSL if args.algorithm == "musl" else (BYTES_JCD if args.material == "jcdamage" and args.precision == "f64" else
                                                         BYTES_JC if args.material == "jc" and args.precision == "f64"
                                                         else BYTES[args.precision])
    bts = table[dom] * npart
    achieved = bts / (per[dom] * 1e-3) / 1e9
    traffic = ncu_traffic(dom, args.precision, variant_tag(args))
    # FP64 roofline: the stage's FP64-pipe instructions (ncu count per particle) over
    # its live CUDA-event time, against the FP64 FMA rate measured in this run
    fp64 = None
    inst = ncu_fp64_inst(dom, variant_tag(args)) if args.precision == "f64" else None
    fma = C.c_double(0.0)
    if inst is not None and _capi.lib().mpm_probe_rates(C.byref(fma), None, None) == 0 and fma.value > 0:
        ach = inst * npart / (per[dom] * 1e-3)
        fp64 = {"bound": "fp64_pipe", "kernel": dom, "fp64_pipe_inst_per_particle": inst, "achieved": ach,
                "peak": fma.value, "unit": "FP64 inst/s", "frac": ach / fma.value,
                "peak_source": "mpm_probe_rates (FP64 FMA throughput, this run)"}
    step_bytes = table["step"] * npart
    # the FP64 state after warm-up, timed steps and stage profile, for the
    # double-word variant's comparison (which runs the same sequence)
    fp64_state = ctx.download_all() if (world == 1 and args.extras and args.workload == "taylor_bar" and
                                        args.precision == "f64") else None
    late = None
    if world == 1 and args.workload == "taylor_bar" and args.late_steps > 0:
        used = args.warmup + args.steps + nprof
        limit = healthy_steps(args)
        room = int(0.8 * limit) - used - args.warmup - args.steps if limit else args.late_steps
        if room >= 100:
            args.late_steps = min(args.late_steps, room)
            late = late_window(args, ctx, npart, used)
        else:
            late = {"skipped": f"the variant reaches its first error (det F <= 0 or a particle leaving the grid) "
                               f"near step {limit}, too early for a late window"}
    ctx.close()

    e2e_wall, e2e_steps, h2d, d2h, rec_bytes, parts = e2e_solve(args, g, s, alg, data, launch, args.precision)
    e2e_t = allreduce_max(dist, e2e_wall)
    e2e_value = allreduce_sum(dist, float(npart * e2e_steps)) / e2e_t

    extras = {}
    if world == 1 and args.extras and args.workload == "taylor_bar" and args.precision == "f64":
        # the benchmark spec's other three targets, each on its own workload
        extras["double_word"] = measure_double_word(args, (g, s, alg, data), mk, npart, nprof, fp64_state, peak,
                                                    peak_kind)
        extras["ensemble"] = measure_ensemble(args, "ensemble", "f64", 512, 1000)
        extras["adjoint"] = measure_adjoint(args, 2000)
        extras["impact_jvp"] = measure_impact_jvp(args, 64, 200)

    if rank == 0:
        cpu = None
        if world == 1 and not args.no_cpu:
            from oracle import oracle
            oracle.build()
            thr = oracle.max_threads() if args.algorithm == "usl" else 1  # the oracle's MUSL is single-threaded
            v_all, n_all, el_all = cpu_sample(lambda: Descriptors(g, s, tolerance=alg.tolerance,
                                                                  body_force=data.get("bodyforce"),
                                                                  dt=data["dt"], **scheme_kw(args)),
                                              npart, thr, args.cpu_seconds)
            v_one, n_one, el_one = cpu_sample(lambda: Descriptors(g, s, tolerance=alg.tolerance,
                                                                  body_force=data.get("bodyforce"),
                                                                  dt=data["dt"], **scheme_kw(args)),
                                              npart, 1, args.cpu_seconds / 3)
            cpu = {"value": v_all, "unit": METRIC, "cores": thr, "kind": "port",
                   "sample": f"{n_all} {args.algorithm.upper()} steps of the same workload in {el_all:.1f} s (FP64 C++ "
                             f"restatement of the reference loops, OpenMP {thr} threads); single thread: "
                             f"{v_one:.4g} {METRIC} over {n_one} steps",
                   "single_thread_value": v_one}
        out = {
            "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": args.precision,
            "data": "synthetic (geometry-generated particles, no dataset)",
            "config": dict(cfg, precision=args.precision, sort_interval=args.sort_interval,
                           algorithm=args.algorithm if args.algorithm == "usl" else f"musl(alpha={args.alpha})",
                           basis=args.basis, p2g=launch["p2g"], threads=launch["threads"],
                           launch_chosen_by="mpm_tune" if tuning else "defaults",
                           parallelism=f"replicas{world}" if world > 1 else "single-gpu"),
            "tuning": tuning,
            "wall_ms_per_step": 1e3 * wall / args.steps,
            "stage_ms_per_step": per,
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind,
                         "algorithmic_bytes_per_launch": bts,
                         "implementation_bytes_per_particle": {"hat_cache": HAT if args.precision == "f64" and
                                                               args.basis == "linear" and args.algorithm == "usl"
                                                               else 0},
                         "step_frac": step_bytes / (t_max / args.steps) / 1e9 / peak, "fp64": fp64},
            "late_window": late,
            "e2e": {"value": e2e_value, "unit": METRIC, "steps": e2e_steps,
                    "h2d_bytes_per_step": h2d / e2e_steps,
                    "d2h_bytes_per_step": d2h / e2e_steps + rec_bytes, "host_memory": "pinned",
                    "how": f"one solve: create from host arrays, {e2e_steps} steps each with its EnergiesFix record "
                           "(mpm_step_energies: formed on the device, all records copied to the host at the end), "
                           "download all",
                    **parts},
            "gpu_launches": launches_per_run(args, len(s), launch["p2g"]),
            "clocks": clocks,
            "cpu_baseline": cpu,
            **extras,
        }
        print(json.dumps(out))
    if dist is not None:
        dist.destroy_process_group()


def measure_double_word(args, problem, mk_fp64, npart, nprof, fp64_state, peak, peak_kind):
    """The MPM_PREC_DW variant of the same step (FP64 fields and node sums, the P2G
    and G2P arithmetic in double-word FP32): the same warm-up, timed steps and
    stage profile as the FP64 context, its device throughput and HBM roofline,
    the largest relative difference per field from the FP64 state at the same
    step, and the end-to-end solve of the FP64 line on a double-word context.
    Reported beside the FP64 headline, not as it."""
    from jump_gb300 import _capi
    from jump_gb300.engine import MPMContext
    d = mk_fp64()
    d.params.precision = _capi.MPM_PREC_DW  # the same descriptors
    ctx = MPMContext(d)
    tuning = ctx.tune(3) if args.tune else None  # CTA size and sort interval (its P2G is per-lane atomics)
    ctx.step(args.warmup)
    ctx.step(args.steps)
    dev_ms = ctx.last_step_ms()
    st = ctx.profile_stages(nprof)
    per = {k: v / nprof for k, v in st.items()}
    dom = max(("p2g", "g2p"), key=lambda k: per[k])
    states = ctx.download_all()
    launch = ctx.launch()
    ctx.close()
    err = {}
    for f in ("pos", "velocity", "volume", "F", "strain", "stress", "alpha", "pstrain"):
        a = np.concatenate([np.ravel(getattr(x, f)) for x in states])
        b = np.concatenate([np.ravel(getattr(x, f)) for x in fp64_state])
        den = float(np.max(np.abs(b))) or 1.0
        err[f] = float(np.max(np.abs(a - b)) / den)
    achieved = BYTES["dw"][dom] * npart / (per[dom] * 1e-3) / 1e9
    g, s, alg, data = problem
    wall, steps, h2d, d2h, rec_bytes, parts = e2e_solve(args, g, s, alg, data, launch, "dw")
    e2e = {"value": npart * steps / wall, "unit": METRIC, "steps": steps, "h2d_bytes_per_step": h2d / steps,
           "d2h_bytes_per_step": d2h / steps + rec_bytes, "host_memory": "pinned",
           "how": "as the FP64 line's e2e, on a double-word context", **parts}
    return {"precision": "dw", "value": npart * args.steps / (dev_ms * 1e-3), "unit": METRIC, "e2e": e2e,
            "ms_per_step": dev_ms / args.steps, "stage_ms_per_step": per, "launch": launch,
            "launch_chosen_by": "mpm_tune" if tuning else "defaults",
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_source": peak_kind,
                         "traffic": ncu_traffic(dom, "dw"),
                         "step_frac": BYTES["dw"]["step"] * npart / (dev_ms * 1e-3 / args.steps) / 1e9 / peak},
            "max_rel_diff_vs_fp64_gpu": err,
            "steps_compared": args.warmup + args.steps + nprof,
            "what": "FP64 particle fields and node accumulators; P2G and G2P arithmetic in double-word FP32 "
                    "(float pairs, 2^-49 relative per rounding); not the FP64 headline"}


ENSEMBLES = {
    # workload: (problem i, default problems per GPU, default steps per solve, config name)
    "ensemble": ("ensemble_member", 512, 1000, "two_disk_ensemble_2d"),
    "impact_ensemble": ("impact_member", 64, 200, "sphere_plate_impact_ensemble_3d_contact"),
}


def _problem_bytes(ens) -> int:
    """Host bytes an Ensemble's creation copies to the device (every descriptor array)."""
    return int(sum(sum(a.nbytes for a in d._keep) for d in ens._descs))


def _states_bytes(states) -> int:
    return int(sum(sum(getattr(st, k).nbytes for k in st.FIELDS) for st in states))


def measure_ensemble(args, workload, precision, n, steps, mine=None, one_by_one=True, accuracy=False):
    """Batched ensemble: solves/s of one batch (strategy and launch shape autotuned;
    device time of `steps` steps after a warm-up), the same problems one after
    another through single contexts (a stratified sample of up to 32 problems,
    scaled to the ensemble), and end to end through the public API: the batch
    built from host arrays (every upload), the solve, and every problem's state
    downloaded, against the wall clock."""
    from jump_gb300 import scenarios
    from jump_gb300.batch import Ensemble
    from jump_gb300.engine import Descriptors, MPMContext
    gen_name, _, _, cfg_name = ENSEMBLES[workload]
    member = getattr(scenarios, gen_name)
    mine = list(range(n)) if mine is None else mine
    probs = [member(i) for i in mine]
    ens = Ensemble(probs, precision=precision)
    tune = ens.tune(probe_steps=10)
    ens.step(args.warmup)
    sampler = ClockSampler()
    t0 = time.perf_counter()
    ens.step(steps)
    wall = time.perf_counter() - t0
    clocks = sampler.stop()
    dev = ens.last_ms() / 1e3
    npart = ens.particles
    acc_idx = list(range(0, len(probs), max(1, len(probs) // 16)))[:16]
    got = [ens.download(i) for i in acc_idx] if accuracy else None
    ens.close()
    # end to end: a new batch of the same problems from host arrays; the tuned
    # strategy and launch shape come from the tuner's cache
    probs2 = [member(i) for i in mine]
    t0 = time.perf_counter()
    e2 = Ensemble(probs2, precision=precision)
    e2.tune(probe_steps=10)
    t1 = time.perf_counter()
    e2.step(steps)
    t2 = time.perf_counter()
    states = [st for i in range(len(probs2)) for st in e2.download(i)]
    e2e_wall = time.perf_counter() - t0
    h2d, d2h = _problem_bytes(e2), _states_bytes(states)
    e2.close()
    out = {"metric": "solves/s", "value": len(mine) / dev, "unit": "solves/s", "steps": steps,
           "warmup": args.warmup, "ms_per_step": 1e3 * dev / steps, "higher_is_better": True, "dtype": precision,
           "data": "synthetic (seeded ensemble)",
           "config": {"workload": cfg_name, "instances": len(mine), "steps_per_solve": steps, "particles": int(npart),
                      "launch": tune},
           "particle_updates_per_s": npart * steps / dev, "wall_s": wall, "clocks": clocks,
           "e2e": {"value": len(mine) / e2e_wall, "unit": "solves/s", "h2d_bytes_per_step": h2d / steps,
                   "d2h_bytes_per_step": d2h / steps, "host_memory": "pageable",
                   "create_ms": 1e3 * (t1 - t0), "steps_ms": 1e3 * (t2 - t1), "download_ms": 1e3 * (t0 + e2e_wall - t2),
                   "how": "Ensemble(...) from the problems' host arrays (descriptors and every upload), "
                          f"{steps} steps, every problem's state downloaded"}}
    if one_by_one:
        sample = list(range(0, len(mine), max(1, len(mine) // 32)))[:32]
        t_one = 0.0
        for k in sample:
            grid, solids, alg, data = member(mine[k])
            scenarios.apply_dirichlet(grid, data)
            c = MPMContext(Descriptors(grid, solids, tolerance=alg.tolerance, body_force=data["bodyforce"],
                                       dt=data["dt"], precision=precision, contact=bool(data.get("contact")),
                                       friction=float(data.get("friction", 0.0))))
            c.step(args.warmup)
            t1 = time.perf_counter()
            c.step(steps)
            t_one += time.perf_counter() - t1
            c.close()
        v = len(sample) / t_one
        out["one_by_one"] = {"value": v, "unit": "solves/s", "sample": len(sample),
                             "how": "same problems, one context each, step graph replayed per step, host-timed"}
        out["speedup_vs_one_by_one"] = out["value"] / v
    if got is not None:
        # the error the FP32 batch's solves/s come at: against an FP64 batch of the same
        # problems after the same steps (max |difference| / max |FP64 value| per field,
        # normalised over the sampled problems: a problem whose disks have not met carries
        # rounding-noise stresses)
        ref = Ensemble([member(mine[i]) for i in acc_idx], precision="f64")
        ref.step(args.warmup + steps)
        diff, size = {}, {}
        for j in range(len(acc_idx)):
            for a_, b_ in zip(got[j], ref.download(j)):
                for f in ("pos", "velocity", "F", "stress"):
                    diff[f] = max(diff.get(f, 0.0), float(np.max(np.abs(getattr(a_, f) - getattr(b_, f)))))
                    size[f] = max(size.get(f, 0.0), float(np.max(np.abs(getattr(b_, f)))))
        ref.close()
        out["error_vs_fp64"] = {"fields": {f: diff[f] / (size[f] or 1.0) for f in diff}, "problems": len(acc_idx),
                                "how": "FP32 batch against an FP64 batch of the same problems after the same steps: "
                                       "max |difference| / max |FP64 value| over the sampled problems, per field"}
    return out


def run_ensemble(args):
    """Batched ensembles as the workload of the line (measure_ensemble); problems
    are sharded across ranks with no collective on the data path.  "ensemble":
    seeded two-disk problems (20^2..80^2 cells, 4 particles per cell).
    "impact_ensemble": seeded sphere-on-plate impacts (3D, 135,952 particles
    each, two velocity fields with the frictionless contact correction, speed in
    [10, 100] m/s, plate E in [1e9, 10e9] Pa)."""
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    dist = dist_init(world)
    import_nvtx()
    _, n_default, steps_default, _ = ENSEMBLES[args.workload]
    per_gpu = args.instances if args.instances is not None else n_default
    steps = args.solve_steps if args.solve_steps is not None else steps_default
    n = per_gpu * world  # problems per GPU fixed: weak scaling
    mine = shard(n, rank, world)  # problems are independent: no collective on the data path
    if dist is not None:
        dist.barrier()
    res = measure_ensemble(args, args.workload, args.precision, n, steps, mine=mine, one_by_one=world == 1,
                           accuracy=args.precision == "f32" and world == 1)
    dev, _, batched = aggregate(dist, res["ms_per_step"] * steps / 1e3, float(len(mine)))
    e2e_t = allreduce_max(dist, len(mine) / res["e2e"]["value"])
    if rank == 0:
        res.update({"value": batched, "n_gpus": world, "ms_per_step": 1e3 * dev / steps, "scaling": "weak",
                    "vs_baseline": None})
        res["config"].update(instances=n, parallelism=f"problems sharded over {world} ranks" if world > 1
                             else "single-gpu")
        res["e2e"]["value"] = n / e2e_t
        res["gpu_launches"] = None if res["config"]["launch"].get("strategy") != "persistent" else 1
        print(json.dumps(res))
    if dist is not None:
        dist.destroy_process_group()


def measure_adjoint(args, nsteps):
    """Differentiable cantilever (16,384 particles, neo-Hookean, per-particle E,
    nsteps steps at dt = 1e-4, checkpoint every 50): forward throughput against
    forward + adjoint throughput (medians of three alternating runs of each),
    the store-every-step mode, end to end (context
    from host arrays, forward with checkpoints, final positions downloaded, the
    reverse sweep, gradients in host memory), and the gradient of the
    tip-displacement loss against central differences on 32 random parameters
    (GPU forward runs)."""
    from jump_gb300 import scenarios
    from jump_gb300.adjoint import final_positions
    from jump_gb300.adjoint import make_context as _make

    def make_context(*a):
        c = _make(*a)
        if args.adjoint_p2g is not None:  # a tile strategy selects the tiled adjoint scatter too
            c.set_launch(p2g=args.adjoint_p2g)
        return c

    problem = scenarios.cantilever()
    grid, solids, alg, data = problem
    scenarios.apply_dirichlet(grid, data)
    every = 50
    E = np.concatenate([s.youngs for s in solids])
    v0 = np.concatenate([s.velocity for s in solids])
    npart = len(E)
    x0 = np.concatenate([s.pos for s in solids])
    tip = x0[:, 0] > np.quantile(x0[:, 0], 0.95)
    c = make_context(problem, 1.3 * E, v0)
    c.step(nsteps)
    target = final_positions(c)[tip]
    c.close()

    def loss_grad(x):
        g = np.zeros_like(x)
        g[tip] = 2.0 * (x[tip] - target)
        return g

    c = make_context(problem, E, v0)
    c.step(args.warmup)
    c.close()
    # forward and forward + adjoint, three of each, alternating, each on a fresh
    # context from the same initial state; the medians are reported
    fwd_s, both_s = [], []
    sampler = ClockSampler()
    for _ in range(3):
        c = make_context(problem, E, v0)
        t0 = time.perf_counter()
        c.step(nsteps)
        fwd_s.append(time.perf_counter() - t0)
        c.close()
        c = make_context(problem, E, v0)
        t0 = time.perf_counter()
        c.fwd_checkpointed(nsteps, every)
        x = final_positions(c)
        g = c.bwd(loss_grad(x))
        both_s.append(time.perf_counter() - t0)
        c.close()
    clocks = sampler.stop()
    fwd, both = float(np.median(fwd_s)), float(np.median(both_s))
    # end to end: the same with the context built from the host arrays inside the clock
    t0 = time.perf_counter()
    c = make_context(problem, E, v0)
    c.fwd_checkpointed(nsteps, every)
    x = final_positions(c)
    g_e2e = c.bwd(loss_grad(x))
    e2e = time.perf_counter() - t0
    c.close()
    # the same with every step's state and node buffer kept (no recompute)
    c = make_context(problem, E, v0)
    t0 = time.perf_counter()
    c.fwd_checkpointed(nsteps, 1)
    x1 = final_positions(c)
    g1 = c.bwd(loss_grad(x1))
    both_all = time.perf_counter() - t0
    c.close()
    store_all_dev = float(np.max(np.abs(g1["E"] - g["E"])) / np.max(np.abs(g["E"])))
    loss = lambda xx: float(np.sum((xx[tip] - target) ** 2))
    rng = np.random.default_rng(11)
    ids = rng.choice(npart, 32, replace=False)
    fd = []
    for p in ids:
        h = 1e-4 * E[p]
        vals = []
        for sgn in (1.0, -1.0):
            Ep = E.copy()
            Ep[p] += sgn * h
            cc = make_context(problem, Ep, v0)
            cc.step(nsteps)
            vals.append(loss(final_positions(cc)))
            cc.close()
        fd.append((vals[0] - vals[1]) / (2 * h))
    fd = np.array(fd)
    ad = g["E"][ids]
    d = grid.dim if hasattr(grid, "dim") else 2
    return {"metric": "particle-updates/s", "value": npart * nsteps / both, "unit": "particle-updates/s",
            "n_gpus": 1, "steps": nsteps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded per-particle E)",
            "config": {"workload": "cantilever_2d_neohookean_adjoint", "particles": npart,
                       "p2g": args.adjoint_p2g or "atomic",
                       "checkpoint_every": every, "loss": "squared tip displacement error (top 5% in x)"},
            "forward_particle_updates_per_s": npart * nsteps / fwd,
            "fwd_adj_over_fwd_throughput": fwd / both,
            "samples_s": {"forward": fwd_s, "forward_adjoint": both_s, "reported": "medians"},
            "clocks": clocks,
            "e2e": {"value": npart * nsteps / e2e, "unit": "particle-updates/s",
                    "h2d_bytes_per_step": (npart * (2 * d + 3 + 3 * d * d + 1) * 8 + x.nbytes) / nsteps,
                    "d2h_bytes_per_step": (x.nbytes + g_e2e["E"].nbytes + g_e2e["v0"].nbytes + g_e2e["x0"].nbytes
                                           + npart * (2 * d + 1 + 3 * d * d + 4 + 4 * d) * 8) / nsteps,
                    "how": "context from host arrays, forward with checkpoints, final state downloaded, reverse "
                           "sweep with dL/dx uploaded, dL/dE, dL/dv0, dL/dx0 downloaded; host-timed"},
            "store_every_step": {"fwd_adj_over_fwd_throughput": fwd / both_all,
                                 "particle_updates_per_s": npart * nsteps / both_all,
                                 "device_memory_gb": round(nsteps * (npart * 25 * 8 + 4745 * 9 * 8) / 1e9, 2),
                                 "grad_max_rel_diff_vs_checkpointed": store_all_dev},
            "fd_check": {"params": 32, "norm_rel_err": float(np.linalg.norm(ad - fd) / np.linalg.norm(fd)),
                         "max_rel_err": float(np.max(np.abs(ad - fd)) / np.max(np.abs(fd))),
                         "step": "1e-4 relative, central, GPU forward runs"}}


def run_adjoint(args):
    import_nvtx()
    print(json.dumps(measure_adjoint(args, args.solve_steps)))


def measure_impact_jvp(args, n, steps):
    """Derivative of every impact problem's plate deflection (mean z of the
    plate particles after the solve) with respect to its plate modulus, by
    forward-mode tangents through the batched contact solve (mpm_batch_jvp,
    FP64, n problems x 135,952 particles), against the forward-only solve;
    checked for all problems at once against central differences of two
    batch runs with every plate modulus scaled by 1 +- 1e-6.  End to end: the
    batch built from host arrays, the tangent solve, the derivatives in host
    memory."""
    import copy
    from jump_gb300 import scenarios
    from jump_gb300.batch import Ensemble
    probs = [scenarios.impact_member(i) for i in range(n)]
    ns = probs[0][1][0].parCount
    seeds = [[0.0, p[1][1].mat.E] for p in probs]  # d/ds with E_plate = s * E0
    ens = Ensemble(probs, precision="f64")
    ens.set_strategy("wide")
    ens.step(args.warmup)
    ens.close()
    fwd = Ensemble(probs, precision="f64")
    fwd.set_strategy("wide")
    fwd.step(steps)
    t_fwd = fwd.last_ms() / 1e3
    fwd.close()
    t0 = time.perf_counter()
    tan = Ensemble(probs, precision="f64")
    h2d = _problem_bytes(tan)
    t1 = time.perf_counter()
    sampler = ClockSampler()
    xd = tan.jvp(steps, seeds)
    e2e = time.perf_counter() - t0
    clocks = sampler.stop()
    t_jvp = tan.last_ms() / 1e3
    ad = np.array([float(np.mean(xd[i][ns:, 2])) for i in range(n)])
    tan.close()
    fd = np.zeros(n)
    for sgn in (1.0, -1.0):
        pp = []
        for g, s, alg, data in probs:
            s = copy.deepcopy(s)
            s[1].mat.E *= 1 + sgn * 1e-6
            pp.append((g, s, alg, data))
        e = Ensemble(pp, precision="f64")
        e.set_strategy("wide")
        e.step(steps)
        fd += sgn * np.array([float(np.mean(e.download(i)[1].pos[:, 2])) for i in range(n)]) / 2e-6
        e.close()
    rel = np.abs(ad - fd) / np.abs(fd)
    npart = sum(sum(x.parCount for x in p[1]) for p in probs)
    return {"metric": "particle-updates/s", "value": npart * steps / t_jvp, "unit": "particle-updates/s",
            "n_gpus": 1, "steps": steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_jvp / steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded ensemble)",
            "config": {"workload": "sphere_plate_impact_ensemble_3d_contact_jvp", "instances": n,
                       "steps_per_solve": steps, "particles": npart,
                       "derivative": "forward mode, d(mean plate z)/d(plate E) per problem"},
            "forward_particle_updates_per_s": npart * steps / t_fwd,
            "fwd_tangent_over_fwd_throughput": t_fwd / t_jvp,
            "solves_per_s_with_derivative": n / t_jvp,
            "e2e": {"value": npart * steps / e2e, "unit": "particle-updates/s", "h2d_bytes_per_step": h2d / steps,
                    "d2h_bytes_per_step": sum(x.nbytes for x in xd) / steps, "create_ms": 1e3 * (t1 - t0),
                    "how": "batch from the problems' host arrays (every upload), tangent solve, dx/ds of every "
                           "particle in host memory; host-timed"},
            "fd_check": {"problems": n, "max_rel_err": float(rel.max()), "median_rel_err": float(np.median(rel)),
                         "step": "1e-6 relative, central, FP64 batch runs"},
            "clocks": clocks}


def run_impact_jvp(args):
    import_nvtx()
    n = args.instances if args.instances is not None else 64
    steps = args.solve_steps if args.solve_steps is not None else 200
    print(json.dumps(measure_impact_jvp(args, n, steps)))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="f64", choices=["f64", "f32", "dw"])
    ap.add_argument("--algorithm", default="usl", choices=["usl", "musl"],
                    help="update scheme: USL (the headline) or MUSL (FLIP/PIC blend --alpha)")
    ap.add_argument("--alpha", type=float, default=1.0, help="MUSL FLIP/PIC blend")
    ap.add_argument("--basis", default="linear", choices=["linear", "quad", "cubic"],
                    help="shape functions: linear hat (the headline), quadratic or cubic B-splines")
    ap.add_argument("--material", default="j2", choices=["j2", "jc", "jcdamage"],
                    help="Taylor bar material: J2 linear hardening (the headline), Johnson-Cook, or Johnson-Cook "
                         "with damage")
    ap.add_argument("--sort-interval", type=int, default=0,
                    help="counting-sort particles by cell every N steps (0: never; with --tune the tuner's choice)")
    ap.add_argument("--tune", action=argparse.BooleanOptionalAction, default=True,
                    help="run the context's autotuner (P2G strategy, CTA size, sort interval) before timing")
    ap.add_argument("--workload", default="taylor_bar",
                    choices=["taylor_bar", "two_disks", "ensemble", "impact_ensemble", "impact_jvp", "adjoint"])
    ap.add_argument("--instances", type=int, default=None,
                    help="ensembles: problems per GPU (default 512 two-disk, 64 impact)")
    ap.add_argument("--solve-steps", type=int, default=None,
                    help="ensembles: steps per solve (default 1000 two-disk, 200 impact); adjoint: steps (2000)")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--late-steps", type=int, default=1000,
                    help="Taylor bar: steps advanced before the late-window measurement (0: none; capped so the "
                         "window ends within 80%% of the steps the variant runs before its first error)")
    ap.add_argument("--adjoint-p2g", default=None, choices=["atomic", "warp", "tile", "tile_warp"],
                    help="adjoint: P2G strategy of its contexts (a tile one selects the tiled adjoint scatter)")
    ap.add_argument("--e2e-steps", type=int, default=500,
                    help="Taylor bar: steps of the end-to-end solve (at least --steps; at most 80%% of the steps "
                         "the variant runs before its first error)")
    ap.add_argument("--extras", action=argparse.BooleanOptionalAction, default=True,
                    help="Taylor bar, FP64, 1 GPU: add the ensemble, adjoint and impact-jvp sub-results")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.workload in ENSEMBLES:
        run_ensemble(args)
    elif args.workload == "adjoint":
        args.solve_steps = args.solve_steps if args.solve_steps is not None else 2000
        run_adjoint(args)
    elif args.workload == "impact_jvp":
        run_impact_jvp(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
