"""Throughput of the nsmp3D hot path on GB300: Mcell-steps/s.

Workload (the 6.3M-prism configuration the headline metric is quoted on):
periodic channel Lx = 2*pi, Ly = pi, height 2, 256x128 quads split into
65,536 jittered triangles (mesh seed 0), 96 sigma layers tanh-clustered to
both walls (beta = 2): 6,291,456 prisms.  Re = 180, dp/dx = -1, Smagorinsky
Cs = 0.1 with van Driest damping, SSP-RK3 composed of the reference's stage
operator, dt = 2.5e-4, BiCGSTAB + Jacobi to 1e-10.  Initial state: the
reference's profile 18 z(2-z) plus uniform noise of half-width 1.8 (seed 1).

One step = one RK3 time step = three hydro() stages, each with its PPE solve.
All inputs are synthetic (no dataset exists for this path).  Timing: CUDA
events on the library's stream around K steps after W warm-up steps; the
working set (~2 GB) is far larger than L2, so no flush is needed.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
PKG_DIR = os.path.join(REPO, "3d-channel-flow-code_gb300")
for _p in (REPO, PKG_DIR):
    if _p not in sys.path:
        sys.path.insert(0, _p)

WORKLOADS = {
    # name: (nx, ny, layers, dt)
    "config0": (32, 16, 32, 1e-3),
    "config1": (128, 64, 64, 5e-4),
    "config2": (256, 128, 96, 2.5e-4),
    "config4": (512, 256, 128, 2.5e-4),
}

# Algorithmic FP64 words moved per interior prism by each kernel (each named
# field read or written once; neighbour reads served by cache; geometry
# amortised per column; vertex fields count N_class/N0 = 0.5 per prism).
WORDS = {
    "k_vertex4": 4 + 4 * 0.5, "k_stage_rhs": 3 + 1.5 + 5 + 3 + 3 + 3 + 1, "k_faces_div": 3 + 0.5 + 6,
    "k_bicg_init": 2 + 3, "k_bicg_p": 4, "k_bicg_spmv_v": 4, "k_bicg_s": 3, "k_bicg_spmv_t": 3,
    "k_bicg_x": 8, "k_pmean": 1, "k_vertex1": 1 + 0.5, "k_project": 1 + 0.5 + 3 + 5 + 4 + 5,
}
# FP64 flops per prism that the solver kernels execute (multiply, add and FMA
# counted as 1, 1 and 2 flops), by form of the SpMV.  Stored couplings: five
# FMAs a row plus the fused dots, (r0, v) or (t, s) and (t, t).  Matrix-free:
# two more multiplies a coupling, kA_j dsigv and the neighbour's D^-1.
# k_bicg_x: x += D^-1 (alpha p + omega s), r = s - omega t, |r|^2, |r|_1,
# (r0, r); k_bicg_p: p = r + beta (p - omega v); k_bicg_s: s = r - alpha v.
_FLOPS_VEC = {"k_bicg_x": 12, "k_bicg_p": 4, "k_bicg_s": 2}
FLOPS = {"stored": dict(_FLOPS_VEC, k_bicg_spmv_v=12, k_bicg_spmv_t=14),
         "matrix-free": dict(_FLOPS_VEC, k_bicg_spmv_v=22, k_bicg_spmv_t=24)}


# bench precision names -> the library's precision modes
PRECISIONS = {"fp64": lambda ng: ng.FP64, "mixed": lambda ng: ng.MIXED, "mixed_f32": lambda ng: ng.MIXED_F32}


def load_peaks():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as fh:
            d = json.load(fh)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group(backend="gloo")
        pg = dist
    return world, rank, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def max_over_ranks(pg, x):
    if pg is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def job_value(world, prisms, steps, ms_max):
    """Whole-job Mcell-steps/s: every rank advances its own replica of the
    workload, timed by the slowest rank."""
    return world * prisms * steps / (ms_max / 1e3) / 1e6


def workload_desc(name):
    nx, ny, layers, dt = WORKLOADS[name]
    return (f"periodic channel 2pi x pi x 2, {nx}x{ny} quads -> {2 * nx * ny} jittered triangles x {layers} "
            f"tanh(beta=2) layers = {2 * nx * ny * layers} prisms; RK3 dt={dt}; LES van Driest; "
            f"BiCGSTAB-Jacobi eps=1e-10")


def cpu_model():
    """One-line description of the host CPU (model name or Arm part)."""
    try:
        txt = open("/proc/cpuinfo").read()
    except OSError:
        return "unknown"
    for key in ("model name", "Model", "CPU part"):
        for ln in txt.splitlines():
            if ln.lower().startswith(key.lower()):
                val = ln.split(":", 1)[1].strip()
                return f"{key}: {val}" if key == "CPU part" else val
    return "unknown"


def oracle_workload(name, nthreads):
    """The CPU oracle on the workload, built from the oracle's own synthetic
    inputs (bit-identical to the library's), so no product code is loaded."""
    from oracle import oracle_ctypes as oc
    nx, ny, layers, dt = WORKLOADS[name]
    o = oc.Oracle(oc.channel_params(nx, ny, layers, dt), oc.make_mesh(nx, ny), nthreads=nthreads)
    return o, oc


def run_reference(args):
    """CPU arm: the reference's algorithm on the host cores -- the oracle
    port, since no Fortran toolchain exists to build the reference itself.
    From the same seeded initial state as the GPU arm it runs W full RK3
    warm-up steps, then times K full RK3 steps (all three stages with their
    PPE solves): the same steps the GPU arm times."""
    world, rank, local, pg = dist_setup()
    if rank != 0:
        return 0
    nthreads = args.ref_threads or os.cpu_count() or 1
    nx, ny, layers, dt = WORKLOADS[args.workload]
    prisms = 2 * nx * ny * layers
    o, oc = oracle_workload(args.workload, nthreads)
    o.user_initial(*o.initial_channel(seed=1))
    warm = []
    for _ in range(args.warmup):
        rc, info = o.step(3)
        warm.append(info["iters_stage"])
    stages = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        rc, info = o.step(3)
        stages.append(info["iters_stage"])
    t = time.perf_counter() - t0
    value = prisms * args.steps / t / 1e6
    its = float(np.mean(stages)) if stages else 0.0
    line = {
        "impl": "reference", "metric": "Mcell-steps/s", "value": value, "unit": "Mcell-steps/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t / max(args.steps, 1) * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": workload_desc(args.workload), "prisms": prisms,
                   "integrator": "SSP-RK3 of the reference stage", "bicgstab_iters_per_stage": round(its, 1)},
        "bicgstab_iters_per_stage_timed": stages, "bicgstab_iters_per_stage_warmup": warm,
        "cpu_baseline": {"value": value, "unit": "Mcell-steps/s", "cores": nthreads, "kind": "port",
                         "cpu": cpu_model(),
                         "sample": f"{args.steps} full RK3 steps (3 stages, PPE to 1e-10) after {args.warmup} "
                                   f"warm-up steps from the seeded initial state, wall clock"},
        "e2e": {"value": value, "unit": "Mcell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def cpu_step_from_state(args, snap, nthreads):
    """The oracle on one full RK3 step from the state the GPU arm's timed
    region started from (uploaded into the oracle): the same work as the
    first timed GPU step.  Returns (seconds, per-stage iterations)."""
    o, oc = oracle_workload(args.workload, nthreads)
    for a, f in zip(snap.cells, (oc.F_U, oc.F_V, oc.F_W, oc.F_P)):
        o.set(f, a)
    for a, f in zip(snap.faces, (oc.F_U1F, oc.F_U2F, oc.F_U3F, oc.F_UTF, oc.F_UBF)):
        o.set(f, a)
    for a, f in zip(snap.hist, (oc.F_RHSU, oc.F_RHSV, oc.F_RHSW)):
        o.set(f, a)
    o.set(oc.F_PV, snap.pv)
    o.flag_ab = snap.flag
    t0 = time.perf_counter()
    rc, info = o.step(3)
    return time.perf_counter() - t0, info["iters_stage"]


# Mixed solver, in 8-byte words per prism.  k_in_pv: s, t, p, v, D^-1 (stencil),
# e and r0 read, p, v, r and e written (11 FP32 words; the pass after an FP64
# update reads r instead of s and t and writes neither r nor e: 8).  k_in_st:
# r, v, D^-1 (stencil) and r0 read, s and t written (6 FP32 words).
# k_mix_update (incremental form): FP64 x and r read, e and the last
# increment's s and p (FP32, stencil) read, FP64 x and r written (5.5 words;
# the from-scratch form on the first call reads b and x instead).
# k_mix_scale: FP64 r, D^-1 and r0 read,
# FP32 r and e written (r0 rewritten only on a Krylov restart).
WORDS_MIXED = {
    "k_in_pv": 11 * 0.5, "k_in_st": 6 * 0.5, "k_mix_update": 1 + 1 + 3 * 0.5 + 2, "k_mix_scale": 1 + 4 * 0.5,
}


class StateBuffers:
    """The full restart state of a solver (u, v, w, p, five face fluxes, three
    AB2 histories, the AB2 flag) in pinned host arrays in the reference's
    Fortran layout."""

    CELLS = ("F_U", "F_V", "F_W", "F_P")
    FACES = ("F_U1FACE", "F_U2FACE", "F_U3FACE", "F_UTFACE", "F_UBFACE")
    HIST = ("F_RHSU", "F_RHSV", "F_RHSW")

    def __init__(self, torch, ng, s, prm):
        pin = lambda shape: torch.empty(shape[::-1], dtype=torch.float64, pin_memory=True).numpy().T
        nc, nz, n0 = s.ncell, s.nz, prm["n0"]
        self.ids = [[getattr(ng, n) for n in grp] for grp in (self.CELLS, self.FACES, self.HIST)]
        self.cells = [pin((nc, nz)) for _ in self.CELLS]
        self.faces = [pin((n0, nz)) for _ in self.FACES]
        self.hist = [pin((nc, nz)) for _ in self.HIST]
        self.flag = 0
        self.nbytes = sum(a.nbytes for a in self.cells + self.faces + self.hist)

    def download(self, s):
        for grp, ids in zip((self.cells, self.faces, self.hist), self.ids):
            for a, f in zip(grp, ids):
                s.download(f, out=a)
        self.flag = s.flag_ab

    def keep_vertex_pressure(self, s, ng):
        """The vertex pressure of the last stage (the lagged pf of
        update_rhsp), for a CPU run that continues from this state."""
        self.pv = s.download(ng.F_PV)

    def upload(self, s, flag):
        s.upload_state(*self.cells, self.faces, self.hist, flag)

    def copy_from(self, other):
        for a, b in zip(self.cells + self.faces + self.hist, other.cells + other.faces + other.hist):
            np.copyto(a, b)
        self.flag = other.flag


def timed_region(s, ng, torch, stream, steps, pg, local, profile=False):
    """K RK3 steps between CUDA events on the library's stream.  With
    profile=True the library also records an event pair around each of its
    kernel launches (per-kernel device time for the roofline); those events
    cost several per cent of the step, so the headline value comes from a
    region run without them."""
    s.prof_enable(profile)
    l0, it0 = s.counters()
    _, up0 = s.solver_counters()
    clocks = ClockSampler(local)
    clocks.start()
    torch.cuda.synchronize()
    barrier(pg)
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    worst = 0
    for _ in range(steps):
        rc, _ = s.step(3, 1)
        worst = max(worst, rc)
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier(pg)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    clk = clocks.stop()
    l1, it1 = s.counters()
    _, up1 = s.solver_counters()
    prof = s.prof_read() if profile else None
    s.prof_enable(False)
    return {"ms": ms, "clocks": clk, "launches": l1 - l0, "iters": it1 - it0, "updates": up1 - up0, "prof": prof,
            "status": worst}


# Kernels that run once per BiCGSTAB iteration (their launches after the
# device-side stopping test return at once and move nothing), and the mixed
# solver's FP64 hand-over kernels, which act once per refinement update.
ITER_KERNELS = ("k_bicg_p", "k_bicg_spmv_v", "k_bicg_s", "k_bicg_spmv_t", "k_bicg_x", "k_in_pv", "k_in_st")
UPDATE_KERNELS = ("k_mix_update", "k_mix_scale")

# End-to-end replays of the timed steps; the median is reported.
E2E_REPLAYS = 3


def step_bytes(prof, iters, updates, steps, prisms, mixed):
    """Algorithmic bytes of the K steps of a region: every kernel's words per
    prism (WORDS, WORDS_MIXED) x 8 B x prisms x the times it did work --
    iterations for the iteration passes, FP64 updates for the hand-over
    kernels, launches for the rest (the kernels around the solve run once
    per stage; 'other' holds the RK combinations, 3 words per cell each).
    Returns (bytes per step, bytes per iteration, bytes per update, fixed
    bytes per step)."""
    words = dict(WORDS)
    if mixed:
        words.update(WORDS_MIXED)
        words["k_bicg_init"] = 2 + 2  # k_mix_init: rhsp, pf read; b, x written
    words["other"] = 3
    per_iter = sum(words[k] for k in ITER_KERNELS if k in words and prof.get(k, (0, 0))[0] > 0) * 8.0 * prisms
    per_upd = sum(words[k] for k in UPDATE_KERNELS if prof.get(k, (0, 0))[0] > 0) * 8.0 * prisms
    fixed = sum(words[k] * 8.0 * prisms * prof[k][0] for k in prof
                if k in words and k not in ITER_KERNELS and k not in UPDATE_KERNELS) / max(steps, 1)
    return fixed + (per_iter * iters + per_upd * updates) / max(steps, 1), per_iter, per_upd, fixed


def kernel_us(prof, iters, updates):
    """Average device time of each kernel per launch that did work, in us:
    per iteration for the iteration passes, per FP64 update for the
    hand-over kernels, per launch for the rest.  The idle launches of the
    solver loops (a few us each) are included in the totals."""
    out = {}
    for k, (n, ms) in prof.items():
        if not n:
            continue
        real = iters if k in ITER_KERNELS else updates if k in UPDATE_KERNELS else n
        if real:
            out[k] = round(ms * 1e3 / real, 2)
    return out


def roofline(prof, iters, prisms, mixed, fp64_peak=None, spmv="stored"):
    hbm_peak, peak_kind = load_peaks()
    words = dict(WORDS)
    if mixed:
        words.update(WORDS_MIXED)
    dom = max((k for k in prof if k in words), key=lambda k: prof[k][1])
    n_launch, dom_ms = prof[dom]
    # solver passes run in chunks and return at once after the stopping test
    # fired: count the iterations that did work, not the launches
    real = iters if (dom.startswith("k_bicg_") or dom.startswith("k_in_")) and dom != "k_bicg_init" else n_launch
    bpl = words[dom] * 8.0 * prisms
    achieved = bpl * real / (dom_ms / 1e3) / 1e9 if dom_ms > 0 else 0.0
    traffic = None
    tpath = os.path.join(REPO, "profiles", "ncu_traffic.json")
    if os.path.exists(tpath):
        with open(tpath) as fh:
            tr = json.load(fh).get("mixed" if mixed else "fp64", {})
        if dom in tr:
            traffic = tr[dom] * prisms
    fl = None if mixed else FLOPS[spmv].get(dom)
    total = sum(v[1] for v in prof.values())
    shares = {k: round(v[1] / max(total, 1e-12), 4) for k, v in prof.items() if v[0]}
    roof = {"bound": "hbm", "kernel": dom,
            "region": "K steps after the timed region, CUDA event pair around each launch on the library's stream", "achieved": round(achieved, 1), "peak": hbm_peak, "unit": "GB/s",
            "frac": round(achieved / hbm_peak, 4), "peak_kind": peak_kind, "traffic": traffic,
            "algorithmic_bytes_per_launch": bpl, "avg_launch_ms": dom_ms / max(real, 1),
            "fp64_tflops": (round(fl * prisms * real / (dom_ms / 1e3) / 1e12, 3) if fl and dom_ms > 0 else None)}
    if roof["fp64_tflops"] is not None and fp64_peak:
        # the FP64 passes are bound by min(HBM, FP64 issue): both fractions
        roof["fp64_peak_tflops"] = round(fp64_peak, 3)
        roof["fp64_peak_kind"] = "measured in this run (nsmp_probe_fp64_fma, FMA chains, CUDA events)"
        roof["fp64_frac"] = round(roof["fp64_tflops"] / fp64_peak, 4)
        roof["bound"] = "fp64" if roof["fp64_frac"] > roof["frac"] else "hbm"
    return roof, shares, total


def run_ours(args):
    import torch

    import nsmp_gb300 as ng

    world, rank, local, pg = dist_setup()
    torch.cuda.set_device(local)
    nx, ny, layers, dt = WORKLOADS[args.workload]
    prisms = 2 * nx * ny * layers
    mesh = ng.make_mesh(nx, ny)
    precs = ["fp64", args.mixed_form] if args.precision == "both" else [args.precision]
    head = precs[-1]
    res, solvers = {}, {}
    snap = u_end = None
    fp64_peak, _ = ng.probe_fp64_fma(local)
    for prec in precs:
        prm = ng.channel_params(nx, ny, layers, dt, device=local,
                                precision=PRECISIONS[prec](ng))
        s = ng.Solver(prm, mesh)
        if prec == "fp64" and args.fp64_spmv == "matrix-free":
            s.set_fp64_spmv(True)
        u0, v0, w0, p0 = ng.initial_channel(prm, s.ncell, seed=1)
        s.user_initial(u0, v0, w0, p0)
        stream = torch.cuda.ExternalStream(s.stream)
        for _ in range(args.warmup):
            rc, _ = s.step(3, 1)
            if rc < 0:
                raise RuntimeError(f"warm-up step failed: {rc}")
        if prec == head:  # the state the timed steps start from, for the end-to-end replay
            snap = StateBuffers(torch, ng, s, prm)
            snap.download(s)
            snap.keep_vertex_pressure(s, ng)
        r = timed_region(s, ng, torch, stream, args.steps, pg, local)
        if prec == head:
            u_end = s.download(ng.F_U)
        r["ms_max"] = max_over_ranks(pg, r["ms"])
        r["value"] = job_value(world, prisms, args.steps, r["ms_max"])
        # per-kernel device times over K further steps of the same run
        rp = timed_region(s, ng, torch, stream, args.steps, pg, local, profile=True)
        r["prof"], r["prof_ms"], r["prof_iters"] = rp["prof"], rp["ms"], rp["iters"]
        r["kernel_us"] = kernel_us(rp["prof"], rp["iters"], rp["updates"])
        r["roof"], r["shares"], r["busy_ms"] = roofline(rp["prof"], rp["iters"], prisms, prec != "fp64",
                                                        fp64_peak, spmv=args.fp64_spmv)
        # whole step: the timed region's iterations and FP64 updates with the
        # per-kernel bytes of the profiled region
        _, b_it, b_up, b_fix = step_bytes(rp["prof"], rp["iters"], rp["updates"], args.steps, prisms,
                                          prec != "fp64")
        bstep = b_fix + (b_it * r["iters"] + b_up * r["updates"]) / args.steps
        hbm_peak, _ = load_peaks()
        r["roof"]["step_bytes"] = bstep
        r["roof"]["step_achieved"] = round(bstep / (r["ms_max"] / args.steps / 1e3) / 1e9, 1)
        r["roof"]["step_frac"] = round(bstep / (r["ms_max"] / args.steps / 1e3) / 1e9 / hbm_peak, 4)
        res[prec] = r
        solvers[prec] = (s, stream, prm)
    s, stream, prm = solvers[head]
    r = res[head]

    if args.profile_run:
        if rank == 0:
            print(json.dumps({"metric": "Mcell-steps/s", "value": r["value"], "profile_run": True,
                              "precision": head, "kernel_share": r["shares"], "kernel_us": r["kernel_us"],
                              "bicgstab_iters_per_stage": r["iters"] / (3.0 * args.steps)}), flush=True)
        for sv in solvers.values():
            sv[0].close()
        return 0

    # mixed vs FP64 after the same W + K steps from the same initial state
    cmp = None
    if len(res) == 2:
        a, b = solvers[head][0], solvers["fp64"][0]
        n0 = prm["n0"]
        cmp = {f"rel_l2_{nm}": float(np.linalg.norm(a.download(f)[:n0, 1:-1] - b.download(f)[:n0, 1:-1]) /
                                     np.linalg.norm(b.download(f)[:n0, 1:-1]))
               for nm, f in (("u", ng.F_U), ("v", ng.F_V), ("w", ng.F_W), ("p", ng.F_P))}
        da, db = a.mass_diag(), b.mass_diag()
        cmp["max_div_mixed"], cmp["max_div_fp64"] = float(da[1]), float(db[1])
        cmp["speedup"] = res[head]["value"] / res["fp64"]["value"]
        cmp["mixed_form"] = head
        cmp["after_steps"] = args.warmup + 2 * args.steps

    # ---- end to end: the timed steps replayed through the C-ABI -------------
    # From the state the timed region started from, every step uploads its
    # full input state from pinned host memory, steps, and downloads its full
    # output state, which is the next step's input.  The K steps are those of
    # the timed region, so the solver work is the same and the copies are
    # what is added; the replay ends on the timed region's final u, bit for
    # bit, when upload and download are exact.  The replay runs E2E_REPLAYS
    # times and the median wall-clock time is reported: the host cores are
    # shared, and a single replay of a few steps has read 4-25 ms a step of
    # copy overhead for about 7 ms of copies.  The replays ping-pong between
    # two buffers of their own, so `snap` stays the timed region's start
    # state for the CPU baseline below.
    st_a = StateBuffers(torch, ng, s, prm)
    st_b = StateBuffers(torch, ng, s, prm)
    t_reps, e2e_exact = [], True
    for _ in range(E2E_REPLAYS):
        st_a.copy_from(snap)
        st_in, st_out, flag = st_a, st_b, snap.flag
        torch.cuda.synchronize()
        barrier(pg)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            st_in.upload(s, flag)
            s.step(3, 1)
            st_out.download(s)
            flag = st_out.flag
            st_in, st_out = st_out, st_in
        torch.cuda.synchronize()
        t_reps.append(max_over_ranks(pg, time.perf_counter() - t0))
        e2e_exact = e2e_exact and bool(np.array_equal(st_in.cells[0], u_end))
    t_e2e = float(np.median(t_reps))
    e2e_value = job_value(world, prisms, args.steps, t_e2e * 1e3)
    e2e_values = [round(job_value(world, prisms, args.steps, t * 1e3), 3) for t in t_reps]
    h2d = d2h = st_in.nbytes

    # ---- CPU baseline (rank 0, N = 1 only) ---------------------------------
    cpu = None
    if rank == 0 and world == 1 and not args.skip_cpu:
        nthreads = os.cpu_count() or 1
        t_cpu, cits = cpu_step_from_state(args, snap, nthreads)
        cpu = {"value": prisms / t_cpu / 1e6, "unit": "Mcell-steps/s", "cores": nthreads, "kind": "port",
               "cpu": cpu_model(), "bicgstab_iters_per_stage": cits,
               "sample": f"one full RK3 step ({t_cpu:.1f} s wall clock) of the oracle from the state the timed "
                         f"region started from: the first timed step's work"}

    if rank == 0:
        line = {
            "metric": "Mcell-steps/s", "value": r["value"], "unit": "Mcell-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms_max"] / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if head == "fp64" else "f32+f64",
            "data": "synthetic (seeded mesh and initial state; no dataset exists for this path)",
            "config": {"workload": workload_desc(args.workload), "prisms": prisms, "precision": head,
                       "integrator": "SSP-RK3 of the reference stage",
                       "parallelism": "replicas" if world > 1 else "1 GPU",
                       "l2": "inputs larger than L2 (working set > 2 GB), no flush",
                       "bicgstab_iters_per_stage": round(r["iters"] / (3.0 * args.steps), 1)},
            "roofline": r["roof"],
            "kernel_share": r["shares"],
            "kernel_us": r["kernel_us"],
            "device_busy_frac": round(r["busy_ms"] / max(r["prof_ms"], 1e-9), 4),
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": "Mcell-steps/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "steps": args.steps,
                    "replay": "the timed steps from their start state, full state up and down each step; "
                              f"median of {E2E_REPLAYS} replays (host wall clock)",
                    "replay_values": e2e_values,
                    "replay_matches_timed_u_bitwise": e2e_exact},
            "clocks": r["clocks"],
            "gpu_launches": r["launches"],
            "status": r["status"],
        }
        if "fp64" in res and head != "fp64":
            f = res["fp64"]
            line["fp64"] = {"value": f["value"], "ms_per_step": f["ms_max"] / args.steps, "spmv": args.fp64_spmv,
                            "bicgstab_iters_per_stage": round(f["iters"] / (3.0 * args.steps), 1),
                            "roofline": f["roof"], "kernel_share": f["shares"], "kernel_us": f["kernel_us"],
                            "gpu_launches": f["launches"],
                            "clocks": f["clocks"]}
        if cmp:
            line["mixed_vs_fp64"] = cmp
        print(json.dumps(line), flush=True)
    for sv in solvers.values():
        sv[0].close()
    if pg is not None:
        pg.destroy_process_group()
    return 0


def run_accuracy(args):
    """Mixed forms vs FP64 after N RK3 steps from the same initial state:
    relative L2 of u, v, w, p over the interior and glob_cfl of each run
    (max |div| is the reference's "Maxim flux").  Arms: FP64; mixed (FP32
    Krylov + FP64 refinement, FP64 stage); mixed_f32 (the same with the stage
    right-hand side in FP32); and, with --accuracy-compat0, the mixed form
    with the reference's quirks corrected (ref_bug_compat = 0)."""
    import nsmp_gb300 as ng

    nx, ny, layers, dt = WORKLOADS[args.workload]
    mesh = ng.make_mesh(nx, ny)
    arms = [("fp64", ng.FP64, 1), ("mixed", ng.MIXED, 1), ("mixed_f32", ng.MIXED_F32, 1)]
    if args.accuracy_compat0:
        arms.append(("mixed_compat0", ng.MIXED, 0))
    sol = {}
    clocks = ClockSampler(0)
    clocks.start()
    for name, prec, compat in arms:
        prm = ng.channel_params(nx, ny, layers, dt, precision=prec, ref_bug_compat=compat)
        s = ng.Solver(prm, mesh)
        u0, v0, w0, p0 = ng.initial_channel(prm, s.ncell, seed=1)
        s.user_initial(u0, v0, w0, p0)
        worst = 0
        it0, _ = s.solver_counters()
        t0 = time.perf_counter()
        for _ in range(args.accuracy_steps):
            rc, _ = s.step(3, 1)
            worst = max(worst, rc)
        wall = time.perf_counter() - t0
        it1, _ = s.solver_counters()
        sol[name] = {"fields": {nm: s.download(f)[:prm["n0"], 1:-1] for nm, f in
                                (("u", ng.F_U), ("v", ng.F_V), ("w", ng.F_W), ("p", ng.F_P))},
                     "cfl": s.cfl_diag(), "status": worst, "s": wall,
                     "its_per_stage": (it1 - it0) / (3.0 * max(args.accuracy_steps, 1))}
        s.close()
    clk = clocks.stop()
    b = sol["fp64"]
    out = {"accuracy": "mixed forms vs fp64", "workload": workload_desc(args.workload),
           "steps": args.accuracy_steps}
    for name in sol:
        a = sol[name]
        d = {"status": a["status"], "wall_s": round(a["s"], 1), "bicgstab_iters_per_stage": round(a["its_per_stage"], 1),
             "max_abs_div": abs(a["cfl"]["flux_max"]), "cfl": a["cfl"]}
        if name != "fp64":
            for nm in ("u", "v", "w", "p"):
                d[f"rel_l2_{nm}"] = float(np.linalg.norm(a["fields"][nm] - b["fields"][nm]) /
                                          np.linalg.norm(b["fields"][nm]))
            d["max_abs_div_diff_vs_fp64"] = abs(abs(a["cfl"]["flux_max"]) - abs(b["cfl"]["flux_max"]))
        out[name] = d
    out["clocks"] = clk
    print(json.dumps(out), flush=True)
    return 0


def run_adjoint_bench(args):
    """Adjoint/forward cost: N FP64 RK3 steps forward, then the same N steps
    through nsmp_adjoint (forward sweep with checkpoints every K steps,
    segment recomputation and the reverse sweep) with a seeded body force."""
    import torch

    import nsmp_gb300 as ng

    nx, ny, layers, dt = WORKLOADS[args.workload]
    prisms = 2 * nx * ny * layers
    mesh = ng.make_mesh(nx, ny)
    mixed = args.precision in ("mixed", "mixed_f32")
    prm = ng.channel_params(nx, ny, layers, dt, precision=(ng.MIXED if mixed else ng.FP64))
    s = ng.Solver(prm, mesh)
    u0, v0, w0, p0 = ng.initial_channel(prm, s.ncell, seed=1)
    s.user_initial(u0, v0, w0, p0)
    n0, nz = prm["n0"], prm["nz"]
    fx = np.zeros((n0, nz), order="F")
    fx[:, 1:-1] = 0.01 * np.random.default_rng(2).standard_normal((n0, nz - 2))
    cells = [s.download(f) for f in (ng.F_U, ng.F_V, ng.F_W, ng.F_P)]
    faces = [s.download(f) for f in (ng.F_U1FACE, ng.F_U2FACE, ng.F_U3FACE, ng.F_UTFACE, ng.F_UBFACE)]
    hist = [s.download(f) for f in (ng.F_RHSU, ng.F_RHSV, ng.F_RHSW)]
    stream = torch.cuda.ExternalStream(s.stream)
    N, K = args.adjoint_steps, args.ckpt

    def timed(fn):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        out = fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1e3, out

    s.set_body_force(fx)
    s.set_adjoint_budget(args.adjoint_budget_gb * 1e9)
    s.upload_state(*cells, faces, hist, 0)
    s.step(3, 1)  # warm-up (first-use allocations, occupancy queries)
    s.upload_state(*cells, faces, hist, 0)
    l0, i0 = s.counters()
    clocks = ClockSampler(0)
    clocks.start()
    t_fwd, _ = timed(lambda: [s.step(3, 1) for _ in range(N)])
    clk_fwd = clocks.stop()
    l1, i1 = s.counters()
    s.upload_state(*cells, faces, hist, 0)
    # device memory in use while the adjoint runs (sampled every 50 ms)
    free_min = [torch.cuda.mem_get_info()[0]]
    total = torch.cuda.mem_get_info()[1]
    stop = threading.Event()

    def poll():
        while not stop.is_set():
            free_min[0] = min(free_min[0], torch.cuda.mem_get_info()[0])
            time.sleep(0.05)

    th = threading.Thread(target=poll, daemon=True)
    th.start()
    clocks = ClockSampler(0)
    clocks.start()
    t_adj, (J, grad, rc) = timed(lambda: s.adjoint(N, K, fx))
    stop.set()
    th.join()
    clk_adj = clocks.stop()
    l2, i2 = s.counters()
    ncf = n0 * nz
    nseg = -(-N // K)
    dev_bytes = 8 * ncf * (30 + 9 * (nseg + 1) + 24 * K) + 8 * 3 * prisms * N
    line = {"metric": "adjoint/forward time", "value": t_adj / t_fwd, "unit": "x", "higher_is_better": False,
            "workload": workload_desc(args.workload), "prisms": prisms, "steps": N, "ckpt_every": K,
            "forward_s": t_fwd, "adjoint_s": t_adj, "J": J, "grad_l2": float(np.linalg.norm(grad)),
            "status": rc, "bicgstab_iters_forward": i1 - i0, "bicgstab_iters_adjoint_call": i2 - i1,
            "adjoint_device_bytes": dev_bytes,
            "adjoint_device_bytes_note": "work buffers of nsmp_adjoint (30 cell fields + 9 per checkpoint + 24 per "
                                         "step of one segment + the pressure tape, 3 solutions per step), on top "
                                         "of the context's forward state",
            "peak_device_bytes_in_use": total - free_min[0],
            "segment_budget_bytes": args.adjoint_budget_gb * 1e9 or "80% of free memory",
            "gpu_launches": l2 - l1, "dtype": "f32+f64" if mixed else "f64",
            "precision": "mixed forward and adjoint solves, FP64 adjoint accumulation" if mixed else "fp64",
            "clocks": {"forward": clk_fwd, "adjoint": clk_adj}}
    print(json.dumps(line), flush=True)
    s.close()
    return 0


def run_aux(args):
    """The kernels around the path, timed on the library's stream at the
    workload's size: turbulence-statistics sampling and plane sums, vertex
    output (tagdir 3) with its download, and the full restart state up and
    down.  Bytes are the compulsory ones: statistics sampling reads u, v, w,
    p, nu_t and updates 12 FP64 sums per cell value (232 B); the plane sums
    read 9 sums per interior prism (72 B); vertex output writes one value per
    vertex and layer (8 B, stencil reads served by cache) and copies it to
    pinned host memory; the state copies move the 12 arrays of the restart
    state; glob_cfl reads the five face fluxes and u, v, w (64 B a prism)."""
    import torch

    import nsmp_gb300 as ng

    nx, ny, layers, dt = WORKLOADS[args.workload]
    mesh = ng.make_mesh(nx, ny)
    prm = ng.channel_params(nx, ny, layers, dt, precision=ng.MIXED)
    s = ng.Solver(prm, mesh)
    u0, v0, w0, p0 = ng.initial_channel(prm, s.ncell, seed=1)
    s.user_initial(u0, v0, w0, p0)
    for _ in range(max(1, args.warmup)):
        s.step(3, 1)
    st = torch.cuda.ExternalStream(s.stream)
    k = max(3, args.steps)

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(k):
            fn()
        e1.record(st)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / k

    s.stats_reset()
    sb = StateBuffers(torch, ng, s, prm)
    sb.download(s)
    vbuf = torch.empty((s.nz - 1, s.nvert), dtype=torch.float64, pin_memory=True).numpy().T
    ncv, nint, nvo = s.n0 * s.nz, s.n0 * (s.nz - 2), s.nvert * (s.nz - 1)
    legs = {
        "stats_sample": (s.stats_sample, 232 * ncv),
        "stats_plane": (s.stats_plane, 72 * nint),
        "vertex_out_tagdir3_with_download": (lambda: s.download_vertex(ng.F_U, 3, out=vbuf), 8 * nvo),
        "upload_state": (lambda: sb.upload(s, sb.flag), sb.nbytes),
        "download_state": (lambda: sb.download(s), sb.nbytes),
        "cfl_diag": (s.cfl_diag, 8 * 8 * nint),
    }
    out = {"aux": "kernels around the path, CUDA events on the library's stream",
           "workload": workload_desc(args.workload), "calls": k}
    clocks = ClockSampler(0)
    clocks.start()
    for name, (fn, nbytes) in legs.items():
        ms = timed(fn)
        out[name] = {"ms": round(ms, 4), "bytes": int(nbytes), "GBps": round(nbytes / (ms / 1e3) / 1e9, 1)}
    out["clocks"] = clocks.stop()
    s.close()
    print(json.dumps(out), flush=True)
    return 0


def run_fp64_peak(args):
    """FP64 FMA issue rate of the device (the roof of the FP64 solver passes),
    measured over several repetitions with clocks sampled."""
    import nsmp_gb300 as ng
    clocks = ClockSampler(0)
    clocks.start()
    runs = [ng.probe_fp64_fma(0, 200000) for _ in range(max(3, args.steps))]
    clk = clocks.stop()
    best = max(t for t, _ in runs)
    print(json.dumps({"fp64_fma_peak": "FP64 FMA chains, full-device grid, CUDA events", "tflops_best": best,
                      "tflops_median": float(np.median([t for t, _ in runs])),
                      "ms_per_run": [round(m, 3) for _, m in runs], "clocks": clk}), flush=True)
    return 0


def run_setup(args):
    """The setup of the workload's mesh: host path (nsmp_geometry) against
    the path nsmp_create runs, with its floating-point geometry on the GPU
    (nsmp_geometry_device), wall clock over several repetitions."""
    import nsmp_gb300 as ng
    nx, ny, layers, dt = WORKLOADS[args.workload]
    mesh = ng.make_mesh(nx, ny)
    prm = ng.channel_params(nx, ny, layers, dt)
    ng.geometry(prm, mesh, ng.G_XC, device=True)  # first use: context creation, module load
    clocks = ClockSampler(0)
    clocks.start()
    out = {"setup": "geometry + topology + device tables of the workload's mesh", "workload": workload_desc(args.workload)}
    for name, dev in (("host_s", False), ("device_s", True)):
        ts = []
        for _ in range(max(3, args.steps)):
            t0 = time.perf_counter()
            ng.geometry(prm, mesh, ng.G_XC, device=dev)
            ts.append(time.perf_counter() - t0)
        out[name] = round(float(np.median(ts)), 4)
    out["clocks"] = clocks.stop()
    print(json.dumps(out), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="config2", choices=sorted(WORKLOADS))
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--ref-threads", type=int, default=0,
                    help="host threads of the --impl reference arm (0: all cores)")
    ap.add_argument("--setup", action="store_true",
                    help="instead of timing the step: the mesh setup, host path against device path")
    ap.add_argument("--fp64-peak", action="store_true",
                    help="instead of timing the step: the device's FP64 FMA rate with clocks sampled")
    ap.add_argument("--precision", default="both", choices=["fp64", "mixed", "mixed_f32", "both"])
    ap.add_argument("--fp64-spmv", default="stored", choices=["stored", "matrix-free"],
                    help="couplings of the FP64 arm's BiCGSTAB products")
    ap.add_argument("--mixed-form", default="mixed", choices=["mixed", "mixed_f32"],
                    help="the mixed-precision arm of --precision both (the headline value)")
    ap.add_argument("--profile-run", action="store_true",
                    help="device-timed region only (no end-to-end leg, no CPU baseline), for ncu captures")
    ap.add_argument("--accuracy-steps", type=int, default=0,
                    help="instead of timing: run both precisions N RK3 steps and print mixed-vs-FP64 errors")
    ap.add_argument("--accuracy-compat0", action="store_true",
                    help="with --accuracy-steps: also run the mixed form with the reference's quirks corrected")
    ap.add_argument("--adjoint-steps", type=int, default=0,
                    help="instead of timing the forward: adjoint/forward cost over N FP64 RK3 steps")
    ap.add_argument("--ckpt", type=int, default=20, help="checkpoint spacing of --adjoint-steps")
    ap.add_argument("--adjoint-budget-gb", type=float, default=0.0,
                    help="device memory for the stage inputs of an adjoint segment (0: automatic)")
    ap.add_argument("--aux", action="store_true",
                    help="instead of timing the step: statistics, vertex output and state copies")
    args = ap.parse_args()
    if args.fp64_peak:
        return run_fp64_peak(args)
    if args.setup:
        return run_setup(args)
    if args.aux:
        return run_aux(args)
    if args.accuracy_steps > 0:
        return run_accuracy(args)
    if args.adjoint_steps > 0:
        return run_adjoint_bench(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
