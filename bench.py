"""Benchmark: cell-steps/s of the EllipsesInFlows time step on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--precision fp64|mixed] [--workload NAME]

One step is one full time step of the solver (dt decision + three RK stages
with the immersed-boundary exchange, the pressure projection, collisions and
the particle fixed point), i.e. src/main.c:71-77 of the reference. The metric
is cells x steps / wall time of the timed steps. The default workload is the
2048 x 4096 grid with 2048 ellipses (aspect ratio U[1,3], density ratio
U[1,1.2], Re 400, seeded placement); inputs are synthetic.

--impl ours        the CUDA library through its C ABI (value: device-timed
                   steps with the state resident in HBM; e2e: the same steps
                   with the state copied host->device before and device->host
                   after every step through the public API).
--impl reference   the CPU restatement of the reference algorithm
                   (oracle/port, OpenMP over all host threads) on the same
                   workload; reported as the reference arm.

Under torchrun with N > 1 every rank advances an independent replica on its
own GPU (the path has no data exchange between suspensions); value is the
sum over ranks, timed as the maximum over ranks.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

MEASURED = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0

# Algorithmic DRAM bytes per cell for one launch of each streaming kernel
# (double precision storage; read + write of every field the kernel touches once).
#   predictor: R ux uy p srcB_x srcB_y, W srcA_x srcA_y ux' uy'       9 words
#   correct:   R ux uy dux duy psi p, W ux uy p                        9 words
#   dct2:      R ux uy dux duy, W qhat                                 5 words
#   tdm:       R qhat, W qhat                                          2 words
#   dct3:      R qhat, W psi                                           2 words
#   decide_dt: R ux uy                                                 2 words
#   gather:    W dux duy                                               2 words
# Algorithmic bytes per cell of one launch of the streaming kernels that time one
# kernel per timer scope: predictor (u, v, p, srcB read; srcA, u', v' written),
# projection (u, v, p read and written, psi and the IBM field read), DCT-II (u, v and
# the IBM field read, the transformed row written), DCT-III (solution read, psi
# written). The mixed form keeps the IBM field in single precision and solves the
# Poisson equation in two single-precision passes: DCT-II of the first pass reads u,
# v and the IBM field (24 B) and writes the right-hand side as a float pair (8 B) and
# its transform (4 B); that of the second reads the pair and psi1 (12 B) and writes
# its transform (4 B): 26 B per launch on average; each DCT-III reads the block
# solution (4 B) and writes psi1 or psi2 (4 B).
HBM_BYTES = {
    "fp64": {"predictor": 72, "correct": 72, "poisson_dct2": 40, "poisson_dct3": 16},
    "mixed": {"predictor": 56, "correct": 64, "poisson_dct2": 26, "poisson_dct3": 8},
}

# DRAM bytes (read + write) per launch from ncu captures of the mixed form at
# 2048 x 4096, with the source file each kernel is built from and that file's SHA-1 at
# the capture: the roofline's `traffic` reports a stored value only while the source is
# unchanged (otherwise null, marked stale)
# (the DCT entries are the mean of the two passes' launches)
_KPROF = "profiles/kernels_suspension_2048x4096_mixed.md"
_FLUID_SHA = "2afdd44547a4d7470dac4d752b3dbe6f0c52ab4e"
_POISSON_SHA = "7b859e57013264f78a70fa51d00e837ea3f919cd"
NCU_TRAFFIC = {
    ("mixed", 2048, 4096): {
        "predictor": (494.9e6, "fluid.cu", _FLUID_SHA, _KPROF),
        "correct": (552.2e6, "fluid.cu", _FLUID_SHA, _KPROF),
        "poisson_dct2": (195.5e6, "poisson.cu", _POISSON_SHA, _KPROF),
        "poisson_dct3": (33.7e6, "poisson.cu", _POISSON_SHA, _KPROF),
    },
}

# Algorithmic bytes per cell-step of the whole step (three RK stages), the formula of
# the double-precision algorithm: the sum over the streaming passes of one stage
# (predictor 9, IBM field update 4, right-hand side and DCT-II 3, tridiagonal solve 2,
# DCT-III 2, projection and pressure 7 words) times three stages, 81 words of 8 bytes;
# the mixed form keeps the explicit terms in single precision (6 words of 4 bytes
# fewer per stage)
STEP_BYTES = {"fp64": 81 * 8, "mixed": 81 * 8 - 3 * 6 * 4}

# Measured single-precision FMA throughput of this GPU (an FMA-chain probe, 2 flops per
# FMA), the denominator of the indicator kernel's pipe roofline
FP32_TFLOPS_MEASURED = 69.9

# FP32 flops (FFMA counted twice, FADD and FMUL once) of the mixed-form indicator kernel
# per normal-foot evaluation (all of the launch's flops, the far-cell tests and sums
# included, over its evaluations): 9.03e8 flops in the captured launch of k_ibm_work_f
# over the 2.86e6 evaluations that launch counts at this workload (value, source)
INDICATOR_FLOPS_PER_EVAL = (316, "ncu capture of k_ibm_work_f, " + "profiles/kernels_suspension_2048x4096_mixed.md")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--no-fp64-leg", action="store_true")
    ap.add_argument("--workload", default="mixed_target",
                    choices=["mixed_target", "poiseuille", "couette_circle", "batch_c5", "adjoint_couette",
                             "adjoint_large"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-log-timing", action="store_true",
                    help="skip timing the logging reductions (keeps launch lists to the step's kernels)")
    ap.add_argument("--accuracy-steps", type=int, default=None,
                    help="steps of the mixed-vs-double comparison (default: the workload's run length)")
    return ap.parse_args()


def make_case(name):
    from ellipsesinflows_gb300 import cases
    return cases.CONFIGS[name]()


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region.

    Samples carry nvidia-smi's own timestamp; `begin()` and `end()` mark the timed region
    on the same clock, and the summary keeps the samples inside it (all samples when the
    region was not marked, the nearest one when it was shorter than the interval)."""

    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    INTERVAL_MS = 20

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []
        self.t0 = self.t1 = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", str(self.INTERVAL_MS)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            # the sampler is running before the region starts
            deadline = time.time() + 3.0
            while not self.lines and time.time() < deadline and self.proc.poll() is None:
                time.sleep(0.01)
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def begin(self):
        self.t0 = time.time()

    def end(self):
        self.t1 = time.time()

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    @staticmethod
    def _stamp(text):
        import datetime
        try:
            return datetime.datetime.strptime(text, "%Y/%m/%d %H:%M:%S.%f").timestamp()
        except ValueError:
            return None

    def summary(self):
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        rows = []
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 10:
                continue
            try:
                rows.append((self._stamp(parts[0]), float(parts[2]), float(parts[3]),
                             [name for k, name in enumerate(names) if parts[6 + k].lower().startswith("active")]))
            except ValueError:
                continue
        where = "all samples"
        if self.t0 is not None and self.t1 is not None and rows:
            inside = [r for r in rows if r[0] is not None and self.t0 <= r[0] <= self.t1]
            if inside:
                rows, where = inside, "timed region"
            else:
                mid = 0.5 * (self.t0 + self.t1)
                stamped = [r for r in rows if r[0] is not None]
                if stamped:
                    rows = [min(stamped, key=lambda r: abs(r[0] - mid))]
                    where = "nearest sample (region shorter than the %d ms interval)" % self.INTERVAL_MS
        sm = [r[1] for r in rows]
        reasons = sorted({n for r in rows for n in r[3]})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": rows[-1][2] if rows else None,
                "reasons": reasons, "samples": len(sm), "window": where}


def peaks():
    try:
        with open(MEASURED) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return FALLBACK_HBM_GBS, "fallback"


def dist_init(gpus):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if os.environ.get("EIF_BENCH_BACKEND", "nccl") == "nccl" else "gloo"
        dist.init_process_group(backend=backend)
        pg = dist
    return world, rank, local, pg


def barrier(pg, device=None):
    if pg is not None:
        if device is not None:
            pg.barrier(device_ids=[device])
        else:
            pg.barrier()


def max_over_ranks(pg, value, device):
    if pg is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device="cuda:%d" % device if device is not None else "cpu")
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def workload_config(case, world):
    """The config object both arms print (the same keys and values for the same workload)."""
    return {"workload": case.name, "itot": case.itot, "jtot": case.jtot, "n_particles": case.n_particles,
            "Re": case.Re,
            "l2": "inputs larger than L2 (~%d MB of device state per step)" % (case.cells * 13 * 8 // 10**6),
            "parallelism": "replicas" if world > 1 else "single GPU"}


def timed_advance(sim, stream, steps, pg, device):
    """Device time (ms, max over ranks) of `steps` steps of eif_advance, CUDA events on
    the library's stream, with a barrier and a synchronisation on both sides."""
    import torch
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier(pg, device)
    torch.cuda.synchronize()
    start.record(stream)
    sim.advance(steps)
    stop.record(stream)
    torch.cuda.synchronize()
    barrier(pg, device)
    return max_over_ranks(pg, start.elapsed_time(stop), device)


def run_ours(args, world, rank, local, pg):
    import torch
    from ellipsesinflows_gb300 import PREC_FP64, PREC_MIXED, Simulation, build
    build.build()
    torch.cuda.set_device(local)
    case = make_case(args.workload)
    prec = PREC_MIXED if args.precision == "mixed" else PREC_FP64
    sim = Simulation.from_case(case, precision=prec, device=local)
    stream = torch.cuda.ExternalStream(sim._fn("stream")(sim.ctx), device=local)
    for _ in range(args.warmup):
        sim.advance(1)
    sim.synchronize()
    sub0 = sim.counters()["substeps"]
    # ---- device-timed region: state resident in HBM, one CUDA graph per step ----
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        barrier(pg, local)
        torch.cuda.synchronize()
        clk.begin()
        start.record(stream)
        sim.advance(args.steps)
        stop.record(stream)
        torch.cuda.synchronize()
        clk.end()
        barrier(pg, local)
    ms = start.elapsed_time(stop)
    ms = max_over_ranks(pg, ms, local)
    substeps_timed = (sim.counters()["substeps"] - sub0) / (3.0 * args.steps)
    # ---- per-kernel device times: a separate pass with the library's event timer
    # (host-driven launches, same kernels), with the indicator work counted ----
    prof_steps = max(1, min(args.steps, 3))
    cnt0 = sim.counters()
    memo0 = sim.memo_count() if precision_is_mixed(args) else 0
    sim._call("profile_reset", sim.ctx)
    sim._call("profile_enable", sim.ctx, 1)
    sim.advance(prof_steps)
    sim.synchronize()
    sim._call("profile_enable", sim.ctx, 0)
    cnt1 = sim.counters()
    prof = profile_entries(sim)
    counts = {k: cnt1[k] - cnt0[k] for k in cnt1}
    counts["memo_tasks"] = (sim.memo_count() - memo0) if precision_is_mixed(args) else 0
    # ---- the logging reductions of one log event (divergence, momentum, energy) on
    # the device, against pulling the two velocity fields for a host reduction ----
    log_ms = None
    if not args.no_log_timing:
        sim.log_quantities()
        t0 = time.perf_counter()
        for _ in range(5):
            sim.log_quantities()
        log_ms = (time.perf_counter() - t0) * 1e3 / 5
    # ---- end-to-end through the public API with host buffers ----
    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(sim, case, args.steps, pg, local)
    tiles = sim.tiles()
    sim.close()
    # ---- the double-precision form and the accuracy of the mixed form against it ----
    accuracy = fp64 = developed = None
    if prec == PREC_MIXED and not args.no_fp64_leg:
        fp64, accuracy, developed = accuracy_leg(args, case, local, pg, world)
    cells = case.cells
    value = world * cells * args.steps / (ms / 1e3)
    hbm, hbm_src = peaks()
    roof = roofline(prof, cells, hbm, hbm_src, args.precision, (case.itot, case.jtot))
    # kernels launched in the timed region: the same kernels per step as the profiled pass
    launches = int(round(sum(e["launches"] for e in prof) * args.steps / prof_steps))
    out = {
        "metric": "cell-steps/s", "value": value, "unit": "cell-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if prec == PREC_FP64 else "f32+f64",
        "data": "synthetic (seeded ellipse placement, fluid at rest)",
        "config": workload_config(case, world),
        "precision": args.precision,
        "e2e": e2e, "roofline": roof, "gpu_launches": launches,
        "step_roofline": {"bytes_per_cell_step": STEP_BYTES[args.precision],
                          "achieved": STEP_BYTES[args.precision] * value / world / 1e9, "peak": hbm,
                          "unit": "GB/s", "frac": STEP_BYTES[args.precision] * value / world / 1e9 / hbm,
                          "what": "algorithmic bytes of the whole step's streaming passes x cell-steps/s"},
        "indicator": indicator_roofline(prof, counts, prof_steps),
        "substeps_per_stage": substeps_timed,
        "fp64_form": fp64, "accuracy_vs_fp64": accuracy, "developed_window": developed,
        "log_reductions_ms": log_ms,
        "clocks": clk.summary(),
        "tiles": tiles,
        "kernels_per_step": {e["name"]: {"launches": round(e["launches"] / prof_steps, 2),
                                         "ms": round(e["ms"] / prof_steps, 4)} for e in prof},
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(args, case)
    return out, rank


def time_batch(sims, mode, args, pg, local, clk=None):
    """device time (ms, max over ranks) of args.steps batch steps of sims after
    args.warmup, with the sub-iteration loops in stage kernels or per branch (mode)"""
    import torch
    from ellipsesinflows_gb300 import Batch
    if mode == "branches":
        os.environ["EIF_BATCH_SUBITER"] = "branches"
    else:
        os.environ.pop("EIF_BATCH_SUBITER", None)
    try:
        batch = Batch(sims)
    finally:
        os.environ.pop("EIF_BATCH_SUBITER", None)
    stream = torch.cuda.ExternalStream(batch.stream(), device=local)
    batch.advance(args.warmup)
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier(pg, local)
    torch.cuda.synchronize()
    if clk:
        clk.begin()
    start.record(stream)
    batch.advance(args.steps)
    stop.record(stream)
    torch.cuda.synchronize()
    if clk:
        clk.end()
    barrier(pg, local)
    batch.close()
    return max_over_ranks(pg, start.elapsed_time(stop), local)


def run_batch(args, world, rank, local, pg):
    """64 independent suspensions of uneven sizes (cases.batch_c5) advanced by one
    step graph per step (eif_batch_*): aggregate cell-steps/s, with the particle
    sub-iterations of all suspensions in one persistent kernel per RK stage; against
    the same batch with a sub-iteration loop per suspension in its graph branch, and
    against the suspensions advanced one after another with eif_advance."""
    import torch
    from ellipsesinflows_gb300 import PREC_FP64, PREC_MIXED, Simulation, build, cases
    build.build()
    torch.cuda.set_device(local)
    cs = cases.batch_c5()
    prec = PREC_MIXED if args.precision == "mixed" else PREC_FP64
    cells = sum(c.cells for c in cs)
    with ClockSampler(local) as clk:
        sims = [Simulation.from_case(c, precision=prec, device=local) for c in cs]
        ms = time_batch(sims, "stage_kernels", args, pg, local, clk)
    for s in sims:
        s.close()
    sims = [Simulation.from_case(c, precision=prec, device=local) for c in cs]
    br_ms = time_batch(sims, "branches", args, pg, local)
    for s in sims:
        s.close()
    sims = [Simulation.from_case(c, precision=prec, device=local) for c in cs]
    # the same suspensions one after another, each advanced the same steps with
    # eif_advance on its own stream, timed with CUDA events like the batch; the
    # separate time is the sum of the suspensions' device times
    sep_ms = 0.0
    for s in sims:
        st = torch.cuda.ExternalStream(s._fn("stream")(s.ctx), device=local)
        sep_ms += timed_advance(s, st, args.steps, pg, local)
    grids = sorted({"%dx%d" % (c.itot, c.jtot) for c in cs})
    out = {
        "metric": "cell-steps/s", "value": world * cells * args.steps / (ms / 1e3), "unit": "cell-steps/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if prec == PREC_FP64 else "f32+f64",
        "data": "synthetic (seeded ellipse placement, fluid at rest)",
        "config": {"workload": "batch_c5_%d" % len(cs), "suspensions": len(cs), "grids": grids,
                   "total_cells": cells, "n_particles_total": int(sum(c.n_particles for c in cs)),
                   "precision": args.precision, "l2": "inputs larger than L2 (~%d MB of device state)" % (cells * 13 * 8 // 10**6),
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "branches": {"value": world * cells * args.steps / (br_ms / 1e3), "unit": "cell-steps/s",
                     "ms_per_step": br_ms / args.steps,
                     "how": "the same batch with the sub-iteration loop of every suspension as a "
                            "conditional node in its own graph branch (EIF_BATCH_SUBITER=branches)"},
        "separate": {"value": cells * args.steps / (sep_ms / 1e3), "unit": "cell-steps/s",
                     "ms_per_step": sep_ms / args.steps,
                     "how": "the same suspensions advanced one after another with eif_advance, each "
                            "timed with CUDA events on its own stream; the sum of their device times"},
        "e2e": None, "roofline": None, "clocks": clk.summary(),
    }
    return out, rank


def run_adjoint(args, world, rank, local, pg):
    """Gradient of a loss of the state after K steps through the discrete adjoint
    (eif_adjoint_*, double-precision form, particles moving): per step one recorded
    forward step and one transposed step, i.e. the work of a checkpoint segment's
    recomputation and reverse sweep. value: cells x steps / time of (recorded
    forward + backward); cost_vs_forward: that time over the plain forward steps
    (eif_integrate with the same dt) on the same state."""
    import numpy as np
    import torch
    from ellipsesinflows_gb300 import Simulation, build
    build.build()
    torch.cuda.set_device(local)
    case = make_case(args.workload)
    sim = Simulation.from_case(case, device=local)
    ux, uy, p = case.fluid()
    uy = uy + getattr(case, "uy_offset", 0.0)
    sim.push_fluid(ux, uy, p)
    sim.dt = 0.5 * sim.decide_dt()
    k = args.steps
    sim.adjoint_begin(k)
    for _ in range(args.warmup):
        sim.integrate()
    state = sim.pull_fluid()[:3]
    rec = sim.pull_particles()

    def timed(fn):
        barrier(pg, local)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fn()
        torch.cuda.synchronize()
        barrier(pg, local)
        return max_over_ranks(pg, (time.perf_counter() - t0) * 1e3, local)

    with ClockSampler(local) as clk:
        fwd_ms = timed(lambda: [sim.integrate() for _ in range(k)])
        sim.push_fluid(*state)
        sim.push_particles(rec)
        rec_ms = timed(lambda: [sim.adjoint_forward(record=True) for _ in range(k)])
        sx, sy = sim.shapes()
        rng = np.random.default_rng(0)
        sim.adjoint_seed(rng.standard_normal(sx), rng.standard_normal(sy))
        bwd_ms = timed(lambda: [sim.adjoint_backward() for _ in range(k)])
    sim.adjoint_end()
    cells = case.cells
    out = {
        "metric": "cell-steps/s", "value": world * cells * k / ((rec_ms + bwd_ms) / 1e3), "unit": "cell-steps/s",
        "n_gpus": world, "steps": k, "warmup": args.warmup, "ms_per_step": (rec_ms + bwd_ms) / k,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded ellipse placement)",
        "config": {"workload": case.name, "itot": case.itot, "jtot": case.jtot, "n_particles": case.n_particles,
                   "what": "discrete adjoint, coupled particles: recorded forward + backward per step",
                   "l2": "state larger than L2" if cells * 8 * 13 > 129e6 else "state fits in L2",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "forward_ms_per_step": fwd_ms / k, "recorded_forward_ms_per_step": rec_ms / k,
        "backward_ms_per_step": bwd_ms / k,
        "cost_vs_forward": {"backward": bwd_ms / fwd_ms, "recompute_and_backward": (rec_ms + bwd_ms) / fwd_ms},
        "e2e": None, "roofline": None, "clocks": clk.summary(), "gpu_launches": None,
    }
    return out, rank


def field_errors(mix, ref):
    """Errors of the mixed form's state against the double-precision form's after the
    same number of steps: u, v (each relative to its own maximum), p with its mean
    removed (relative), particle centres and angles (absolute), translational velocity
    (relative to the largest |U|, |V|) and angular velocity (relative to the largest |W|)."""
    from ellipsesinflows_gb300.capi import F
    mu, mv, mp, _ = mix.pull_fluid()
    du, dv, dp, _ = ref.pull_fluid()
    rel = lambda a, b: float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))  # noqa: E731
    pi_m, pi_d = mp[1:-1, 1:-1] - mp[1:-1, 1:-1].mean(), dp[1:-1, 1:-1] - dp[1:-1, 1:-1].mean()
    out = {"u": rel(mu, du), "v": rel(mv, dv), "p": rel(pi_m, pi_d)}
    pm, pd = mix.pull_particles(), ref.pull_particles()
    if len(pd):
        dyw = np.abs(pm[:, F["y"]] - pd[:, F["y"]])
        dyw = np.minimum(dyw, ref.cfg.ly - dyw)   # centres wrap in y
        daz = np.abs(pm[:, F["az"]] - pd[:, F["az"]])
        daz = np.minimum(daz, 2 * np.pi - daz)    # angles wrap at 2 pi
        uscale = max(np.abs(pd[:, F["ux"]]).max(), np.abs(pd[:, F["uy"]]).max(), 1e-300)
        out.update({"x": float(np.abs(pm[:, F["x"]] - pd[:, F["x"]]).max()), "y": float(dyw.max()),
                    "az": float(daz.max()),
                    "U": float(np.abs(pm[:, F["ux"]] - pd[:, F["ux"]]).max() / uscale),
                    "V": float(np.abs(pm[:, F["uy"]] - pd[:, F["uy"]]).max() / uscale),
                    "Omega": rel(pm[:, F["vz"]], pd[:, F["vz"]])})
    umag = max(np.abs(du).max(), np.abs(dv).max())
    vel = float(max(np.abs(mu - du).max(), np.abs(mv - dv).max()) / umag)
    return out, vel


def accuracy_leg(args, case, device, pg, world):
    """The plain double-precision form on the same workload: its cell-steps/s on the
    headline's window (steps W+1 .. W+K from the initial state) and on the last steps of
    the run, and the error of the mixed form against it after the workload's full run
    length (per field), with both forms' maximum divergence."""
    import torch
    from ellipsesinflows_gb300 import PREC_FP64, PREC_MIXED, Simulation
    n = args.accuracy_steps or case.steps
    win = max(1, min(20, n // 5))
    ref = Simulation.from_case(case, precision=PREC_FP64, device=device)
    mix = Simulation.from_case(case, precision=PREC_MIXED, device=device)
    rs = torch.cuda.ExternalStream(ref._fn("stream")(ref.ctx), device=device)
    ms_ = torch.cuda.ExternalStream(mix._fn("stream")(mix.ctx), device=device)
    w, k = args.warmup, args.steps
    if n < w + k + win:
        raise ValueError("accuracy run of %d steps is shorter than warm-up + timed steps + %d" % (n, win))
    ref.advance(w)
    ms64 = timed_advance(ref, rs, k, pg, device)
    ref.advance(n - w - k - win)
    s0 = ref.counters()["substeps"]
    ms64_dev = timed_advance(ref, rs, win, pg, device)
    sub64 = (ref.counters()["substeps"] - s0) / (3.0 * win)
    mix.advance(n - win)
    s0 = mix.counters()["substeps"]
    msmx_dev = timed_advance(mix, ms_, win, pg, device)
    submx = (mix.counters()["substeps"] - s0) / (3.0 * win)
    fields, vel = field_errors(mix, ref)
    divmax, _ = mix.divergence()
    divmax64, _ = ref.divergence()
    tm, td = mix.time_state()[1], ref.time_state()[1]
    ref.close()
    mix.close()
    cells = case.cells
    window = "steps %d-%d" % (n - win + 1, n)
    fp64 = {"value": world * cells * k / (ms64 / 1e3), "unit": "cell-steps/s", "ms_per_step": ms64 / k,
            "window": "steps %d-%d (the headline's window)" % (w + 1, w + k),
            "developed": {"window": window, "value": world * cells * win / (ms64_dev / 1e3),
                          "ms_per_step": ms64_dev / win, "substeps_per_stage": sub64}}
    accuracy = {"steps_compared": n, "fields": fields, "velocity_rel_err": vel, "max_divergence": divmax,
                "max_divergence_fp64": divmax64, "time_mixed": tm, "time_fp64": td,
                "how": "both forms advanced %d steps from the same initial state, each with its own dt; "
                       "u, v, p (mean removed), U, V, Omega relative; x, y, az absolute" % n}
    developed = {"window": window, "value": world * cells * win / (msmx_dev / 1e3), "unit": "cell-steps/s",
                 "ms_per_step": msmx_dev / win, "substeps_per_stage": submx,
                 "vs_fp64_developed": ms64_dev / msmx_dev}
    return fp64, accuracy, developed


def precision_is_mixed(args):
    return args.precision == "mixed"


def indicator_roofline(prof, counts, prof_steps):
    """The indicator kernel (normal-foot iteration of every near cell, the step's largest
    kernel): work counted on the device during the profiling pass, over the live event
    time of its launches with geometry (scope ibm_indicator; the stage starts' launches,
    whose weights come from the memo, are timed as ibm_stage_start and reported beside);
    FP32 pipe use from the flops per normal-foot evaluation of an ncu capture."""
    e = next((q for q in prof if q["name"] == "ibm_indicator"), None)
    if e is None or e["ms"] <= 0 or counts.get("normal_foot_evals", 0) <= 0:
        return None
    total = sum(q["ms"] for q in prof) or 1.0
    sec = e["ms"] / 1e3
    evals, cells = counts["normal_foot_evals"], counts["indicator_cells"]
    out = {"kernel": "ibm_indicator", "bound": "issue", "launches_per_step": e["launches"] / prof_steps,
           "box_cells_per_launch": cells / e["launches"], "normal_foot_evals_per_launch": evals / e["launches"],
           "box_cells_per_s": cells / sec, "normal_foot_evals_per_s": evals / sec,
           "share_of_step": e["ms"] / total}
    st = next((q for q in prof if q["name"] == "ibm_stage_start"), None)
    if st is not None and st["launches"] > 0:
        out["stage_start"] = {"launches_per_step": st["launches"] / prof_steps,
                              "us_per_launch": 1e3 * st["ms"] / st["launches"], "share_of_step": st["ms"] / total,
                              "tasks_from_memo_per_step": counts.get("memo_tasks", 0) / prof_steps,
                              "what": "the first evaluation of each RK stage: weights copied from the memo where "
                                      "the particle's single-precision geometry is bitwise unchanged, computed "
                                      "(and counted above) elsewhere"}
    fl = INDICATOR_FLOPS_PER_EVAL
    if fl is not None:
        achieved = evals / sec * fl[0] / 1e12
        out.update({"fp32_flops_per_eval": fl[0], "flops_source": fl[1], "achieved": achieved,
                    "peak": FP32_TFLOPS_MEASURED, "unit": "TFLOP/s", "frac": achieved / FP32_TFLOPS_MEASURED,
                    "peak_source": "measured FP32 FMA-chain probe"})
    return out


def profile_entries(sim):
    import ctypes
    n = ctypes.c_int()
    sim._call("profile_count", sim.ctx, ctypes.byref(n))
    fn = sim._fn("profile_get")
    fn.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_char_p, ctypes.c_int,
                   ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_double)]
    out = []
    for k in range(n.value):
        name = ctypes.create_string_buffer(64)
        launches, ms = ctypes.c_longlong(), ctypes.c_double()
        fn(sim.ctx, k, name, 64, ctypes.byref(launches), ctypes.byref(ms))
        out.append({"name": name.value.decode(), "launches": launches.value, "ms": ms.value})
    out.sort(key=lambda e: -e["ms"])
    return out


def source_sha(name):
    import hashlib
    path = os.path.join(ROOT, "ellipsesinflows_gb300", "csrc", name)
    try:
        with open(path, "rb") as f:
            return hashlib.sha1(f.read()).hexdigest()
    except OSError:
        return None


def stored_traffic(precision, grid, kernel):
    """(bytes, source) of a stored ncu capture of `kernel`, or (None, why not)."""
    rec = NCU_TRAFFIC.get((precision,) + tuple(grid or ()), {}).get(kernel)
    if rec is None:
        return None, None
    value, src, sha, where = rec
    if sha is None or source_sha(src) != sha:
        return None, "stale: %s changed since the capture in %s" % (src, where)
    return value, "ncu capture (%s, %s at sha1 %s)" % (where, src, sha[:12])


def roofline(prof, cells, hbm, hbm_src, precision, grid=None):
    """Roofline of the dominant streaming kernel against the measured copy bandwidth."""
    table = HBM_BYTES[precision]
    total = sum(e["ms"] for e in prof) or 1.0
    stream = [e for e in prof if e["name"] in table and e["launches"] > 0]
    if not stream:
        return None
    top = stream[0]
    per_launch_ms = top["ms"] / top["launches"]
    bytes_per_launch = table[top["name"]] * float(cells)
    achieved = bytes_per_launch / (per_launch_ms / 1e3) / 1e9
    dominant = prof[0]
    traffic, traffic_src = stored_traffic(precision, grid, top["name"])
    return {"bound": "hbm", "kernel": top["name"], "achieved": achieved, "peak": hbm, "unit": "GB/s",
            "frac": achieved / hbm, "peak_source": hbm_src, "traffic": traffic,
            "traffic_source": traffic_src,
            "algorithmic_bytes_per_launch": bytes_per_launch, "share_of_step": top["ms"] / total,
            "dominant_kernel": dominant["name"], "dominant_share": dominant["ms"] / total}


def run_e2e(sim, case, steps, pg, device):
    """Every step: host->device copy of the state, one step, device->host copy of the result
    (eif_push_fluid, eif_push_particles, eif_advance_pull)."""
    import torch
    from ellipsesinflows_gb300.capi import NFIELDS
    ux, uy, p, _ = sim.pull_fluid()
    parts = sim.pull_particles()
    pin = lambda a: torch.from_numpy(a).pin_memory().numpy()  # noqa: E731
    # the state a step reads and the result it leaves: ux, uy, p and the particle records
    # (what the reference saves, src/save.c:41-90); psi is an intermediate of the step
    hux, huy, hp = pin(ux), pin(uy), pin(p)
    hpart = pin(parts)
    h2d = hux.nbytes + huy.nbytes + hp.nbytes + hpart.nbytes
    d2h = hux.nbytes + huy.nbytes + hp.nbytes + hpart.nbytes
    barrier(pg, device)
    t0 = time.perf_counter()
    for _ in range(steps):
        sim.push_fluid(hux, huy, hp)
        sim.push_particles(hpart)
        # eif_advance_pull: the step, then its fields and records into the host arrays
        # (the fields' copy overlaps the last stage's particle work)
        sim.advance_pull(1, (hux, huy, hp), hpart)
    el = time.perf_counter() - t0
    el = max_over_ranks(pg, el, device)
    world = pg.get_world_size() if pg is not None else 1
    return {"value": world * case.cells * steps / el, "unit": "cell-steps/s", "h2d_bytes_per_step": h2d,
            "d2h_bytes_per_step": d2h, "n_particle_fields": NFIELDS}


def cpu_baseline(args, case):
    """The CPU restatement on the host cores, on a bounded sample: one time step of the workload."""
    from oracle import port
    threads = os.cpu_count() or 1
    s = port.PortSolver(case.config(), threads=threads)
    s.push_fluid(*case.fluid())
    s.push_particles(case.particles)
    t0 = time.perf_counter()
    s.step()
    el = time.perf_counter() - t0
    return {"value": case.cells / el, "unit": "cell-steps/s", "cores": threads, "kind": "port",
            "sample": "1 time step of the full %s workload from its initial state" % case.name}


def run_reference(args, world, rank):
    """Reference arm: the CPU restatement of the reference algorithm (oracle/port, pinned
    bit-for-bit to the reference's own sources) on all host threads, on the same
    workload, metric and step counts: W warm-up steps, then K timed steps, each one
    full time step of the workload from its initial state."""
    if rank != 0:
        return None, rank
    from oracle import port
    case = make_case(args.workload)
    threads = os.cpu_count() or 1
    s = port.PortSolver(case.config(), threads=threads)
    s.push_fluid(*case.fluid())
    s.push_particles(case.particles)
    for _ in range(args.warmup):
        s.step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        s.step()
    el = time.perf_counter() - t0
    value = case.cells * args.steps / el
    sample = "%d timed full time steps of %s after %d warm-up steps, from its initial state" % (
        args.steps, case.name, args.warmup)
    out = {"metric": "cell-steps/s", "value": value, "unit": "cell-steps/s", "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (seeded ellipse placement, fluid at rest)",
           "config": workload_config(case, world), "precision": "fp64",
           "impl": "reference",
           "cpu_baseline": {"value": value, "unit": "cell-steps/s", "cores": threads, "kind": "port",
                            "sample": sample},
           "e2e": {"value": value, "unit": "cell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    return out, rank


def main():
    args = parse()
    world, rank, local, pg = dist_init(args.gpus)
    if args.impl == "reference":
        out, rank = run_reference(args, world, rank)
    elif args.workload == "batch_c5":
        out, rank = run_batch(args, world, rank, local, pg)
    elif args.workload.startswith("adjoint"):
        out, rank = run_adjoint(args, world, rank, local, pg)
    else:
        out, rank = run_ours(args, world, rank, local, pg)
    if rank == 0 and out is not None:
        print(json.dumps(out), flush=True)
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
