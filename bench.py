#!/usr/bin/env python
"""Time-steps/s of the LeachingSim per-time-step hot path on GB300.

Workload (the reference README shape): 338 x 338 x 283 voxels (--xext 338 --yext 338
--zext 283, i.e. (I, J, K) = (283, 338, 338)), uint8 labels from a seeded Gaussian
random field (porosity 0.25, correlation length 6, 15% of the solid reactive mineral,
Air inlet planes i = 0, 1), D = 1, kreac = 1, dt = 1, tmax = 50, nout = 10, csat = 1.

A "step" is one full time step of src/main.cpp:303-432 (props, pressure solve, flux,
saturation, surface clogging, conc + acid transport, precipitation, dissolution,
snapshot). `value` times --steps steps after --warmup steps with the state resident
in HBM; `e2e` runs the whole configured simulation (tmax / dt steps) from a label
image in pinned host memory, reading every output step's fields back into pinned
host memory (file writing excluded); `e2e.parts` splits its wall time (context
creation and upload, the cold first step, the other steps' median / mean / maximum,
the output steps, the final drain of the copies).

  python bench.py [--gpus N --steps K --warmup W] [--impl reference]

The CPU baseline (`cpu_baseline` and the `--impl reference` arm) runs the oracle's
production mode on the same 338 x 338 x 283 grid, on all host cores, with no scaling:
multigrid-preconditioned CG for the pressure (the stand-in for the algebraic multigrid the
reference's job scripts select, -press_pc_type hypre) and GMRES(30)+Jacobi for the
transport systems, each solve run twice like the reference's KSPSolve pair. The
`cpu_baseline` leg times a few steps from the state the GPU run reached and compares the
fields the two then produce; the reference arm runs the whole workload from the labels.

`flow_mode` (inside the line, or alone with `--flow`): the same geometry without the Air
planes, driven by the flow-through pressure boundary (P = 1 on the Pore voxels of z = 0,
P = 0 on those of z = max, no-flow sides), so that every step solves a changed pressure
system.

Separate lines: `--mixed` (the 512^3 uint16 fractured geometry, mixed precision against
FP64 settings, per-field error and memory footprint) and `--geometry` (the geometry
pre-processing pipeline at 512^3).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "time-steps/s at 338x338x283"
UNIT = "time-steps/s"
SHAPE = (283, 338, 338)  # (I, J, K) = (zext, yext, xext)
GEOM = dict(porosity=0.25, corr_len=6.0, mineral_fraction=0.15, seed=0)
DT, TMAX, NOUT = 1.0, 50.0, 10
CPU_STEPS = 3  # steps of the cpu_baseline leg at the full grid
PRECISION = ("FP64 fields, residuals, refinement and budgets; FP32 inner Krylov / multigrid "
             "iterations of the pressure and transport solves")
# output arrays of src/Simulation.cpp:1401-1485 (label, frac, 10 float64 fields)
OUTPUT_FIELDS = ["label", "conc", "pressure", "frac", "flux_x", "flux_y", "flux_z", "saturation",
                 "cap_pressure", "rel_perm", "permeability", "acid"]


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(x, ws, device="cuda"):
    """The largest of a per-rank value: the slowest replica sets the job's time."""
    if ws <= 1:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def replica_rate(ws, steps_per_rank, seconds):
    """Whole-job steps/s of ws independent replicas (no data-path collective), each running
    steps_per_rank steps, over the slowest replica's time."""
    return ws * steps_per_rank / seconds


def make_geometry(shape):
    from leachingsim_gb300.geometry import grf_geometry
    lab, seed = grf_geometry(shape, air_inlet=True, **GEOM)
    return lab, seed


# Solver tolerances of the workload: transport and saturation at the reference's own KSP
# default (rtol 1e-6, src/Simulation.cpp:156 -- the tolerance of the CPU baseline's
# reference-algorithm mode too), the pressure at the FP64 relative residual 1e-8 of the
# second metric.
CONC_RTOL = 1e-6
PRESS_RTOL = 1e-8


def params(solver, **kw):
    from leachingsim_gb300._abi import PRESS_FP64, PRESS_JACOBI64, PRESS_MIXED, default_params
    s = {"mixed": PRESS_MIXED, "fp64": PRESS_FP64, "jacobi64": PRESS_JACOBI64}[solver]
    return default_params(c_sat=1.0, D=1.0, kreac=1.0, press_solver=s, conc_rtol=CONC_RTOL,
                          sat_rtol=CONC_RTOL, press_rtol=PRESS_RTOL, **kw)


def workload_config(shape, seed):
    """The `config` object both arms print (identical, so the driver can pair them)."""
    return {"workload": f"{shape[2]}x{shape[1]}x{shape[0]} uint8 GRF geometry (porosity 0.25, corr 6, 15% "
                        "mineral, Air inlet), dt 1, tmax 50, nout 10, D 1, kreac 1, csat 1, transport rtol "
                        "1e-6 (the reference's KSP default), pressure rtol 1e-8",
            "shape_ijk": list(shape), "seed": seed,
            "l2": "working set > L2" if shape[0] * shape[1] * shape[2] * 8 > 129e6 else "working set < L2"}


# ---------------------------------------------------------------------------
# clocks

CLOCK_FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")


class ClockSampler:
    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={CLOCK_FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"], stdout=self.fh,
                stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if self.proc is None or not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "samples": len(sm),
                "reasons": sorted(reasons)}


# ---------------------------------------------------------------------------
# GPU arm

def run_steps(ctx, t0, n0, count, dt):
    """count accepted steps with the reference's retry manager; returns (t, n, infos)."""
    t, n = t0, n0
    infos = []
    for _ in range(count):
        cur = dt
        while True:
            ok, info = ctx.step(t, cur)
            if ok:
                break
            ctx.rollback()
            cur *= 0.5
            if cur < 1e-3:
                raise RuntimeError("time step shrank below 1 ms")
        infos.append(info)
        t += cur
        n += 1
    return t, n, infos


def roofline(ctx, shape, nsteps):
    """Roofline of the dominant kernel class, the transport operator applications of the
    inner BiCGStab (k_ti_v and k_ti_st). The library accumulates their algorithmic bytes per
    launch: N x (six FP32 scaled off-diagonals 24 + per live right-hand side 4 bytes for each
    vector read or written once: 12 for v = A p (p in, rhat in, v out; 16 on the first
    iteration, which also stores p = r), 20 for s = r - alpha v, t = A s (r, v, rhat in; s, t
    out)); one right-hand side is live in this workload (the acid field is zero)."""
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    peaks = json.load(open(peaks_path)) if os.path.exists(peaks_path) else None
    ms, cnt = ctx.timing_get("kry_apply")
    nbytes = ctx.timing_bytes("kry_apply")
    if cnt == 0 or ms <= 0:
        return None
    achieved = nbytes / (ms / 1e3) / 1e9
    peak, src = (peaks["hbm_gbs"], "measured") if peaks else (6800.0, "fallback")
    vox = shape[0] * shape[1] * shape[2]
    # DRAM traffic per launch: dram__bytes_read.sum + dram__bytes_write.sum per voxel from one
    # ncu capture of the 160x256x256 case (inputs > L2), k_ti_v_pair 35.13 B and k_ti_st_pair
    # 42.42 B, scaled by the voxel count; the timed launches alternate the two kernels
    traffic = 0.5 * (35.13 + 42.42) * vox
    return {"bound": "hbm", "kernel": "transport operator apply (k_ti_v_pair, k_ti_st_pair)",
            "achieved": round(achieved, 1), "peak": peak, "peak_source": src, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "traffic": round(traffic),
            "bytes_per_launch": round(nbytes / cnt), "bytes_per_voxel": round(nbytes / cnt / vox, 2),
            "launches": cnt, "us_per_launch": round(ms * 1e3 / cnt, 2)}


def true_rel_residual(ctx):
    """||b - A x||_2 / ||b||_2 in FP64 for the assembled pressure system and its last solution
    (outside the timed solves: A x through the library's FP64 operator on the host arrays)."""
    Pp = ctx.download("pressure", padded=True).ravel()
    sh = ctx.J * ctx.K if ctx.params.compat_shift else 0
    x = Pp[sh:sh + ctx.N]
    b = ctx.pressure_rhs()
    r = b - ctx.pressure_apply(x)
    nb = float(np.linalg.norm(b))
    return float(np.linalg.norm(r) / nb) if nb > 0 else float(np.linalg.norm(r))


def cold_pressure_solves(ctx, shape, solver, reps=2):
    """The second metric: cold solves of the first step's pressure system (t = 0, zero
    start, rtol 1e-8 on the Jacobi-scaled FP64 residual) with the plain FP64 multigrid-PCG,
    with the mixed-precision K-cycle FCG, and with the mixed solver from the learned start
    (when trained weights exist). Each: assembly + [network inference] + solve, wall time
    with the device idle on both sides, the last of `reps` runs (the first pays the buffer
    allocations of a precision switch). The P slots are zeroed around every solve, so the
    run that follows starts from the same state."""
    import torch
    from leachingsim_gb300 import learned as L
    from leachingsim_gb300._abi import PRESS_FP64, PRESS_LEARNED, PRESS_MIXED
    zeros_p = np.zeros(ctx.NP)
    zeros = torch.zeros(shape, dtype=torch.float32, device="cuda")
    weights = L.load_weights()
    ls = L.LearnedStart(shape, weights) if weights is not None else None
    variants = [("plain_fp64", PRESS_FP64, None), ("plain", PRESS_MIXED, None)]
    if ls is not None:
        variants.append(("learned", PRESS_MIXED, ls))
    pw = L.load_precond_weights()
    if pw is not None:
        # the network as the coarse solver inside the flexible CG, the plain cycle as fallback
        ctx.set_precond_weights(pw)
        variants.append(("learned_precond", PRESS_LEARNED, None))
    # context for the learned start: the untrained guess P = p_top on every Pore row
    variants.append(("constant_start", PRESS_MIXED, "constant"))
    ctx.props()
    out = {}
    for name, s, start in variants:
        base = params("fp64" if s == PRESS_FP64 else "mixed")
        base.press_solver = s
        ctx.set_params(base)
        fb0 = ctx.pressure_fallbacks()
        for _ in range(reps):
            ctx.upload("pressure", zeros_p, padded=True)
            ctx.synchronize()
            torch.cuda.synchronize()
            w0 = time.perf_counter()
            ctx.pressure_setup(0.0)
            w1 = time.perf_counter()
            if start == "constant":
                x0 = ctx.pressure_learned_inputs()[0]
            else:
                x0 = start.start(ctx) if start is not None else zeros
            torch.cuda.synchronize()
            w2 = time.perf_counter()
            ok, info = ctx.pressure_solve_start(x0, 1.0 if start is not None else 0.0)
            ctx.synchronize()
            w3 = time.perf_counter()
        out[name] = {"solver": "fp64" if s == PRESS_FP64 else "mixed", "ms": round((w3 - w0) * 1e3, 3),
                     "setup_ms": round((w1 - w0) * 1e3, 3), "solve_ms": round((w3 - w2) * 1e3, 3),
                     "iterations": info["iterations"], "outer": info["outer_iterations"],
                     "scaled_rel_residual": info["rel_residual"],
                     "true_rel_residual": true_rel_residual(ctx), "converged": bool(ok)}
        if start is not None:
            out[name]["start_ms"] = round((w2 - w1) * 1e3, 3)
        if s == PRESS_LEARNED:
            out[name]["fallbacks_per_solve"] = (ctx.pressure_fallbacks() - fb0) / reps
    if ls is not None:
        ls.close()
    ctx.set_params(params(solver))
    ctx.upload("pressure", zeros_p, padded=True)
    ctx.synchronize()
    return out


def gpu_arm(args, ws, rank, local):
    import torch
    from leachingsim_gb300.runtime import Context

    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    shape = tuple(int(v) for v in args.shape.split(",")) if args.shape else SHAPE
    t0 = time.time()
    lab, seed = make_geometry(shape)
    log(f"[rank {rank}] geometry {shape} seed {seed} in {time.time() - t0:.1f}s")
    p = params(args.solver)

    def barrier():
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    # ---- resident-state throughput ------------------------------------------------
    ctx = Context(shape, label_bytes=1, params=p)
    ctx.upload("label", lab)
    ctx.init_all()
    stream = torch.cuda.ExternalStream(ctx.stream())
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    # second metric: cold pressure solves of the first step's system (plain FP64, mixed,
    # learned start), then the run's own first step, whose pressure solve is a cold solve
    # too (assembly + setup + solve from the library's CUDA-event timers)
    cold = cold_pressure_solves(ctx, shape, args.solver) if not args.no_cold else {}
    ctx.timing(True)
    ctx.timing_reset()
    if args.nvtx:
        torch.cuda.nvtx.range_push("cold")
    t, n, first = run_steps(ctx, 0.0, 0, 1, DT)
    ctx.synchronize()
    if args.nvtx:
        torch.cuda.nvtx.range_pop()
    pinfo = first[0]["pressure"]
    psolve_ms = sum(ctx.timing_get(k)[0] for k in ("press_setup", "press_inner", "press_outer"))
    psolve = dict(cold)
    psolve["first_step"] = {"solver": args.solver, "ms": round(psolve_ms, 3), "iterations": pinfo["iterations"],
                            "outer": pinfo["outer_iterations"], "scaled_rel_residual": pinfo["rel_residual"],
                            "converged": bool(pinfo["converged"])}
    psolve.setdefault("learned", None)
    psolve["note"] = ("cold solves of the first step's pressure system (true_rel_residual: ||b - A x||_2 / "
                      "||b||_2 of the result in FP64, the solves stop on the Jacobi-scaled one): t = 0, zero "
                      "start (learned: the "
                      "network's start; constant_start: P = p_top on the Pore rows; learned_precond: the "
                      "network as the multigrid's level-4 solver inside the flexible CG, with the plain "
                      "cycle taking over on stagnation), rtol 1e-8 on the "
                      "Jacobi-scaled FP64 residual; ms = assembly + [start: inputs, distance transform, "
                      "network] + multigrid setup + solve; first_step = the run's own first step (device "
                      "timers)")
    ctx.timing(False)
    t, n, _ = run_steps(ctx, t, n, max(args.warmup - 1, 0), DT)
    ctx.timing(True)
    ctx.timing_reset()
    barrier()
    with ClockSampler(local) as clk:
        if args.nvtx:
            torch.cuda.nvtx.range_push("timed")
        ev0.record(stream)
        w0 = time.perf_counter()
        t, n, infos = run_steps(ctx, t, n, args.steps, DT)
        ev1.record(stream)
        ev1.synchronize()
        wall = time.perf_counter() - w0
        if args.nvtx:
            torch.cuda.nvtx.range_pop()
    barrier()
    dev_ms = ev0.elapsed_time(ev1)
    launches = ctx.launches()
    classes = {k: ctx.timing_get(k) for k in ("props", "press_setup", "press_inner", "press_outer",
                                              "flux", "saturation", "transport", "precip",
                                              "dissolve", "snapshot", "kry_apply", "cg_apply")}
    roof = roofline(ctx, shape, args.steps)
    ctx.timing(False)
    mem = ctx.device_bytes()
    # the CPU baseline leg at the full grid, from this state (rank 0 of a 1-GPU run)
    cpu = None
    if ws == 1 and rank == 0 and not args.no_cpu:
        cpu = cpu_leg(ctx, shape, p, t, n, args.cpu_steps)
        t += args.cpu_steps * DT
        n += args.cpu_steps
    # the GPU plain path: the same number of steps on the same state with the FP64 inner
    # multigrid-PCG for the pressure (the plain FP64 solver), right after the timed steps
    plain = None
    if not args.no_plain and args.solver != "fp64":
        ctx.set_params(params("fp64"))
        t, n, _ = run_steps(ctx, t, n, 1, DT)  # untimed: the switch allocates the FP64 buffers
        barrier()
        ev0.record(stream)
        t, n, _ = run_steps(ctx, t, n, args.steps, DT)
        ev1.record(stream)
        ev1.synchronize()
        barrier()
        pms = max_over_ranks(ev0.elapsed_time(ev1) / 1e3, ws)
        plain = {"value": round(replica_rate(ws, args.steps, pms), 4), "unit": UNIT,
                 "ms_per_step": round(pms * 1e3 / args.steps, 3), "press_solver": "fp64",
                 "note": "the same steps with the plain FP64 multigrid-PCG pressure solver, on the state "
                         "the timed steps left (warm pressure starts, as in the timed steps)"}
        ctx.set_params(p)
    ctx.close()
    t_max = max_over_ranks(dev_ms / 1e3, ws)

    # ---- end to end: full configured run from a host image ---------------------------
    e2e = None
    if not args.no_e2e:
        nsteps = int(round(TMAX / DT))
        pinned_lab = torch.empty(lab.size, dtype=torch.uint8, pin_memory=True)
        pinned_lab.numpy()[:] = lab.ravel()
        N = lab.size
        out_bufs = {}
        for f in OUTPUT_FIELDS:
            dt_ = torch.uint8 if f == "label" else (torch.float32 if f == "frac" else torch.float64)
            out_bufs[f] = torch.empty(N, dtype=dt_, pin_memory=True).numpy()
        barrier()
        w0 = time.perf_counter()
        ctx = Context(shape, label_bytes=1, params=p)
        ctx.upload("label", pinned_lab.numpy())
        ctx.init_all()
        w1 = time.perf_counter()
        h2d = N
        d2h = 0
        te, ne = 0.0, 0
        pending = None
        step_s, out_s = [], []
        for _ in range(nsteps):
            s0 = time.perf_counter()
            te, ne, _ = run_steps(ctx, te, ne, 1, DT)   # returns after the step's scalars are read
            if (ne - 1) % NOUT == 0:
                ctx.props()   # property sync before output (src/main.cpp:491-494)
                if pending is not None:
                    pending.wait()  # the previous output's copies (long done) before reusing its buffers
                # the copies drain on the context's copy stream while the next steps run
                pending = ctx.download_async(OUTPUT_FIELDS, [out_bufs[f] for f in OUTPUT_FIELDS])
                d2h += sum(out_bufs[f].nbytes for f in OUTPUT_FIELDS)
                out_s.append(time.perf_counter() - s0)
            else:
                step_s.append(time.perf_counter() - s0)
        w2 = time.perf_counter()
        if pending is not None:
            pending.wait()
        ctx.synchronize()
        e2e_wall = time.perf_counter() - w0
        e2e_parts = {"create_upload_init_ms": round((w1 - w0) * 1e3, 2),
                     "first_step_ms": round(out_s[0] * 1e3, 2) if out_s else None,
                     "step_ms_median": round(statistics.median(step_s) * 1e3, 2) if step_s else None,
                     "step_ms_mean": round(statistics.mean(step_s) * 1e3, 2) if step_s else None,
                     "step_ms_max": round(max(step_s) * 1e3, 2) if step_s else None,
                     "output_step_ms_mean": round(statistics.mean(out_s[1:]) * 1e3, 2) if len(out_s) > 1 else None,
                     "final_drain_ms": round((time.perf_counter() - w2) * 1e3, 2)}
        ctx.close()
        e2e_wall = max_over_ranks(e2e_wall, ws)
        e2e = {"value": round(replica_rate(ws, nsteps, e2e_wall), 4), "unit": UNIT,
               "h2d_bytes_per_step": int(h2d / nsteps), "d2h_bytes_per_step": int(d2h / nsteps),
               "steps": nsteps, "wall_s": round(e2e_wall, 3), "parts": e2e_parts,
               "note": ("fresh run from a pinned host label image, every nout-th step's fields read back to "
                        "pinned host memory (copies on the context's copy stream, overlapping the next "
                        "steps; all landed before the clock stops)")}

    flow = None if args.no_flow else flow_run(args, shape, ws, barrier)
    if rank != 0:
        return None
    value = replica_rate(ws, args.steps, t_max)
    # the metric names the grid as the reference's CLI does: xext x yext x zext = K x J x I
    metric = METRIC if shape == SHAPE else f"time-steps/s at {shape[2]}x{shape[1]}x{shape[0]}"
    line = {
        "metric": metric, "value": round(value, 4), "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dev_ms / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64/f32" if args.solver == "mixed" else "f64", "precision": PRECISION,
        "data": "synthetic", "config": workload_config(shape, seed),
        "press_solver": args.solver, "parallelism": f"replicas{ws}",
        "wall_ms_per_step": round(wall * 1e3 / args.steps, 3),
        "gpu_launches": launches,
        "device_bytes": mem,
        "timers_ms": {k: round(v[0], 3) for k, v in classes.items()},
        "roofline": roof,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "pressure_solve": psolve,
        "plain_path": plain,
        "flow_mode": flow,
        "clocks": clk.summary(),
    }
    return line


# ---------------------------------------------------------------------------
# flow-through model: the workload's geometry without the Air planes, pressure held at 1 on
# the Pore voxels of z = 0 and at 0 on those of z = max (no-flow sides), acid flowing in at
# z = 0; the acid dissolves mineral, leached voxels open new pore space, and every step solves
# a changed pressure system

FLOW_PIN, FLOW_POUT, FLOW_ACID = 1.0, 0.0, 1.0


def flow_params(solver):
    from leachingsim_gb300._abi import BC_FLOW_I
    return params(solver, bc_mode=BC_FLOW_I, p_inlet=FLOW_PIN, p_outlet=FLOW_POUT, acid_inlet=FLOW_ACID)


def flow_run(args, shape, ws, barrier):
    """Steps/s of the flow-through model on the workload's grid: the first (cold) step, then
    --warmup - 1 untimed and --steps timed steps with the mixed solver, then the same number
    with the plain FP64 multigrid-PCG pressure solver on the state they left; per-step pressure
    iterations and the pressure solve's share of the step from the library's timers."""
    import torch
    from leachingsim_gb300.geometry import grf_geometry
    from leachingsim_gb300.runtime import Context
    lab, seed = grf_geometry(shape, air_inlet=False, **GEOM)
    ctx = Context(shape, label_bytes=1, params=flow_params(args.solver))
    ctx.upload("label", lab)
    ctx.init_all()
    stream = torch.cuda.ExternalStream(ctx.stream())
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ctx.timing(True)
    ctx.timing_reset()
    t, n, first = run_steps(ctx, 0.0, 0, 1, DT)
    cold = {k: round(ctx.timing_get(k)[0], 3) for k in ("press_setup", "press_inner", "press_outer")}
    t, n, _ = run_steps(ctx, t, n, max(args.warmup - 1, 0), DT)

    def timed(solver):
        nonlocal t, n
        ctx.set_params(flow_params(solver))
        ctx.timing_reset()
        barrier()
        ev0.record(stream)
        t, n, infos = run_steps(ctx, t, n, args.steps, DT)
        ev1.record(stream)
        ev1.synchronize()
        barrier()
        sec = max_over_ranks(ev0.elapsed_time(ev1) / 1e3, ws)
        tm = {k: ctx.timing_get(k)[0] for k in ("press_setup", "press_inner", "press_outer")}
        return {"value": round(replica_rate(ws, args.steps, sec), 4), "unit": UNIT,
                "ms_per_step": round(sec * 1e3 / args.steps, 3),
                "pressure_ms_per_step": round(sum(tm.values()) / args.steps, 3),
                "press_inner_ms_per_step": round(tm["press_inner"] / args.steps, 3),
                "pressure_iterations": [i["pressure"]["iterations"] for i in infos],
                "pressure_rel_residual_max": max(i["pressure"]["rel_residual"] for i in infos),
                "dissolve_ms_per_step": round(ctx.timing_get("dissolve")[0] / args.steps, 3),
                "transport_ms_per_step": round(ctx.timing_get("transport")[0] / args.steps, 3),
                "leached_per_step": [i["leached"] for i in infos],
                "leach_substeps": [i["leaching"]["num_steps"] for i in infos],
                "mineral_budget_last": infos[-1]["budget"]["mineral"],
                "dissolution_fallbacks": ctx.dissolve_fallbacks()}

    mixed = timed(args.solver)
    plain = timed("fp64") if args.solver != "fp64" else None
    ctx.timing(False)
    ctx.close()
    return {"metric": f"time-steps/s at {shape[2]}x{shape[1]}x{shape[0]}, flow-through pressure",
            "workload": (f"the workload's geometry (seed {seed}) without Air planes; P = {FLOW_PIN:g} on the Pore "
                         f"voxels of z = 0, P = {FLOW_POUT:g} on those of z = max, no-flow sides; acid "
                         f"{FLOW_ACID:g} flowing in at z = 0; dt 1, D 1, kreac 1, csat 1, pressure rtol 1e-8, "
                         "transport rtol 1e-6"),
            "steps": args.steps, "warmup": args.warmup, "mixed": mixed, "plain_fp64": plain,
            "cold_step_pressure_ms": cold,
            "cold_step_pressure_iterations": first[0]["pressure"]["iterations"]}


# ---------------------------------------------------------------------------
# CPU: the oracle's production mode (multigrid-preconditioned CG for the pressure, the
# stand-in for the reference job scripts' -press_pc_type hypre; GMRES(30)+Jacobi for the
# transport; two KSPSolve calls per solve; tolerances of the workload) on the full grid

STATE_FIELDS = ["label", "frac", "precipitate", "saturation", "pressure", "conc", "acid", "flux_x", "flux_y",
                "flux_z", "cap_pressure", "rel_perm", "permeability", "viscosity"]
CMP_FIELDS = ["pressure", "flux_x", "flux_y", "flux_z", "conc", "precipitate", "saturation"]


def cpu_threads():
    return os.cpu_count() or 1


def oracle_production(shape, p, threads):
    from oracle import oracle as om
    o = om.Oracle(shape, params=p, mode=om.SOLVE_PRODUCTION, threads=threads)
    o.set_solver(om.SOLVE_PRODUCTION)
    return o


def rel_l2(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    d = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / d) if d > 0 else float(np.linalg.norm(a - b))


def cpu_leg(ctx, shape, p, t, n, steps):
    """The cpu_baseline leg: the state the GPU run has reached (every field, padded) goes to
    the oracle, which runs `steps` steps on all host cores (timed); the GPU runs the same
    steps from the same state (untimed), and the fields of both are compared."""
    state = {f: ctx.download(f, padded=True).copy() for f in STATE_FIELDS}
    for k in range(steps):
        ok, _ = ctx.step(t + k * DT, DT)
        if not ok:
            raise RuntimeError("GPU step failed in the comparison leg")
    gpu = {f: ctx.download(f, padded=True).copy() for f in CMP_FIELDS + ["label"]}
    threads = cpu_threads()
    o = oracle_production(shape, p, threads)
    for f, v in state.items():
        o.set(f, v.astype(np.uint16) if f == "label" else v, padded=True)
    w0 = time.perf_counter()
    iters = []
    for k in range(steps):
        ok, info = o.step(t + k * DT, DT)
        if not ok:
            raise RuntimeError("CPU reference step failed")
        iters.append((info["pressure"]["iterations"], info["conc"]["iterations"]))
    wall = time.perf_counter() - w0
    cpu = {f: o.get(f, padded=True) for f in CMP_FIELDS + ["label"]}
    o.close()
    vel = lambda d: np.concatenate([d[k].ravel() for k in ("flux_x", "flux_y", "flux_z")])  # noqa: E731
    cmp = {"pressure": rel_l2(gpu["pressure"], cpu["pressure"]), "velocity": rel_l2(vel(gpu), vel(cpu)),
           "conc": rel_l2(gpu["conc"], cpu["conc"]), "saturation": rel_l2(gpu["saturation"], cpu["saturation"]),
           "precipitate_abs": float(np.abs(gpu["precipitate"] - cpu["precipitate"]).max()),
           "label_mismatches": int(np.count_nonzero(gpu["label"].astype(np.int64) != cpu["label"].astype(np.int64)))}
    return {"value": round(steps / wall, 6), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": (f"{steps} steps of the full {shape[2]}x{shape[1]}x{shape[0]} grid (no scaling) from the "
                       f"state the GPU run reached after its timed steps (t = {t:g} s), oracle production mode: "
                       "multigrid-PCG pressure (for the job scripts' hypre AMG), GMRES(30)+Jacobi transport, "
                       "KSPSolve twice, pressure rtol 1e-8, transport rtol 1e-6"),
            "wall_s": round(wall, 3), "iterations": iters,
            "gpu_vs_cpu_rel_l2": cmp,
            "gpu_vs_cpu_note": ("the GPU's fields after the same steps from the same state, relative L2 per field "
                                "(velocity = the three face fluxes together; precipitate as the largest absolute "
                                "difference); both solve to the workload's tolerances")}


def reference_arm(args, ws, rank):
    """The reference's algorithm on the host cores, from the labels: the workload's own
    geometry on the full grid, --warmup untimed steps (the first solves the cold pressure
    system), then --steps timed steps. Rank 0 only."""
    if rank != 0:
        return None
    shape = tuple(int(v) for v in args.shape.split(",")) if args.shape else SHAPE
    t0 = time.time()
    lab, seed = make_geometry(shape)
    threads = cpu_threads()
    o = oracle_production(shape, params(args.solver), threads)
    o.load_labels(lab)
    o.init_all()
    log(f"reference: geometry + init {time.time() - t0:.1f}s on {threads} threads")
    t = 0.0
    w0 = time.perf_counter()
    for _ in range(args.warmup):
        ok, _ = o.step(t, DT)
        if not ok:
            raise RuntimeError("CPU reference step failed")
        t += DT
    warm_wall = time.perf_counter() - w0
    w0 = time.perf_counter()
    for _ in range(args.steps):
        ok, _ = o.step(t, DT)
        if not ok:
            raise RuntimeError("CPU reference step failed")
        t += DT
    wall = time.perf_counter() - w0
    o.close()
    value = args.steps / wall
    metric = METRIC if shape == SHAPE else f"time-steps/s at {shape[2]}x{shape[1]}x{shape[0]}"
    return {
        "impl": "reference", "metric": metric, "value": round(value, 6), "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(wall * 1e3 / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": workload_config(shape, seed),
        "cpu_baseline": {"value": round(value, 6), "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": (f"the whole workload from the labels on the full grid: {args.warmup} untimed "
                                    f"steps (the first a cold pressure solve, {warm_wall:.1f} s) then {args.steps} "
                                    "timed steps; oracle production mode (multigrid-PCG pressure for the job "
                                    "scripts' hypre AMG, GMRES(30)+Jacobi transport, KSPSolve twice)")},
        "e2e": {"value": round(value, 6), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


# ---------------------------------------------------------------------------
# geometry pre-processing (a separate line, --geometry): grey-level classification,
# clean_micro_ct.py, micro_fracture.py and coarsen_grid.py on a 512^3 uint16 image

GEO_SHAPE = (512, 512, 512)
GEO_CPU_SAMPLE = (96, 96, 96)


def geometry_pipeline(grey, thr, impl):
    """classify -> clean (core_sample) -> fracture -> coarsen; returns stage times in ms and
    the final labels."""
    if impl == "gpu":
        from leachingsim_gb300 import runtime as rt
        classify = lambda g: rt.geom_classify(g, thr, [2, 3, 4], 2)  # noqa: E731
        clean, fracture, coarsen = rt.geom_clean, rt.geom_fracture, rt.geom_coarsen
    else:
        from oracle import geometry_oracle as go
        classify = lambda g: go.classify(g, thr, np.array([2, 3, 4], np.uint16))  # noqa: E731
        clean, fracture, coarsen = go.clean, go.fracture, go.coarsen
    ms = {}
    t = time.perf_counter()
    lab = classify(grey)
    ms["classify"] = (time.perf_counter() - t) * 1e3
    t = time.perf_counter()
    lab, _ = clean(lab, "core_sample")
    ms["clean"] = (time.perf_counter() - t) * 1e3
    t = time.perf_counter()
    lab, drilled, enc = fracture(lab)
    ms["fracture"] = (time.perf_counter() - t) * 1e3
    t = time.perf_counter()
    out = coarsen(lab)
    ms["coarsen"] = (time.perf_counter() - t) * 1e3
    return ms, out, drilled, enc


def geometry_arm(args):
    from leachingsim_gb300.geometry import grey_levels
    shape = tuple(int(v) for v in args.shape.split(",")) if args.shape else GEO_SHAPE
    grey = grey_levels(shape, corr_len=6.0, seed=0, n_fractures=4)
    sub = grey[::4, ::4, ::4].ravel()
    thr = [int(np.quantile(sub, 0.2)), int(np.quantile(sub, 0.88))]
    small = np.ascontiguousarray(grey[:64, :64, :64])
    for _ in range(max(args.warmup, 1)):
        geometry_pipeline(small, thr, "gpu")
    runs = [geometry_pipeline(grey, thr, "gpu") for _ in range(args.steps)]
    vox = grey.size
    total = [sum(r[0].values()) for r in runs]
    med = statistics.median(total)
    stages = {k: round(statistics.median(r[0][k] for r in runs), 3) for k in runs[0][0]}
    line = {"metric": f"geometry pre-processing voxels/s at {shape[0]}x{shape[1]}x{shape[2]} uint16",
            "value": round(vox / (med / 1e3), 1), "unit": "voxels/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(med, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u16", "data": "synthetic",
            "config": {"workload": f"{shape[0]}x{shape[1]}x{shape[2]} uint16 grey-level random field "
                                   "(corr 6, 4 planar fractures of 1-3 voxel aperture), thresholds at the "
                                   "20% / 88% grey quantiles -> Pore / Rock / Sulphide, clean "
                                   "(core_sample), micro-fracture drilling, 2x2x2 coarsening",
                       "thresholds": thr},
            "stages_ms": stages, "drilled": int(runs[0][2]), "encapsulated": int(runs[0][3]),
            "e2e": {"value": round(vox / (med / 1e3), 1), "unit": "voxels/s",
                    "h2d_bytes_per_step": int(vox * 2 * 4), "d2h_bytes_per_step": int(vox * 2 * 3 + vox // 4),
                    "note": "the ls_geom_* entry points take host buffers: every stage copies its "
                            "image in and out, so value and e2e are the same measurement"}}
    if not args.no_cpu:
        cs = GEO_CPU_SAMPLE
        g = np.ascontiguousarray(grey[:cs[0], :cs[1], :cs[2]])
        t = time.perf_counter()
        ms, _, _, _ = geometry_pipeline(g, thr, "cpu")
        wall = time.perf_counter() - t
        line["cpu_baseline"] = {"value": round(g.size / wall, 1), "unit": "voxels/s", "cores": 1, "kind": "port",
                                "sample": f"{cs[0]}x{cs[1]}x{cs[2]} corner of the same image through the "
                                          "oracle (numpy / scipy, the reference scripts' libraries)",
                                "stages_ms": {k: round(v, 1) for k, v in ms.items()}}
    return line


# ---------------------------------------------------------------------------
# mixed precision at 512^3 (a separate line, --mixed): the uint16 grey-level geometry with
# planar fractures, stepped with the FP32-inner solvers (FP64 refinement) and again with the
# FP64 settings; per-field relative-L2 error of the first against the second

MIX_SHAPE = (512, 512, 512)
MIX_STEPS = 10


MIX_CONTRAST = 1e4  # permeability of the fracture voxels over that of the matrix's pores


def mixed_geometry(shape):
    """uint16 labels of the mixed-precision workload: the grey-level random field (corr 6)
    with 4 planar fractures of 1-3 voxel aperture (grey 0), classified on the GPU at the 20% /
    88% grey quantiles into Pore / Rock / Sulphide (the fractures fall below the lowest
    threshold: Pore). The fracture voxels get the intrinsic-permeability multiplier 1e4
    (fracture / matrix contrast 1e4); the flow-through boundary drives the pressure."""
    from leachingsim_gb300 import runtime as rt
    from leachingsim_gb300.geometry import grey_levels
    grey = grey_levels(shape, corr_len=6.0, seed=0, n_fractures=4)
    sub = grey[::4, ::4, ::4].ravel()
    thr = [int(np.quantile(sub, 0.2)), int(np.quantile(sub, 0.88))]
    lab = rt.geom_classify(grey, thr, [2, 3, 4], 2)
    kmult = np.where(grey == 0, MIX_CONTRAST, 1.0).astype(np.float32)
    return lab, kmult, thr


MIX_FIELDS = ("pressure", "flux_x", "flux_y", "flux_z", "conc", "acid", "precipitate", "label")


def mixed_params(fp64):
    from leachingsim_gb300._abi import BC_FLOW_I, PRESS_FP64, PRESS_MIXED, default_params
    base = dict(c_sat=1.0, D=1.0, kreac=1.0, bc_mode=BC_FLOW_I, p_inlet=FLOW_PIN, p_outlet=FLOW_POUT,
                acid_inlet=FLOW_ACID)
    if fp64:
        return default_params(press_solver=PRESS_FP64, press_rtol=1e-12, conc_rtol=1e-12, sat_rtol=1e-12, **base)
    return default_params(press_solver=PRESS_MIXED, press_rtol=PRESS_RTOL, conc_rtol=CONC_RTOL, sat_rtol=CONC_RTOL,
                          **base)


def mixed_run(lab, kmult, p, steps, keep=()):
    """steps accepted time steps from a fresh state; returns wall ms per step, the fields
    after the first step, after each step in `keep` and after the last, the context's device
    bytes and the solver iterations."""
    import torch
    from leachingsim_gb300.runtime import Context
    ctx = Context(lab.shape, label_bytes=2, params=p)
    ctx.upload("label", lab)
    ctx.upload("kmult", kmult)
    ctx.init_all()
    ctx.synchronize()
    times, iters, kept = [], [], {}
    t, n = 0.0, 0
    first = None
    for _ in range(steps):
        w0 = time.perf_counter()
        t, n, info = run_steps(ctx, t, n, 1, DT)
        ctx.synchronize()
        times.append((time.perf_counter() - w0) * 1e3)
        iters.append((info[0]["pressure"]["iterations"], info[0]["conc"]["iterations"], info[0]["leached"]))
        if first is None:  # after the first (cold) step, outside the timed step
            first = {f: ctx.download(f, padded=f != "label").copy() for f in MIX_FIELDS}
        if n in keep:
            kept[n] = {f: ctx.download(f, padded=f != "label").copy() for f in MIX_FIELDS}
    out = {f: ctx.download(f, padded=f != "label").copy() for f in MIX_FIELDS}
    mem = ctx.device_bytes()
    ctx.close()
    torch.cuda.synchronize()
    return times, (first, out), mem, iters, kept


def mixed_arm(args):
    import torch
    shape = tuple(int(v) for v in args.shape.split(",")) if args.shape else MIX_SHAPE
    steps = MIX_STEPS  # ten steps per precision (the first a cold step)
    t0 = time.time()
    lab, kmult, thr = mixed_geometry(shape)
    log(f"mixed: geometry {shape} in {time.time() - t0:.1f}s, labels {np.bincount(lab.ravel()).tolist()}, "
        f"fracture voxels {int((kmult > 1).sum())}")
    cpu_steps = max(0, args.mixed_cpu_steps)
    with ClockSampler(0) as clk:
        tm, fm, mem, im, km = mixed_run(lab, kmult, mixed_params(False), steps, keep=(cpu_steps,))
    tf, ff, _, iff, _ = mixed_run(lab, kmult, mixed_params(True), steps)

    vel = lambda f: np.concatenate([f[k].ravel() for k in ("flux_x", "flux_y", "flux_z")])  # noqa: E731

    def errors(a, b):
        return {"pressure": rel_l2(a["pressure"], b["pressure"]), "velocity": rel_l2(vel(a), vel(b)),
                "conc": rel_l2(a["conc"], b["conc"]), "acid": rel_l2(a["acid"], b["acid"]),
                "precipitate_abs": float(np.abs(a["precipitate"] - b["precipitate"]).max()),
                "label_mismatches": int(np.count_nonzero(a["label"] != b["label"]))}

    err = {"first_step": errors(fm[0], ff[0]), "last_step": errors(fm[1], ff[1])}
    cpu = None
    if cpu_steps > 0:
        # the FP64 oracle (CPU, production mode at tight tolerances) from the same labels
        from oracle import oracle as om
        po = mixed_params(True)
        threads = cpu_threads()
        o = om.Oracle(shape, label_bytes=2, params=po, mode=om.SOLVE_PRODUCTION, threads=threads)
        o.set_solver(om.SOLVE_PRODUCTION, rtol=1e-12)
        o.load_labels(lab)
        o.set("kmult", kmult)
        o.init_all()
        w0 = time.perf_counter()
        t = 0.0
        for _ in range(cpu_steps):
            ok, _ = o.step(t, DT)
            if not ok:
                raise RuntimeError("oracle step failed")
            t += DT
        wall = time.perf_counter() - w0
        of = {f: o.get(f, padded=f != "label") for f in MIX_FIELDS}
        o.close()
        cpu = {"steps": cpu_steps, "wall_s": round(wall, 1), "cores": threads,
               "mixed_vs_oracle": errors(km[cpu_steps], of),
               "note": ("the mixed-precision GPU fields after the first steps against the CPU oracle's (FP64, "
                        "multigrid-PCG pressure and GMRES transport to rtol 1e-12) from the same labels")}
    warm_m = statistics.median(tm[1:])
    warm_f = statistics.median(tf[1:])
    vox = lab.size
    total = torch.cuda.get_device_properties(0).total_memory
    c5 = 1024 * 1024 * 768
    return {"metric": f"time-steps/s at {shape[0]}x{shape[1]}x{shape[2]} uint16, mixed precision",
            "value": round(1e3 / warm_m, 4), "unit": "time-steps/s", "n_gpus": 1, "steps": steps - 1,
            "warmup": 1, "ms_per_step": round(warm_m, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64/f32", "data": "synthetic",
            "config": {"workload": f"{shape[0]}x{shape[1]}x{shape[2]} uint16 grey-level random field "
                                   "(corr 6) with 4 planar fractures of 1-3 voxel aperture, classified at the "
                                   "20% / 88% grey quantiles -> Pore / Rock / Sulphide (fractures: Pore with "
                                   f"intrinsic permeability x{MIX_CONTRAST:g}, contrast {MIX_CONTRAST:g} to the "
                                   "matrix), flow-through pressure (P = 1 at z = 0, 0 at z = max), acid 1 "
                                   "flowing in, dt 1, D 1, kreac 1, csat 1; mixed: FP32 inner MG-FCG / BiCGStab "
                                   "with FP64 refinement to pressure rtol 1e-8, transport 1e-6; fp64: FP64 "
                                   "inner MG-PCG to pressure rtol 1e-12, transport 1e-12",
                       "thresholds": thr, "l2": "working set > L2"},
            "first_step_ms": {"mixed": round(tm[0], 3), "fp64": round(tf[0], 3)},
            "fp64_ms_per_step": round(warm_f, 3),
            "iterations": {"mixed": im, "fp64": iff},
            "rel_l2_vs_fp64": err,
            "vs_cpu_oracle": cpu,
            "memory": {"device_bytes": mem, "bytes_per_voxel": round(mem / vox, 1),
                       "gpu_total_bytes": int(total),
                       "projected_1024x1024x768_bytes": int(mem / vox * c5),
                       "fits_1024x1024x768": bool(mem / vox * c5 < total)},
            "clocks": clk.summary(),
            "e2e": None}


# ---------------------------------------------------------------------------
# The learned preconditioner over a long run: the flow-through model on the workload's grid,
# acid flowing in so that dissolution changes the permeability every step.

C4_STEPS = 200


def c4_arm(args):
    """tmax = 200 steps (dt 1) of the flow-through model at 338x338x283 from the same fresh
    state, once per pressure solver: the learned coarse solver inside the flexible CG with the
    plain cycle as fallback (press_solver LEARNED), the plain mixed-precision K-cycle FCG, and
    the plain FP64 multigrid-PCG; per arm the pressure solve's device time per step (assembly,
    setup, inner and refinement timers), its iterations, the fallbacks and the whole run's
    steps/s."""
    import torch
    from leachingsim_gb300 import learned as L
    from leachingsim_gb300._abi import PRESS_FP64, PRESS_LEARNED, PRESS_MIXED
    from leachingsim_gb300.geometry import grf_geometry
    from leachingsim_gb300.runtime import Context
    torch.cuda.set_device(0)
    shape = tuple(int(v) for v in args.shape.split(",")) if args.shape else SHAPE
    steps = args.steps if args.steps != 40 else C4_STEPS
    lab, seed = grf_geometry(shape, air_inlet=False, **GEOM)
    pw = L.load_precond_weights()
    arms = {}
    for name, solver in (("learned_precond", PRESS_LEARNED), ("plain_mixed", PRESS_MIXED), ("plain_fp64", PRESS_FP64)):
        if solver == PRESS_LEARNED and pw is None:
            arms[name] = None
            continue
        p = flow_params("fp64" if solver == PRESS_FP64 else "mixed")
        p.press_solver = solver
        ctx = Context(shape, label_bytes=1, params=p)
        if solver == PRESS_LEARNED:
            ctx.set_precond_weights(pw)
        ctx.upload("label", lab)
        ctx.init_all()
        ctx.timing(True)
        per_step, its = [], []
        t, n = 0.0, 0
        ctx.synchronize()
        w0 = time.perf_counter()
        for _ in range(steps):
            ctx.timing_reset()
            t, n, info = run_steps(ctx, t, n, 1, DT)
            per_step.append(sum(ctx.timing_get(k)[0] for k in ("press_setup", "press_inner", "press_outer")))
            its.append(info[0]["pressure"]["iterations"])
        ctx.synchronize()
        wall = time.perf_counter() - w0
        fb = ctx.pressure_fallbacks()
        mineral = info[0]["budget"]["mineral"]
        ctx.timing(False)
        ctx.close()
        arms[name] = {"pressure_ms_per_step_mean": round(statistics.mean(per_step), 3),
                      "pressure_ms_per_step_median": round(statistics.median(per_step), 3),
                      "pressure_ms_first_step": round(per_step[0], 3),
                      "pressure_ms_total": round(sum(per_step), 1),
                      "iterations_mean": round(statistics.mean(its), 2), "iterations_first": its[0],
                      "fallbacks": fb, "steps_per_s": round(steps / wall, 3), "wall_s": round(wall, 1),
                      "mineral_after": mineral}
        log(f"c4 {name}: {arms[name]}")
    base = arms["plain_mixed"]["pressure_ms_total"]
    return {"metric": f"pressure solve ms per step over {steps} steps at {shape[2]}x{shape[1]}x{shape[0]}, "
                      "flow-through model with evolving porosity",
            "value": arms["learned_precond"]["pressure_ms_per_step_mean"] if arms["learned_precond"] else None,
            "unit": "ms/step", "higher_is_better": False, "n_gpus": 1, "steps": steps, "data": "synthetic",
            "config": {"workload": f"the workload's geometry (seed {seed}) without Air planes, P = {FLOW_PIN:g} / "
                                   f"{FLOW_POUT:g} on the Pore voxels of z = 0 / z = max, acid {FLOW_ACID:g} "
                                   f"flowing in, dt {DT:g}, {steps} steps from a fresh state per arm, pressure rtol "
                                   "1e-8"},
            "arms": arms,
            "learned_vs_plain_mixed": (round(arms["learned_precond"]["pressure_ms_total"] / base, 3)
                                       if arms["learned_precond"] else None)}


# ---------------------------------------------------------------------------
# The large single domain: 1024x1024x768 uint16 (805 M voxels) with the lean device layout.

LARGE_SHAPE = (768, 1024, 1024)  # (I, J, K) = (zext, yext, xext)
LARGE_POROSITY = 0.20
LARGE_FRACTURES = 8
LARGE_DT = 0.5


def large_geometry(shape, seed=0, porosity=LARGE_POROSITY, n_fractures=LARGE_FRACTURES, corr_len=6.0):
    """uint16 labels and the permeability multiplier of the large fractured workload, made on
    the GPU (a NumPy field of 805 M voxels takes minutes): a seeded Gaussian random field
    (corr_len, periodic), scaled to grey levels 0..65535, n_fractures planar fractures of 1-3
    voxel aperture at random orientations stamped in at grey 0, classified at the porosity /
    88% grey quantiles (of a 1/64 subsample) into Pore / Rock / Sulphide as
    ls_geom_classify does (label index = number of thresholds <= grey). Fracture voxels get
    the multiplier MIX_CONTRAST. Returns host arrays (labels, kmult, thresholds)."""
    import torch
    import torch.nn.functional as F
    dev = torch.device("cuda")
    gen = torch.Generator(device=dev)
    gen.manual_seed(seed)
    f = torch.randn(shape, generator=gen, device=dev, dtype=torch.float32)
    half = int(3.0 * corr_len + 0.5)
    x = torch.arange(-half, half + 1, device=dev, dtype=torch.float32)
    w = torch.exp(-0.5 * (x / corr_len) ** 2)
    w = (w / w.sum()).view(1, 1, -1)
    for axis in range(3):
        g = f.movedim(axis, 2).contiguous()
        a, b, n = g.shape
        g = F.pad(g.view(a * b, 1, n), (half, half), mode="circular")
        g = F.conv1d(g, w).view(a, b, n)
        f = g.movedim(2, axis).contiguous()
        del g
    lo, hi = f.min(), f.max()
    grey = ((f - lo) / (hi - lo).clamp_min(1e-30) * 65535.0).to(torch.int32)
    del f
    rng = np.random.Generator(np.random.PCG64(seed))
    I, J, K = shape
    ii = torch.arange(I, device=dev, dtype=torch.float32).view(I, 1, 1) - I / 2.0
    jj = torch.arange(J, device=dev, dtype=torch.float32).view(1, J, 1) - J / 2.0
    kk = torch.arange(K, device=dev, dtype=torch.float32).view(1, 1, K) - K / 2.0
    for _ in range(n_fractures):
        nrm = rng.standard_normal(3)
        nrm /= np.linalg.norm(nrm)
        offset = rng.uniform(-0.3, 0.3) * min(shape)
        ap = rng.integers(1, 4) / 2.0
        dist = ii * float(nrm[0]) + jj * float(nrm[1]) + kk * float(nrm[2]) - float(offset)
        grey.masked_fill_(dist.abs() <= ap, 0)
        del dist
    sub = grey[::4, ::4, ::4].flatten().float()
    thr = [int(torch.quantile(sub, porosity).item()), int(torch.quantile(sub, 0.88).item())]
    lab = (2 + (grey >= thr[0]).to(torch.int32) + (grey >= thr[1]).to(torch.int32)).to(torch.int16)
    kmult = torch.where(grey == 0, MIX_CONTRAST, 1.0).to(torch.float32)
    del grey
    out = lab.cpu().numpy().view(np.uint16), kmult.cpu().numpy(), thr
    del lab, kmult
    torch.cuda.empty_cache()
    return out


def large_arm(args):
    """Time steps of the large single domain with the lean layout (memory_mode MEM_LEAN): the
    first (cold) step and args.warmup - 1 more untimed, args.steps timed with the mixed solver,
    then args.steps with the plain FP64 multigrid-PCG pressure solver (same rtol) on the state
    they left; the device footprint (the pool's reserved high-water mark) and the host snapshot."""
    import torch
    from leachingsim_gb300._abi import BC_FLOW_I, MEM_LEAN
    from leachingsim_gb300.runtime import Context
    torch.cuda.set_device(0)
    shape = tuple(int(v) for v in args.shape.split(",")) if args.shape else LARGE_SHAPE
    t0 = time.time()
    lab, kmult, thr = large_geometry(shape)
    gen_s = time.time() - t0
    counts = np.bincount(lab[::4, ::4, ::4].ravel(), minlength=5).tolist()
    log(f"large: geometry {shape} in {gen_s:.1f}s, labels (1/64 sample) {counts}")

    def lp(solver):
        return params(solver, bc_mode=BC_FLOW_I, p_inlet=FLOW_PIN, p_outlet=FLOW_POUT, acid_inlet=FLOW_ACID,
                      memory_mode=MEM_LEAN)

    t1 = time.time()
    ctx = Context(shape, label_bytes=2, params=lp("mixed"))
    ctx.upload("label", lab)
    ctx.upload("kmult", kmult)
    del lab, kmult
    ctx.init_all()
    ctx.synchronize()
    setup_s = time.time() - t1
    stream = torch.cuda.ExternalStream(ctx.stream())
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ctx.timing(True)
    ctx.timing_reset()
    w0 = time.perf_counter()
    t, n, first = run_steps(ctx, 0.0, 0, 1, LARGE_DT)
    ctx.synchronize()
    cold_ms = (time.perf_counter() - w0) * 1e3
    t, n, _ = run_steps(ctx, t, n, max(args.warmup - 1, 0), LARGE_DT)

    def timed(solver, steps):
        nonlocal t, n
        ctx.set_params(lp(solver))
        ctx.timing_reset()
        torch.cuda.synchronize()
        ctx.synchronize()
        ev0.record(stream)
        t, n, infos = run_steps(ctx, t, n, steps, LARGE_DT)
        ev1.record(stream)
        ev1.synchronize()
        sec = ev0.elapsed_time(ev1) / 1e3
        tm = {k: round(ctx.timing_get(k)[0] / steps, 3)
              for k in ("press_setup", "press_inner", "press_outer", "transport", "dissolve", "snapshot")}
        return {"value": round(steps / sec, 4), "unit": UNIT, "ms_per_step": round(sec * 1e3 / steps, 3),
                "ms_per_step_by_phase": tm,
                "pressure_iterations": [i["pressure"]["iterations"] for i in infos],
                "pressure_rel_residual_max": max(i["pressure"]["rel_residual"] for i in infos),
                "leached_per_step": [i["leached"] for i in infos],
                "mineral_budget_last": infos[-1]["budget"]["mineral"]}

    with ClockSampler(0) as clk:
        mixed = timed("mixed", args.steps)
    plain = timed("fp64", max(1, min(args.steps, 2))) if not args.no_plain else None
    ctx.timing(False)
    vox = shape[0] * shape[1] * shape[2]
    peak = ctx.device_peak_bytes()
    host = ctx.host_bytes()
    ctx.close()
    total = torch.cuda.get_device_properties(0).total_memory
    return {"metric": f"time-steps/s at {shape[2]}x{shape[1]}x{shape[0]} uint16, lean layout",
            "value": mixed["value"], "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": mixed["ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64/f32", "data": "synthetic",
            "config": {"workload": f"{shape[2]}x{shape[1]}x{shape[0]} uint16 grey-level random field (corr 6, "
                                   f"made on the GPU) with {LARGE_FRACTURES} planar fractures of 1-3 voxel "
                                   f"aperture, classified at the {LARGE_POROSITY:g} / 0.88 grey quantiles -> "
                                   f"Pore / Rock / Sulphide (fractures: Pore with intrinsic permeability "
                                   f"x{MIX_CONTRAST:g}), flow-through pressure (P = {FLOW_PIN:g} at z = 0, "
                                   f"{FLOW_POUT:g} at z = max), acid {FLOW_ACID:g} flowing in, dt {LARGE_DT:g}, D 1, "
                                   "kreac 1, csat 1, pressure rtol 1e-8, transport rtol 1e-6; lean device layout",
                       "thresholds": thr, "memory_mode": "lean", "l2": "working set > L2"},
            "mixed": mixed, "plain_fp64": plain,
            "first_step_ms": round(cold_ms, 1), "first_step_pressure_iterations": first[0]["pressure"]["iterations"],
            "geometry_s": round(gen_s, 1), "setup_s": round(setup_s, 1),
            "memory": {"device_peak_bytes": int(peak), "bytes_per_voxel": round(peak / vox, 1),
                       "host_snapshot_bytes": int(host), "gpu_total_bytes": int(total)},
            "clocks": clk.summary(), "e2e": None}


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--solver", default="mixed", choices=["mixed", "fp64", "jacobi64"])
    ap.add_argument("--shape", default=None, help="override (I,J,K) for quick checks")
    ap.add_argument("--cpu-steps", type=int, default=CPU_STEPS)
    ap.add_argument("--no-flow", action="store_true", help="skip the flow-through model measurement")
    ap.add_argument("--mixed-cpu-steps", type=int, default=2,
                    help="--mixed: steps of the CPU oracle comparison (0: none)")
    ap.add_argument("--flow", action="store_true",
                    help="only the flow-through model measurement, as its own JSON line")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-cold", action="store_true", help="skip the separate cold pressure solves")
    ap.add_argument("--no-plain", action="store_true",
                    help="skip the steps with the plain FP64 pressure solver after the timed region")
    ap.add_argument("--nvtx", action="store_true",
                    help="wrap the first (cold) step in an NVTX range 'cold' and the timed steps in "
                         "'timed' (for ncu --nvtx-include cold/ or timed/)")
    ap.add_argument("--geometry", action="store_true",
                    help="time the geometry pre-processing pipeline instead (a separate JSON line)")
    ap.add_argument("--mixed", action="store_true",
                    help="mixed precision against FP64 settings on the 512^3 uint16 fractured geometry "
                         "(a separate JSON line)")
    ap.add_argument("--large", action="store_true",
                    help="the 1024x1024x768 uint16 fractured domain with the lean device layout, mixed "
                         "precision against the plain FP64 pressure solver (a separate JSON line)")
    ap.add_argument("--c4", action="store_true",
                    help="200 steps of the flow-through model with the learned preconditioner against the "
                         "plain solvers (a separate JSON line)")
    args = ap.parse_args()
    if args.c4:
        print(json.dumps(c4_arm(args)), flush=True)
        return
    if args.large:
        if args.steps == 40:
            args.steps = 3  # the default count is for the 338x338x283 workload
        print(json.dumps(large_arm(args)), flush=True)
        return
    if args.geometry:
        print(json.dumps(geometry_arm(args)), flush=True)
        return
    if args.mixed:
        print(json.dumps(mixed_arm(args)), flush=True)
        return
    if args.flow:
        import torch
        torch.cuda.set_device(0)
        shape = tuple(int(v) for v in args.shape.split(",")) if args.shape else SHAPE
        with ClockSampler(0) as clk:
            fl = flow_run(args, shape, 1, torch.cuda.synchronize)
        fl.update({"value": fl["mixed"]["value"], "unit": UNIT, "n_gpus": 1, "higher_is_better": True,
                   "ms_per_step": fl["mixed"]["ms_per_step"], "scaling": "weak", "vs_baseline": None,
                   "dtype": "f64/f32", "data": "synthetic", "config": {"workload": fl["workload"]},
                   "clocks": clk.summary(), "e2e": None})
        print(json.dumps(fl), flush=True)
        return
    ws, rank, local = dist_env()
    if args.warmup < 3 and args.impl == "ours":
        log("note: fewer than 3 warm-up steps")
    if args.impl == "reference":
        line = reference_arm(args, ws, rank)
    else:
        line = gpu_arm(args, ws, rank, local)
    if line is not None:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
