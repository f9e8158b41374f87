"""Benchmark of the focused-ultrasound hot path (one JSON line on stdout).

Default workload: the plain FP32 Westervelt configuration (128x128x256 cells,
dx = 0.1875 mm, heterogeneous c, one relaxation process, 20-cell sponge, 1 MHz
10-cycle bowl burst, 3000 time steps).  One benchmark step = one complete
3000-time-step solve.  Metric: Westervelt Gcell-updates/s.

  value      K solves on K sessions whose inputs are already on the device,
             timed with CUDA events on the library's stream
  e2e        K calls of bd_westervelt_run through the C ABI with host buffers:
             c map and source tables uploaded, peak and energy maps read back
  roofline   algorithmic bytes of the step kernel (56 B/cell) / its event-timed
             duration, against the measured HBM copy bandwidth
  cpu_baseline  the CPU oracle (OpenMP, all host cores) on a bounded sample

--impl reference times the reference's own Westervelt kernels built for the
host (oracle/_ref) on the same grid (its two-layer physics), all host cores.
--impl reference-gpu times the reference's own CUDA kernels (W's step loop,
G's DPRK_step one thread per bubble; oracle/_ref/libbdref_gpu.so) beside this
library on the same problems (the comparison baseline of the speed-ups).
The default one-GPU line also carries the cfg3, cfg4, cfg5 and cfg2
summaries and the reference's own Westervelt and Gilmore kernels on the GPU
beside this library (--no-extra skips them).
--workload threshold-scale runs G's search over its whole table with capped
integrations.
--gpus N under torchrun: N independent replicas of the cfg1 solve (weak
scaling); the z-slab split of a solve across devices is checked as slabs of
one device in the tests.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

CFG1 = dict(nx=128, ny=128, nz=256, n_steps=3000)
BYTES_PER_CELL = 56          # p^n..p^{n-4} 20 B, p^{n+1} 4, R 12, c 4, peak 8, energy 8
METRIC = "Westervelt Gcell-updates/s"
UNIT = "Gcell-updates/s"
# dram__bytes_read.sum + dram__bytes_write.sum of one step-kernel launch on the
# cfg1 grid (ncu capture of tile variant 21, the wv_tma_pair_kernel the
# autotuner picks, in its peak-and-energy mode: 172,525,824 + 29,673,472)
NCU_TRAFFIC_BYTES = 202199296


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for l in self.lines:
            p = [x.strip() for x in l.split(",")]
            if len(p) < 8:
                continue
            try:
                sm.append(float(p[0]))
                smax.append(float(p[1]))
            except ValueError:
                continue
            for nm, v in zip(names, p[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return world, rank, local


def dist_max(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def cfg1_problem(precision=None, tile_variant=-1):
    from bubbledynamics_gb300 import abi, presets
    p = presets.cfg1(CFG1["nx"], CFG1["ny"], CFG1["nz"], CFG1["n_steps"],
                     precision=abi.BD_F32 if precision is None else precision)
    p.params.tile_variant = tile_variant
    return p


def cpu_baseline_port(sample_steps):
    """The CPU oracle on cfg1's grid for a few time steps, all host cores."""
    from bubbledynamics_gb300 import abi, presets
    from oracle.oracle import Oracle
    o = Oracle()
    p = presets.cfg1(CFG1["nx"], CFG1["ny"], CFG1["nz"], sample_steps, precision=abi.BD_F64)
    t = time.perf_counter()
    o.westervelt(p, want=("peak",))
    dt = time.perf_counter() - t
    cells = CFG1["nx"] * CFG1["ny"] * CFG1["nz"] * sample_steps
    return {"value": cells / dt / 1e9, "unit": UNIT, "cores": o.threads(), "kind": "port",
            "sample": "%d time steps of the 128x128x256 grid (FP64 oracle, OpenMP), %.1f s" % (sample_steps, dt)}


def reference_cpu(sample_steps):
    """The reference's own Westervelt kernels (W:62-236) built for the host,
    on a 128x128x256 grid with the reference's two-layer physics."""
    from bubbledynamics_gb300 import presets
    from oracle.oracle import RefLib
    k = presets.ref_W_constants()
    k["Nxy"] = CFG1["nx"]
    k["Nz"] = CFG1["nz"]
    r = RefLib()
    t = time.perf_counter()
    r.w_steps(k, sample_steps)
    dt = time.perf_counter() - t
    cells = CFG1["nx"] * CFG1["nx"] * CFG1["nz"] * sample_steps
    return cells / dt / 1e9, dt


def run_reference(args, world, rank):
    if rank != 0:
        return
    import multiprocessing
    cores = multiprocessing.cpu_count()
    try:
        from oracle import build as ob
        if ob.build_ref() is None:
            raise FileNotFoundError("reference kernel sections not available")
        kind = "reference"
        sample = 6
        for _ in range(args.warmup):
            reference_cpu(1)
        vals = []
        t0 = time.perf_counter()
        for _ in range(args.steps):
            v, dt = reference_cpu(sample)
            vals.append(v)
        wall = time.perf_counter() - t0
        value = statistics.median(vals)
        desc = ("%d time steps of W's Westervelt_space6 + source + Mur kernels and the 9-copy rotation "
                "(W:139-236, W:62-135, W:575-584) on a 128x128x256 grid, host build, OpenMP over blocks" % sample)
    except Exception as e:  # the reference build is unavailable: time the oracle port instead
        kind = "port"
        cb = cpu_baseline_port(6)
        value = cb["value"]
        wall = 0.0
        desc = "oracle port (reference build unavailable: %s)" % str(e).splitlines()[0]
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": wall * 1e3 / max(args.steps, 1), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "westervelt 128x128x256 (reference two-layer physics, CPU)", "grid": [128, 128, 256]},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": kind, "sample": desc},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_westervelt(args, world, rank, local):
    import torch
    from bubbledynamics_gb300 import api
    torch.cuda.set_device(local)
    ctx = api.Context(local)
    pk, pk_kind = peaks()
    ncell = CFG1["nx"] * CFG1["ny"] * CFG1["nz"]
    T = CFG1["n_steps"]
    # ---- device-resident solves (value)
    sessions = [ctx.westervelt_session(cfg1_problem(tile_variant=args.tile_variant))
                for _ in range(args.warmup + args.steps)]
    for s in sessions[: args.warmup]:
        s.advance(T)
    dist_barrier(world)
    torch.cuda.synchronize()
    l0 = ctx.kernel_launches()
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        dev_ms = []
        for s in sessions[args.warmup:]:
            s.advance(T)
            dev_ms.append(s.last_ms())
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    launches = ctx.kernel_launches() - l0
    dist_barrier(world)
    total_ms = sum(dev_ms)
    total_ms = dist_max(total_ms, world)
    value = world * ncell * T * args.steps / (total_ms * 1e-3) / 1e9
    for s in sessions:
        s.close()
    # ---- step kernel roofline: algorithmic bytes / event-timed step duration
    step_us = total_ms * 1e3 / (args.steps * T)
    achieved = BYTES_PER_CELL * ncell / (step_us * 1e-6) / 1e9
    roof = {"bound": "hbm", "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
            "frac": achieved / pk["hbm_gbs"], "traffic": NCU_TRAFFIC_BYTES,
            "algorithmic_bytes": BYTES_PER_CELL * ncell, "peak_kind": pk_kind}
    # ---- end to end through the C ABI with host buffers
    prob = cfg1_problem(tile_variant=args.tile_variant)
    cmap = prob.array("c_map")
    h2d = cmap.nbytes + prob.grid.nx * prob.grid.ny * (4 + 4 * 4 + 4) + T * (8 + 16 + 4)
    d2h = 2 * ncell * 4
    warm = ctx.westervelt(prob, want=("peak", "energy"))   # warm; the variant the tuner chose
    dist_barrier(world)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ctx.westervelt(prob, want=("peak", "energy"))
    torch.cuda.synchronize()
    e2e_s = dist_max(time.perf_counter() - t0, world)
    e2e = {"value": world * ncell * T * args.steps / e2e_s / 1e9, "unit": UNIT,
           "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)}
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_baseline_port(args.cpu_sample)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "cfg1 plain Westervelt FP32 128x128x256, 3000 time steps per step",
                   "grid": [128, 128, 256], "time_steps_per_step": T, "dx_mm": 0.1875, "relax_processes": 1,
                   "sponge_cells": 20, "tile_variant": int(warm["tile_variant"]),
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "l2": "inputs larger than L2 (about 170 MB of fields streamed per time step)"},
        "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "clocks": clk.summary(),
        "gpu_launches": int(launches),
    }
    if not args.no_extra and world == 1:
        # the other rows of the measurement ride on the one-GPU line; the
        # multi-GPU lines carry the replicated cfg1 solve alone
        line["adjoint"] = extra_row(adjoint_summary, ctx)
        line["cfg3"] = extra_row(cfg3_summary, ctx)
        line["cfg5"] = extra_row(cfg5_summary, ctx)
        line["gilmore"] = extra_row(gilmore_summary, ctx, with_cpu=not args.no_cpu)
        # the reference's own W and G kernels built for this GPU: W's step loop on
        # the cfg1 grid with its physics, G's DPRK_step on 2^15 cfg2 bubbles
        line["reference_gpu"] = extra_row(reference_gpu_summary, ctx)
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()


def extra_row(fn, *args, **kw):
    """One extra measurement row; an exception there is recorded in the row
    instead of losing the headline line."""
    try:
        return fn(*args, **kw)
    except Exception as e:
        msg = str(e).splitlines()[0] if str(e) else type(e).__name__
        return {"error": msg}


def adjoint_summary(ctx):
    """cfg4: forward solve vs loss + gradient, sqrt(N) checkpoints and whole history."""
    from bubbledynamics_gb300 import presets
    prob, loss = presets.cfg4()
    n = prob.params.n_steps
    fwd = ctx.westervelt(prob, want=("energy",))             # warm (autotune, allocation)
    fwd = ctx.westervelt(prob, want=("energy",))
    out = {"workload": "cfg4 adjoint FP32 192^3, 3 slabs, 256-element cap array, %d steps" % n,
           "forward_ms": fwd["elapsed_ms"]}
    for name, k in (("sqrtN", 0), ("history", -1)):
        loss.checkpoint_every = k
        L, gp, ga, tm = ctx.westervelt_adjoint(prob, loss)
        tot = tm["forward_ms"] + tm["recompute_ms"] + tm["backward_ms"]
        out[name] = {"total_ms": tot, "forward_ms": tm["forward_ms"], "recompute_ms": tm["recompute_ms"],
                     "backward_ms": tm["backward_ms"], "ratio": tot / fwd["elapsed_ms"]}
    out["backward_us_per_step"] = out["history"]["backward_ms"] * 1e3 / n
    out["loss"] = L
    return out


HEAT_BYTES_PER_CELL = 28    # theta read + write 8 B, Q 4 B, FP64 dose read + write 16 B


def cfg3_summary(ctx, n_spots=49):
    """cfg3 in full: the acoustic solve (25.2 M cells, CW until ten periods
    after the front crossed the box), the W -> T hand-off, and all 49 spiral
    spots of bioheat + CEM43 dose (2000 steps of 1 ms each, 98,000 steps)."""
    from bubbledynamics_gb300 import pipeline, presets
    pk, pk_kind = peaks()
    ac = presets.cfg3_acoustic()
    g = ac.grid
    ncell = g.nx * g.ny * g.nz
    t0 = time.perf_counter()
    res = pipeline.cfg3_run(ctx, acoustic=ac, n_spots=n_spots)
    wall = time.perf_counter() - t0
    n = ac.params.n_steps
    heat_steps = res["heat_steps"]
    heat_us = res["heat_ms"] * 1e3 / heat_steps
    achieved = HEAT_BYTES_PER_CELL * ncell / (heat_us * 1e-6) / 1e9
    return {
        "workload": "cfg3 liver heating, 256x256x384, FP32 Westervelt (%d steps) -> Q -> %d of 49 spots x 2000 "
                    "heat steps (FP32 dT, FP64 dose)" % (n, n_spots),
        "acoustic_ms": res["acoustic_ms"], "acoustic_gcells": ncell * n / (res["acoustic_ms"] * 1e-3) / 1e9,
        "heat_ms": res["heat_ms"], "heat_steps": heat_steps, "heat_us_per_step": heat_us,
        "heat_gcells": ncell / (heat_us * 1e-6) / 1e9,
        "heat_roofline": {"bound": "hbm", "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
                          "frac": achieved / pk["hbm_gbs"], "algorithmic_bytes": HEAT_BYTES_PER_CELL * ncell,
                          "peak_kind": pk_kind},
        "full_run_s": (res["acoustic_ms"] + res["heat_ms"]) * 1e-3,
        "focal_peak_mpa": float(res["peak"].max() / 1e6),
        "T_max_C": float(res["T"].max() - 273.15), "dose_max_min": float(res["dose"].max() / 60.0),
        "wall_s": wall,
    }


def cfg5_summary(ctx, n_steps=12000, n_bubbles=1 << 18, t_end=0.1e-6):
    """cfg5 in full (512x512x768, 2 relaxation processes, three tones, 12,000
    steps, the 9-frequency DFT over the last 10 us on the 200 planes around the
    focus); then n_bubbles bubbles at random focal-region points driven by the
    DFT-reconstructed local pressure for t_end."""
    from bubbledynamics_gb300 import pipeline, presets
    pk, pk_kind = peaks()
    prob = presets.cfg5(n_steps=n_steps)
    g = prob.grid
    p = prob.params
    ncell = g.nx * g.ny * g.nz
    # one session: the steps before the DFT window, then the window, timed apart
    s = ctx.westervelt_session(prob)
    s.advance(p.dft_start)
    out_us = s.last_ms() * 1e3 / p.dft_start
    s.advance(p.dft_len)
    win_ms = s.last_ms()
    r = s.finish(want=("dft", "peak"))
    s.close()
    # p ring 24 B + two relaxation processes 24 B + peak 8 B (no c map; the
    # energy accumulator only inside the window, +8 B, with the DFT's 16 B per
    # frequency on its planes)
    b_cell = 56
    dft_cells = (p.dft_z_hi - p.dft_z_lo) * g.nx * g.ny
    win_bytes = (b_cell + 8) * ncell + 16 * p.n_dft * dft_cells
    win_us = win_ms * 1e3 / p.dft_len
    out = {"workload": "cfg5 512x512x768 FP32, %d steps, 9-frequency DFT over the last 10 us (530 steps) "
                       "on %d planes; %d bubbles driven by the local field for %g s" % (n_steps, p.dft_z_hi - p.dft_z_lo,
                                                                                         n_bubbles, t_end),
           "run_s": (out_us * p.dft_start + win_ms * 1e3) * 1e-6,
           "us_per_step_outside_window": out_us, "gcells_outside_window": ncell / (out_us * 1e-6) / 1e9,
           "roofline_outside_window": {"achieved": b_cell * ncell / (out_us * 1e-6) / 1e9, "peak": pk["hbm_gbs"],
                                       "frac": b_cell * ncell / (out_us * 1e-6) / 1e9 / pk["hbm_gbs"],
                                       "unit": "GB/s", "algorithmic_bytes_per_cell": b_cell},
           "us_per_step_in_window": win_us,
           "roofline_in_window": {"achieved": win_bytes / (win_us * 1e-6) / 1e9, "peak": pk["hbm_gbs"],
                                  "frac": win_bytes / (win_us * 1e-6) / 1e9 / pk["hbm_gbs"], "unit": "GB/s"},
           "focal_peak_mpa": float(r["peak"].max() / 1e6)}
    b, _ = pipeline.bubbles_from_dft(prob, r["dft_re"], r["dft_im"], n_bubbles)
    res, ms = ctx.gilmore(presets.cfg2_medium(), b, presets.cfg2_ode(t_end=t_end))
    att = float(res["n_accept"].sum() + res["n_reject"].sum())
    out["bubbles"] = {"n": n_bubbles, "t_end_s": t_end, "ms": ms, "attempts_per_s": att / (ms * 1e-3),
                      "threshold_fraction": float(res["threshold"].mean()),
                      "R_max_over_R0_median": float(np.median(res["R_max"] / b["R0"]))}
    out["run_with_bubbles_s"] = out["run_s"] + ms * 1e-3
    return out


def gilmore_summary(ctx, n=1 << 20, t_end=0.004e-6, cpu_n=1 << 12, with_cpu=True):
    """cfg2 bubbles (all 2^20 by default) over a bounded window through two
    kernels: the persistent work-stealing fast path and the naive baseline,
    one thread per bubble in the reference's operation order (7 right-hand
    sides with their pow calls per attempt, G:212-318) at the same cfg2
    settings (phases, rtol 1e-8).  The CPU oracle runs the first cpu_n of them
    over the same window, all host cores.  (The fast arithmetic one thread per
    bubble is `--workload gilmore --schedule static`.)"""
    import numpy as np
    from bubbledynamics_gb300 import abi, presets
    med = presets.cfg2_medium()
    b = presets.cfg2_bubbles(1 << 20)[:n]
    out = {"workload": "cfg2 Gilmore FP64, %d of the 2^20 seeded bubbles, t = 0..%g s, rtol 1e-8" % (n, t_end)}
    if with_cpu:
        from oracle.oracle import Oracle
        orc = Oracle()
        bc = np.ascontiguousarray(b[:cpu_n])
        t0 = time.perf_counter()
        orc.gilmore(med, (abi.Bubble * len(bc)).from_buffer_copy(bc.tobytes()), presets.cfg2_ode(t_end=t_end))
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"bubbles_per_s": cpu_n / dt, "bubble_us_per_s": cpu_n * t_end * 1e6 / dt,
                               "cores": orc.threads(), "kind": "port",
                               "sample": "first %d bubbles, same window, FP64 oracle (OpenMP)" % cpu_n}
    for name, sched, ref in (("persistent", abi.BD_SCHEDULE_PERSISTENT, 0), ("naive_static", abi.BD_SCHEDULE_STATIC, 1)):
        o = presets.cfg2_ode(t_end=t_end)
        o.schedule = sched
        o.ref_arith = ref
        r, ms = ctx.gilmore(med, b, o)
        att = float(r["n_accept"].sum() + r["n_reject"].sum())
        out[name] = {"ms": ms, "bubbles_per_s": n / (ms * 1e-3), "attempts_per_s": att / (ms * 1e-3),
                     "bubble_us_per_s": n * t_end * 1e6 / (ms * 1e-3)}
        if name == "persistent":
            acc = r["n_accept"].astype(np.float64)
    out["accepted_steps"] = {"mean": float(acc.mean()), "max": float(acc.max())}
    out["speedup_vs_naive_static"] = out["naive_static"]["ms"] / out["persistent"]["ms"]
    return out


def reference_gpu_summary(ctx, w_steps=100, g_n=1 << 15, g_t_end=0.1e-6, gilmore=True):
    """The reference's own CUDA kernels (oracle/_ref/libbdref_gpu.so) against
    this library on the same problems: W's step loop on the cfg1 grid with the
    reference's two-layer physics, and G's DPRK_step one thread per bubble on
    cfg2 bubbles (zero phases, G's 1e-9 tolerances) over a short window."""
    import numpy as np
    from bubbledynamics_gb300 import abi, presets
    try:
        from oracle.oracle import RefGpuLib, ref_g_cfg
        rg = RefGpuLib()
    except Exception as e:
        return {"unavailable": str(e).splitlines()[0]}
    out = {}
    # ---- Westervelt, cfg1 grid, reference physics
    k = presets.ref_W_constants()
    k["Nxy"], k["Nz"] = CFG1["nx"], CFG1["nz"]
    ms_ref, _ = rg.w_steps(k, w_steps, warm=10)
    ncell = k["Nxy"] * k["Nxy"] * k["Nz"]
    ref_us = ms_ref * 1e3 / w_steps
    w = {"workload": "W step loop (Westervelt_space6 + source + Mur + 9 copies), 128x128x256, FP64, %d steps"
                     % w_steps,
         "reference_us_per_step": ref_us, "reference_gcells": ncell / (ref_us * 1e-6) / 1e9}
    for name, prec in (("ours_f64_us_per_step", abi.BD_F64), ("ours_f32_us_per_step", abi.BD_F32)):
        prob = presets.make_ref_W(k, prec)
        prob.params.q_mode = abi.BD_Q_NONE
        prob.params.n_dft = 0
        s = ctx.westervelt_session(prob)
        s.advance(10)
        s.advance(w_steps)
        w[name] = s.last_ms() * 1e3 / w_steps
        s.close()
    w["speedup_f64"] = ref_us / w["ours_f64_us_per_step"]
    w["speedup_f32"] = ref_us / w["ours_f32_us_per_step"]
    out["westervelt"] = w
    if not gilmore:
        return out
    # ---- Gilmore, one thread per bubble with G's DPRK_step
    med = presets.cfg2_medium()
    b = presets.cfg2_bubbles(1 << 20)[:g_n]
    A = b["a"][:, 0] * np.sqrt(3.0)
    f3 = b["f"][:, :3].copy()
    st, counts, ms_g = rg.g_forward(ref_g_cfg(med), b["R0"], A, f3, g_t_end, max_steps=10 ** 8)
    bz = b.copy()
    bz["phi"] = 0.0
    o = presets.cfg2_ode(t_end=g_t_end, atol=1e-9, rtol=1e-9)
    res, ms_o = ctx.gilmore(med, bz, o)
    out["gilmore"] = {
        "workload": "first %d cfg2 bubbles, zero phases, t = 0..%g s, atol = rtol = 1e-9 (G:214-215)" % (g_n, g_t_end),
        "reference_ms": ms_g, "ours_ms": ms_o, "speedup": ms_g / ms_o,
        "reference_steps_mean": float(counts.mean()), "ours_steps_mean": float(res["n_accept"].mean()),
        "R_rel_diff_median": float(np.median(np.abs(res["R"] - st[:, 1]) / st[:, 1])),
    }
    return out


def run_gilmore(args):
    """cfg2 bubbles through one schedule: the case the Gilmore ncu captures run."""
    from bubbledynamics_gb300 import abi, api, presets
    ctx = api.Context(0)
    med = presets.cfg2_medium()
    b = presets.cfg2_bubbles(1 << 20)[:args.bubbles]
    o = presets.cfg2_ode(t_end=args.t_end)
    o.schedule = abi.BD_SCHEDULE_STATIC if args.schedule == "static" else abi.BD_SCHEDULE_PERSISTENT
    o.ref_arith = 1 if args.ref_arith else 0
    r, ms = ctx.gilmore(med, b, o)
    att = float(r["n_accept"].sum() + r["n_reject"].sum())
    print(json.dumps({"workload": "cfg2 Gilmore sample", "bubbles": args.bubbles, "t_end": args.t_end,
                      "schedule": args.schedule, "ref_arith": int(o.ref_arith), "ms": ms, "attempts": int(att),
                      "attempts_per_s": att / (ms * 1e-3)}), flush=True)
    ctx.close()


def run_threshold_scale(args):
    """G's threshold search over its whole table (27,775 combinations x 100
    radii = 2,777,500 items, G:498-520, G:457-460, G:573) with every
    integration capped at --max-steps accepted steps: every item climbs the
    0.1 MPa ladder to 10 MPa, so the run measures the search kernel's attempt
    rate and item coverage at the reference's scale (an uncapped search of the
    table is about 1.7e13 attempts)."""
    import numpy as np
    from bubbledynamics_gb300 import api, presets
    ctx = api.Context(0)
    combos = api.gilmore_combos()
    R0 = presets.ref_G_R0s()
    A, ms = ctx.gilmore_threshold(presets.ref_G_medium(), combos, R0, ref_arith=0, max_steps=args.max_steps)
    items = A.size
    attempts_lower_bound = items * 100 * args.max_steps      # every ladder that climbs to 10 MPa
    print(json.dumps({"workload": "G threshold search, whole table, integrations capped at %d steps" % args.max_steps,
                      "items": int(items), "ms": ms, "items_per_s": items / (ms * 1e-3),
                      "accepted_steps_per_s_lower_bound": attempts_lower_bound / (ms * 1e-3),
                      "every_item_written": bool(np.all(A > 0)),
                      "items_reaching_threshold_within_cap": int((A < 1e7).sum())}), flush=True)
    ctx.close()


def run_heat(args):
    """cfg3 heat steps on the 256x256x384 grid with a Gaussian focal source, one
    spot: the case the heat-kernel ncu captures run."""
    from bubbledynamics_gb300 import api, presets
    ctx = api.Context(0)
    ac = presets.cfg3_acoustic()
    th = presets.cfg3_thermal(ac, n_spots=1, steps_per_spot=args.time_steps)
    Q = presets.gaussian_focus_Q(ac.shape, (ac.meta.get("iz_focus", 287), 128, 128), (20.0, 4.0, 4.0), 1e7)
    r = ctx.heat(th.thermal, Q, th.traj)
    n = ac.grid.nx * ac.grid.ny * ac.grid.nz
    print(json.dumps({"workload": "cfg3 heat steps", "steps": int(r["steps_done"]), "ms": r["elapsed_ms"],
                      "gcells": n * r["steps_done"] / (r["elapsed_ms"] * 1e-3) / 1e9}), flush=True)
    ctx.close()


def run_adjoint(args):
    """cfg4 loss + gradient over --time-steps steps (whole history): the case the
    adjoint-kernel ncu captures run."""
    from bubbledynamics_gb300 import api, presets
    ctx = api.Context(0)
    prob, loss = presets.cfg4(n_steps=args.time_steps)
    if args.tile_variant >= 0:
        prob.params.tile_variant = args.tile_variant
    loss.checkpoint_every = -1
    L, gp, ga, tm = ctx.westervelt_adjoint(prob, loss)
    print(json.dumps({"workload": "cfg4 adjoint", "time_steps": args.time_steps, "timings_ms": tm}), flush=True)
    ctx.close()


def run_dft(args):
    """cfg5 physics on a 256x256x384 box with every step inside the 9-frequency
    DFT window: the case the DFT-path ncu captures run."""
    from bubbledynamics_gb300 import api, presets
    ctx = api.Context(0)
    prob = presets.cfg5(nx=256, ny=256, nz=384, n_steps=args.time_steps, window_steps=args.time_steps)
    if args.tile_variant >= 0:
        prob.params.tile_variant = args.tile_variant
    r = ctx.westervelt(prob, want=("dft",))
    print(json.dumps({"workload": "cfg5 box in the DFT window", "time_steps": args.time_steps,
                      "tile_variant": int(r["tile_variant"]),
                      "us_per_step": 1e3 * r["elapsed_ms"] / args.time_steps}), flush=True)
    ctx.close()


def run_step_kernel(args):
    """cfg1 time steps with plain launches and a fixed tile variant (or every
    TMA variant): microseconds per time step from the library's CUDA events.
    The case the ncu captures of the step kernel run."""
    from bubbledynamics_gb300 import api
    ctx = api.Context(0)
    variants = [args.tile_variant] if args.tile_variant >= 0 else list(range(8, 24))
    out = {}
    for v in variants:
        prob = cfg1_problem()
        prob.params.n_steps = args.time_steps
        prob.params.graph_chunk = -1
        prob.params.tile_variant = v
        r = ctx.westervelt(prob, want=("peak",))
        out[str(v)] = 1e3 * r["elapsed_ms"] / args.time_steps
    print(json.dumps({"workload": "cfg1 step kernel, plain launches", "time_steps": args.time_steps,
                      "us_per_step_by_variant": out}), flush=True)
    ctx.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference", "reference-gpu"])
    ap.add_argument("--workload", default="westervelt",
                    choices=["westervelt", "step-kernel", "gilmore", "heat", "adjoint", "dft", "threshold-scale"])
    ap.add_argument("--max-steps", type=int, default=100, help="threshold-scale workload: step cap per integration")
    ap.add_argument("--bubbles", type=int, default=1 << 16, help="gilmore workload: bubbles")
    ap.add_argument("--t-end", type=float, default=2e-6, help="gilmore workload: window [s]")
    ap.add_argument("--schedule", default="persistent", choices=["persistent", "static"])
    ap.add_argument("--ref-arith", action="store_true", help="gilmore workload: the reference's operation order")
    ap.add_argument("--time-steps", type=int, default=30, help="step-kernel workload: time steps per solve")
    ap.add_argument("--tile-variant", type=int, default=-1,
                    help="tile variant (-1: autotuned; the step-kernel workload then times every TMA variant)")
    ap.add_argument("--cpu-sample", type=int, default=60)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extra", action="store_true", help="skip the adjoint and Gilmore summaries")
    args = ap.parse_args()
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
    elif args.impl == "reference-gpu":
        if rank == 0:
            from bubbledynamics_gb300 import api
            ctx = api.Context(0)
            print(json.dumps({"impl": "reference-gpu", "comparison": reference_gpu_summary(ctx)}), flush=True)
            ctx.close()
    elif args.workload == "step-kernel":
        if rank == 0:
            run_step_kernel(args)
    elif args.workload in ("gilmore", "heat", "adjoint", "dft", "threshold-scale"):
        if rank == 0:
            {"gilmore": run_gilmore, "heat": run_heat, "adjoint": run_adjoint, "dft": run_dft,
             "threshold-scale": run_threshold_scale}[args.workload](args)
    else:
        run_westervelt(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
