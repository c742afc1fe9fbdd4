#!/usr/bin/env python
"""Benchmark of the GB300 projection step on the NACA 0012 MAC workload.

Workload (the metric's configuration): MAC grid 2048x512, NACA 0012 at 10 deg
(chord 256 cells, leading edge at cell (400, 256)), Re = 1000, Smagorinsky LES
C_s = 0.17, dt from CFL 0.5 on the device, pressure solved to a 1e-6 relative
residual (FP64 norm) by the converging multigrid.  One "step" is one full
projection step (LES, RK3 predictor, divergence, pressure solve, correction,
boundary conditions).

Arms on the GPU (whole step captured in one CUDA graph each):
  nn       aj_step_nn: the learned warm start (trained weights in
           aerojax_gb300/weights) corrects the double-FP32 extrapolation of the
           last two pressures, then the converging multigrid
  extrap   aj_step with the extrapolated warm start alone
  prev     aj_step warm-started from the previous step's FP32 pressure (the
           "without network" baseline of the learned warm start)
  plain    the plain GPU multigrid step: zero initial guess, same tolerance
value = cell-steps/s of `nn` (the metric's arm); the others are reported in
config.arms.

`python bench.py --impl reference` times the same workload and method on the
host cores: the oracle's NumPy restatement (the reference's GUI step, the
converging multigrid to the same tolerance, the same extrapolation and
network), one replica per core, run concurrently (oracle/method_np.py); the
reference's own V-cycle (5 cycles) is reported beside it.  The reference
itself is JAX and cannot be installed here.  The GPU line's cpu_baseline is
the same restatement started from the GPU's developed state, and its
parity_sample checks one step of the method's arm against the FP64 oracle.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mcell-steps/s at 2048×512 FP32, NN-warm-start+MG vs plain MG at equal div tol"
UNIT = "Mcell-steps/s"
FLUSH_BYTES = 256 << 20          # larger than the 126 MB L2
NN_FACTOR = 8                    # network grid 256x64 at 2048x512
# DRAM bytes of one k_cv_up0 launch at 2048x512 from an ncu capture
TRAFFIC_UP0 = 22080256


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="naca",
                    choices=["naca", "ensemble", "tri4096", "post", "adjoint", "parity"],
                    help="naca: the metric's workload (default); ensemble: 64 cylinder "
                         "channels of uneven sizes in one graph launch; tri4096: the "
                         "4096x2048 three-cylinder dynamic-LES flow")
    ap.add_argument("--nx", type=int, default=2048)
    ap.add_argument("--ny", type=int, default=512)
    ap.add_argument("--cpu-sample-steps", type=int, default=10)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--quick", action="store_true",
                    help="timed GPU arms only (no clock soak, e2e or CPU leg)")
    ap.add_argument("--profile", action="store_true",
                    help="warm-up and timed steps of the method arm only, then exit "
                         "(the command a kernel profiler wraps)")
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi sampled every 200 ms during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.idx)], stdout=subprocess.PIPE,
                stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, val in zip(names, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "samples": len(sm),
                "reasons": sorted(reasons)}


# ------------------------------------------------------------------ CPU arm
WEIGHTS_NACA = os.path.join(ROOT, "aerojax_gb300", "weights", "warmstart_naca0012_2048x512_f8.npz")
METHOD = ("learned warm start (4-level BF16 conv encoder-decoder on the 256x64 grid correcting "
          "the extrapolation p1 + (dt/dt1)(p1 - p2) of the last two pressures), then converging "
          "multigrid to a 1e-6 relative residual (FP64 norms)")


def bench_config(nx, ny):
    """The workload and method both arms run; identical in the two lines."""
    return {"workload": f"naca0012_{nx}x{ny}_mac_re1000_les", "nx": nx, "ny": ny, "grid": "mac",
            "les": "smagorinsky C_s=0.17", "dt": "CFL 0.5", "method": METHOD,
            "rel_residual_target": 1e-6,
            "l2": "GPU arm: flushed before every step (256 MiB write outside the timed events); "
                  "CPU arm: one replica per core, working set far above the caches"}


def cpu_replicas(nx, ny, steps, warmup, mode="nn", init=None):
    """The same step on the host cores: one replica of the oracle's
    restatement of the method (oracle/method_np.py) per core, run
    concurrently; returns (aggregate Mcell-steps/s, info)."""
    from oracle import method_np as M
    return M.run_replicas(nx, ny, mode, WEIGHTS_NACA if mode == "nn" else None, steps, warmup,
                          init=init)


def reference_arm(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    steps, warm = max(1, args.steps), max(0, args.warmup)
    val, info = cpu_replicas(args.nx, args.ny, steps, warm, "nn")
    # the reference's own algorithm (its V-cycle, 5 cycles, no convergence
    # target) on the same cores, for context
    rsteps = min(steps, 10)
    rval, rinfo = cpu_replicas(args.nx, args.ny, rsteps, min(warm, 2), "reference")
    sample = (f"{info['procs']} concurrent replicas x {steps} full {args.nx}x{args.ny} MAC steps "
              f"after {warm} warm-up steps from the seeded start ({info['seconds']:.1f} s), "
              f"NumPy restatement of the method (float32 predictor, float64 multigrid and network)")
    print(json.dumps({
        "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": args.gpus, "steps": steps,
        "warmup": warm, "ms_per_step": info["seconds"] / steps * 1e3 / info["procs"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "impl": "reference", "data": "synthetic (seeded NACA 0012 flow)",
        "config": bench_config(args.nx, args.ny),
        "cpu_baseline": {"value": val, "unit": UNIT, "cores": info["procs"], "kind": "port",
                         "sample": sample},
        "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "mg_cycles_mean": info["mg_cycles_mean"],
        "reference_algorithm": {
            "value": rval, "unit": UNIT, "cores": rinfo["procs"],
            "what": f"the reference's GUI step with its own V-cycle (5 cycles, no convergence "
                    f"target), {rsteps} steps per replica"},
    }))


# ------------------------------------------------------------------ GPU arm
def gpu_arm(args):
    import torch
    import aerojax_gb300 as aj
    from aerojax_gb300 import _lib, configs
    from aerojax_gb300 import nn as NNW
    from aerojax_gb300.build import build

    from aerojax_gb300 import replicas
    world, rank, local = replicas.dist_env()
    torch.cuda.set_device(local)
    replicas.init()
    build()
    dev = torch.device("cuda", local)
    L = _lib.lib()

    case = configs.naca_mac_2048x512(device=dev, nx=args.nx, ny=args.ny, mg_mode="converge",
                                     seed=rank)
    cells = args.nx * args.ny
    mask = case["mask"]
    flush = torch.empty(FLUSH_BYTES, dtype=torch.uint8, device=dev)

    tuned = []
    net = None
    if os.path.exists(NNW.WEIGHTS):
        net = NNW.WarmStartNet.load(NNW.WEIGHTS, device=dev)

    def make_arm(kind):
        """plain: zero initial guess; prev: the previous step's FP32 pressure;
        extrap: double-FP32 extrapolation of the last two solutions; nn: the
        extrapolation plus the network's correction (the metric's arm)."""
        from dataclasses import replace
        warm = {"plain": False, "prev": True, "extrap": "extrapolate", "nn": "extrapolate"}[kind]
        cfg = replace(case["cfg"], warm_start=warm, nn_factor=NN_FACTOR if kind == "nn" else 0)
        plan = aj.get_plan(cfg, dev)
        plan.prepare(mask)
        if not tuned:                       # the level-0 tile shape of this grid, once
            from aerojax_gb300.ensemble import autotune
            tuned.append(autotune(plan))
        bufs = [(case["u"].clone(), case["v"].clone(), torch.zeros((args.nx, args.ny), device=dev))
                for _ in range(2)]
        return plan, bufs

    def step(plan, kind, src, dst):
        if kind == "nn":
            NNW.run_step_nn(plan, net, src[0], src[1], mask, src[2], out=dst)
        else:
            aj.run_step(plan, src[0], src[1], mask, p_guess=src[2], out=dst)

    def run(plan, bufs, k, timed, kind):
        """k steps, ping-ponging two state buffers; per-step CUDA events."""
        st = torch.cuda.current_stream()
        times, cycles = [], []
        cur = 0
        for _ in range(k):
            src, dst = bufs[cur], bufs[1 - cur]
            flush.zero_()                               # evict the working set from L2
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            step(plan, kind, src, dst)
            e1.record(st)
            times.append((e0, e1))
            cur = 1 - cur
            if timed:
                cycles.append(plan.stats_buf.clone())
        torch.cuda.synchronize()
        per = [a.elapsed_time(b) for a, b in times]
        cyc = []
        for s in cycles:
            raw = _lib.AjStats.from_buffer_copy(bytes(s.cpu().numpy().tobytes()))
            cyc.append((raw.cycles, raw.rel_residual, raw.err))
        return sum(per), cyc, per

    barrier = replicas.barrier
    max_over_ranks = replicas.max_over_ranks

    def soak(plan, bufs, kind, seconds):
        t0 = time.perf_counter()
        while time.perf_counter() - t0 < seconds:
            run(plan, bufs, 20, False, kind)

    head = "nn" if net is not None else "extrap"
    if args.profile:
        plan, bufs = make_arm(head)
        run(plan, bufs, max(3, args.warmup), False, head)
        ms, cyc, _ = run(plan, bufs, args.steps, True, head)
        if rank == 0:
            print(json.dumps({"profile_steps": args.steps, "arm": head,
                              "ms_per_step": ms / args.steps,
                              "cycles": [c[0] for c in cyc], "errors": [c[2] for c in cyc]}))
        return

    results = {}
    clocks = ClockSampler(local)
    clk = None
    for kind in ("plain", "prev", "extrap", "nn"):
        if kind == "nn" and net is None:
            continue
        if kind == "prev" and args.quick:
            continue
        plan, bufs = make_arm(kind)
        run(plan, bufs, max(3, args.warmup), False, kind)
        barrier()
        sample_clocks = kind == head and not args.quick
        if sample_clocks:
            clocks.start()                      # sample clocks over >= 1.5 s of load
        soak(plan, bufs, kind, 0.0 if args.quick else 1.0)   # the same flow stage for every arm
        ms, cyc, per = run(plan, bufs, args.steps, True, kind)
        if sample_clocks:
            soak(plan, bufs, kind, 0.5)
            clk = clocks.stop()
        barrier()
        ms = max_over_ranks(ms)
        results[kind] = dict(ms=ms, cycles=cyc, plan=plan, bufs=bufs, per=per)

    def arm_summary(r):
        ms = r["ms"] / args.steps
        return {"value": replicas.throughput(cells, args.steps, r["ms"], world), "ms_per_step": ms,
                "mg_cycles_mean": statistics.mean(c[0] for c in r["cycles"]),
                "rel_residual_max": max(c[1] for c in r["cycles"]),
                "device_errors": sorted({c[2] for c in r["cycles"]}),
                # spread of this rank's per-step device times (CUDA events,
                # L2 flushed before each step)
                "step_ms": {"median": statistics.median(r["per"]), "min": min(r["per"]),
                            "max": max(r["per"]),
                            "stdev": statistics.stdev(r["per"]) if len(r["per"]) > 1 else 0.0}}

    arms = {k: arm_summary(r) for k, r in results.items()}
    meth = results[head]
    ms_step = meth["ms"] / args.steps
    value = replicas.throughput(cells, args.steps, meth["ms"], world)
    plain_value = arms["plain"]["value"]
    cyc_m = [c[0] for c in meth["cycles"]]
    plan = meth["plan"]
    bpc = step_bytes_per_cell(statistics.mean(cyc_m))
    hbm = 6800.0
    if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")):
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            hbm = float(json.load(f)["hbm_gbs"])
    step_roofline = {"bytes_per_cell": bpc, "bytes_per_step": bpc * cells,
                     "achieved_gbs": bpc * cells / (ms_step * 1e-3) / 1e9,
                     "frac_of_measured_hbm": bpc * cells / (ms_step * 1e-3) / 1e9 / hbm}
    launches = sum(int(L.aj_kernel_count(ctypes.byref(plan.params), c)) for c in cyc_m)

    # ---- a developed state of the method's arm for the CPU legs: two more
    # steps record the solve history, a third is the sampled step whose fields
    # are checked against the FP64 oracle (untimed)
    sample_in = None
    if rank == 0 and not args.no_cpu_baseline and not args.quick:
        sb = meth["bufs"]
        hist = []
        for k in range(3):
            src, dst = sb[k % 2], sb[1 - k % 2]
            if k == 2:
                sample_in = tuple(t.detach().cpu().numpy() for t in src[:2])
            step(plan, head, src, dst)
            st_k = plan.stats()
            hist.append((dst[2].detach().cpu().numpy(), st_k["dt"], st_k))
        sample_out = tuple(t.detach().cpu().numpy() for t in sb[1])
        sample_dt, sample_stats = hist[2][1], hist[2][2]

    # ---- e2e: host buffers through aj_step_host (one graph launch: the H2D of
    # the step's inputs, the step, the D2H of its result)
    nxu, nyv = (args.nx + 1) * args.ny, args.nx * (args.ny + 1)
    pin = lambda t: t.detach().cpu().pin_memory()
    h_in = [pin(meth["bufs"][0][0]), pin(meth["bufs"][0][1]), pin(meth["bufs"][0][2])]
    h_out = (torch.empty_like(h_in[0]).pin_memory(), torch.empty_like(h_in[1]).pin_memory(),
             torch.empty_like(h_in[2]).pin_memory())
    st = torch.cuda.current_stream()

    def e2e_steps(k):
        ev = []
        for _ in range(k):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            aj.run_step_host(plan, h_in[0], h_in[1], mask, h_in[2], h_out=h_out,
                             net=net if head == "nn" else None)
            e1.record(st)
            ev.append((e0, e1))
            torch.cuda.synchronize()                 # the host owns the result now
            for a, b in zip(h_in, h_out):
                a.copy_(b)
        return sum(a.elapsed_time(b) for a, b in ev)
    h2d = 4 * (nxu + nyv + cells)
    d2h = 4 * (nxu + nyv + cells)
    e2e = None
    if not args.quick:
        e2e_steps(3)
        barrier()
        e2e_ms = max_over_ranks(e2e_steps(args.steps)) / args.steps
        e2e = {"value": world * cells / (e2e_ms * 1e-3) / 1e6, "unit": UNIT,
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h}

    # ---- roofline: the dominant kernel timed alone (events on the launch stream)
    roof = roofline(args, plan, meth["bufs"][0], mask, flush, L)

    if rank != 0:
        replicas.finalize()
        return
    cpu = parity = None
    if sample_in is not None:
        cpu, parity = cpu_leg(args, mask.detach().cpu().numpy(), hist, sample_in, sample_out,
                              sample_dt, sample_stats)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded NACA 0012 flow; the solver generates every step)",
        "config": bench_config(args.nx, args.ny),
        "arms": arms,
        "speedup_vs_plain": value / plain_value,
        "autotuned_level0_tiles": tuned[0] if tuned else None,
        "step_roofline": step_roofline,
        "e2e_api": "aj_step_host: pinned host u, v, p in; u, v, p out; copies inside the "
                   "step's graph",
        "parallelism": "replicas only" if world > 1 else "single GPU",
        "roofline": roof,
        "cpu_baseline": cpu,
        "parity_sample": parity,
        "e2e": e2e,
        "gpu_launches": launches,
        "clocks": clk,
    }
    print(json.dumps(line))
    replicas.finalize()


def cpu_leg(args, mask, hist, sample_in, sample_out, sample_dt, sample_stats):
    """The CPU baseline and the parity sample (host only, after every GPU
    measurement).

    cpu_baseline: the oracle's restatement of the same method, one replica
    per host core, started from the GPU's developed state (velocities and the
    last two pressures), so that its solves see the same flow stage.

    parity_sample: one step of the method's arm against the FP64 oracle from
    the same input state - the maximum relative error of u, v, p against the
    exact step (pressure solved to 1e-12), beside the distance of the
    reference's own step evaluated in FP32, and the post-projection
    divergence of the GPU step, of the reference's own step (its V-cycle, 5
    cycles) and of the exact step."""
    import tempfile
    import numpy as np
    from oracle import ref_np as R
    from oracle import method_np as M
    nx, ny = args.nx, args.ny
    with tempfile.TemporaryDirectory() as tmp:
        init = os.path.join(tmp, "state.npz")
        np.savez(init, u=sample_in[0], v=sample_in[1], p1=hist[1][0], dt1=hist[1][1],
                 p2=hist[0][0], dt2=hist[0][1])
        steps = 3
        val, info = cpu_replicas(nx, ny, steps, 1, "nn", init=init)
    cpu = {"value": val, "unit": UNIT, "cores": info["procs"], "kind": "port",
           "sample": f"{info['procs']} concurrent replicas x {steps} full {nx}x{ny} MAC steps "
                     f"after 1 warm-up step from the GPU's developed state ({info['seconds']:.1f} "
                     f"s; {info['mg_cycles_mean']} V-cycles per solve), NumPy restatement of the "
                     "method", "mg_cycles_mean": info["mg_cycles_mean"]}
    case = M.naca_case(nx, ny)
    u0, v0 = (a.astype(np.float64) for a in sample_in)
    m = mask.astype(np.float64)
    kw = dict(sdf=None, dx=case["dx"], dy=case["dy"], nu=case["nu"], U_inf=1.0, grid_type="mac",
              use_les=True, les_model="smagorinsky", smagorinsky_constant=0.17,
              brinkman_eta=1e-4)
    ex = R.step_gui(u0, v0, m, sample_dt, mg=R.MGConfig(mode="converge", rtol=1e-12,
                                                         max_cycles=80), **kw)
    f = np.float32
    kw32 = {k: (f(x) if isinstance(x, float) else x) for k, x in kw.items()}
    r32 = R.step_gui(u0.astype(f), v0.astype(f), m.astype(f), f(sample_dt),
                     mg=R.MGConfig(mode="converge", rtol=1e-12, max_cycles=80), **kw32)
    ref = R.step_gui(u0, v0, m, sample_dt, v_cycles=5, **kw)

    def rel(a, b):
        return float(np.max(np.abs(np.asarray(a, np.float64) - b)) / max(np.max(np.abs(b)), 1e-300))

    def div(u, v):
        d = R.divergence_staggered(np.asarray(u, np.float64), np.asarray(v, np.float64),
                                   case["dx"], case["dy"])
        return float(np.sqrt(np.sum(d * d) * case["dx"] * case["dy"]))
    parity = {
        "what": "one step of the method's arm from a developed state against the FP64 oracle "
                "(max |x - x_exact| / max |x_exact|)",
        "max_rel_err": {k: rel(g, e) for k, g, e in zip("uvp", sample_out, ex)},
        "fp32_reference_max_rel_err": {k: rel(g, e) for k, g, e in zip("uvp", r32, ex)},
        "post_projection_divergence_l2": {"gpu": div(*sample_out[:2]), "exact": div(*ex[:2]),
                                          "reference_step_5_vcycles": div(*ref[:2])},
        "rel_residual": sample_stats["rel_residual"], "mg_cycles": sample_stats["cycles"],
    }
    return cpu, parity


def step_bytes_per_cell(n_cycles, les=True):
    """Algorithmic bytes per cell of one projection step (FP32, each logical
    phase reading its inputs and writing its outputs once): RK3 stages
    20 + 28 + 32 = 80 B, LES 12 B plus 4 B per stage = 24 B, divergence and
    right-hand side 16 B, projection and boundary rows 24 B, and per V-cycle
    96 B (two pre and two post sweeps 2 x 12 B each, residual and restriction
    9 B, prolongation 9 B at the fine level times sum 4^-l = 1.328, plus the
    coarse solve and the residual norm)."""
    return 120 + (24 if les else 0) + 96 * n_cycles


def roofline(args, plan, state, mask, flush, L):
    """Times the converging multigrid's level-0 post-smoothing kernel alone
    (k_cv_up0: prolongation, 1 red-black sweep, double-FP32 pressure update
    and residual for the next cycle).  Per cell it reads r (4 B), e (4 B),
    the coarse correction (4 B / 4 cells), the double-FP32 pressure (8 B) and
    b (4 B), and writes the new pressure (8 B) and the next residual (4 B): 33
    algorithmic bytes per cell.  The L2 is flushed before every launch; the
    duration is the mean of 40 launches (the event timer ticks in steps of
    about 2 us on this part, so single launches are not resolved)."""
    import torch
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    peak, src = 6800.0, "fallback"
    if os.path.exists(peaks_path):
        with open(peaks_path) as f:
            peak, src = float(json.load(f)["hbm_gbs"]), "measured"
    st = torch.cuda.current_stream()
    which, bpc = 1, 33
    times = []
    for k in range(43):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        rc = L.aj_profile_kernel(ctypes.byref(plan.params), which, state[0].data_ptr(),
                                 state[1].data_ptr(), mask.data_ptr(), plan.ws.data_ptr(),
                                 plan.nbytes, st.cuda_stream)
        e1.record(st)
        if rc:
            return None
        if k >= 3:
            times.append((e0, e1))
    torch.cuda.synchronize()
    dur = statistics.mean(a.elapsed_time(b) for a, b in times) * 1e-3
    algo = bpc * args.nx * args.ny
    achieved = algo / dur / 1e9
    return {"kernel": "k_cv_up0 (level 0: prolongation + 1 red-black sweep + double-FP32 "
                      "update and residual)",
            "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_source": src, "traffic": TRAFFIC_UP0,
            "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch "
                              "(profiles/k_cv_up0_naca0012_mac_2048x512.md)",
            "algorithmic_bytes_per_launch": algo, "launch_us": dur * 1e6}


def side_workload(args):
    """Lines for the ensemble and the 4096x2048 workloads (not the metric's
    configuration): cell-steps/s of the GPU path, CUDA-event timed."""
    import torch
    from dataclasses import replace
    import aerojax_gb300 as aj
    from aerojax_gb300.build import build
    build()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    st = torch.cuda.current_stream()
    if args.workload == "ensemble":
        from aerojax_gb300 import ensemble as E
        ens = E.Ensemble(E.draw_instances(64, seed=0), device=dev)
        for _ in range(max(3, args.warmup)):
            ens.step()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(args.steps):
            ens.step()
        e1.record(st)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / args.steps

        def solve_stats(e, k=8):
            """cycles and final residuals of every instance over k more
            (untimed) steps: the device statistics hold the last step only"""
            out = []
            for _ in range(k):
                e.step()
                out.extend(e.stats())
            return out
        sts = solve_stats(ens)
        # the same physics on one grid of about the ensemble's total cell
        # count (4096x2048, Re 300, D 16 cells): what a batch could reach if
        # its instances ran as one large launch per phase
        big = E.Ensemble([E.Instance(4096, 2048, 16.0, 0.15, 0.5, 300.0)], device=dev, seed=0)
        for _ in range(max(3, args.warmup)):
            big.step()
        torch.cuda.synchronize()
        b0, b1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        b0.record(st)
        for _ in range(args.steps):
            big.step()
        b1.record(st)
        torch.cuda.synchronize()
        big_ms = b0.elapsed_time(b1) / args.steps
        big_value = big.cells / (big_ms * 1e-3) / 1e6
        big_sts = solve_stats(big)
        print(json.dumps({
            "metric": "aggregate Mcell-steps/s, 64-instance cylinder-channel ensemble",
            "value": ens.cells / (ms * 1e-3) / 1e6, "unit": UNIT, "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "dtype": "f32", "data": "synthetic (seeded draws)",
            "config": {"workload": "ensemble64_cylinders", "cells_per_step": ens.cells,
                       "instances": 64, "graph_launches_per_step": 1,
                       "autotuned_tiles": {f"{k[0]}x{k[1]}": v for k, v in ens.tuned.items()},
                       "mg_cycles_mean": statistics.mean(s["cycles"] for s in sts),
                       "mg_cycles_max": max(s["cycles"] for s in sts),
                       "rel_residual_max": max(s["rel_residual"] for s in sts),
                       "solve_stats_over": "8 steps after the timed ones, every instance",
                       "l2": "working set above the L2 size (no flush)"},
            "one_grid_same_cells": {
                "what": "one 4096x2048 instance, same physics (WENO5, converging MG to 1e-6)",
                "value": big_value, "ms_per_step": big_ms,
                "mg_cycles_mean": statistics.mean(s["cycles"] for s in big_sts),
                "mg_cycles_max": max(s["cycles"] for s in big_sts),
                "ensemble_fraction": (ens.cells / (ms * 1e-3) / 1e6) / big_value}}))
        return
    if args.workload == "post":
        # the post-step epilogue (vorticity, divergence, speed and the dye step
        # in one kernel): 2048x512 MAC and 4096x2048 collocated, inputs larger
        # than L2 at the larger size; algorithmic bytes = read u, v, c + write
        # c_new, vorticity, divergence, speed
        out = {}
        for name, nx, ny, grid in (("mac_2048x512", 2048, 512, "mac"),
                                   ("collocated_4096x2048", 4096, 2048, "collocated")):
            g = torch.Generator(device=dev).manual_seed(0)
            mac = grid == "mac"
            u = torch.rand(((nx + 1) if mac else nx, ny), device=dev, generator=g)
            v = torch.rand((nx, (ny + 1) if mac else ny), device=dev, generator=g)
            c = torch.rand((nx, ny), device=dev, generator=g)
            outs = [torch.empty((nx, ny), device=dev) for _ in range(4)]
            from aerojax_gb300 import _lib
            from aerojax_gb300.solver import make_params, StepConfig
            prm = make_params(StepConfig(nx=nx, ny=ny, dx=1 / 64, dy=1 / 64, nu=1.0,
                                         grid_type=grid))
            L = _lib.lib()

            def call(s_):
                rc = L.aj_post_step(ctypes.byref(prm), u.data_ptr(), v.data_ptr(), c.data_ptr(),
                                    outs[0].data_ptr(), 1e-3, 1e-3, outs[1].data_ptr(),
                                    outs[2].data_ptr(), outs[3].data_ptr(), s_)
                assert rc == 0, rc
            for _ in range(max(3, args.warmup)):
                call(torch.cuda.current_stream().cuda_stream)
            # the launches in a CUDA graph, so that host overhead cannot pad the time
            graph = torch.cuda.CUDAGraph()
            with torch.cuda.graph(graph):
                for _ in range(10):
                    call(torch.cuda.current_stream().cuda_stream)
            graph.replay()
            torch.cuda.synchronize()
            reps = max(1, args.steps // 10)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            for _ in range(reps):
                graph.replay()
            e1.record(st)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / (10 * reps)
            nbytes = 4 * (u.numel() + v.numel() + c.numel() + 4 * nx * ny)
            out[name] = {"ms_per_call": ms, "value": nx * ny / (ms * 1e-3) / 1e6,
                         "achieved_gbs": nbytes / (ms * 1e-3) / 1e9,
                         "algorithmic_bytes": nbytes}
        big = out["collocated_4096x2048"]
        print(json.dumps({
            "metric": "Mcell/s of the post-step epilogue (diagnostics + dye step, one kernel)",
            "value": big["value"], "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": big["ms_per_call"], "higher_is_better": True,
            "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": "post_step_epilogue", "sizes": out,
                       "l2": "4096x2048 inputs above the L2 size (no flush); launches "
                             "replayed from a CUDA graph of 10"}}))
        return
    if args.workload == "adjoint":
        adjoint_workload(args, dev, st)
        return
    if args.workload == "parity":
        parity_workload(args, dev, st)
        return
    from aerojax_gb300 import configs
    from aerojax_gb300 import nn as NNW
    case = configs.tri_cyl_4096x2048(device=dev)
    net = NNW.WarmStartNet.load(NNW.WEIGHTS_TRI, device=dev) \
        if os.path.exists(NNW.WEIGHTS_TRI) else None
    out = {}
    for arm, warm in (("plain", False), ("extrap", "extrapolate"), ("nn", "extrapolate")):
        if arm == "nn" and net is None:
            continue
        plan = aj.get_plan(replace(case["cfg"], warm_start=warm,
                                   nn_factor=NN_FACTOR if arm == "nn" else 0), dev)
        plan.prepare(case["mask"], case["sdf"])
        u, v = case["u"].clone(), case["v"].clone()
        p = torch.zeros_like(u)

        def step(u, v, p):
            if arm == "nn":
                return NNW.run_step_nn(plan, net, u, v, case["mask"], p)
            return aj.run_step(plan, u, v, case["mask"], p_guess=p)
        for _ in range(max(3, args.warmup)):
            u, v, p = step(u, v, p)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        cyc = []
        for _ in range(args.steps):
            u, v, p = step(u, v, p)
            cyc.append(plan.stats_buf.clone())
        e1.record(st)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / args.steps
        from aerojax_gb300 import _lib
        c = [_lib.AjStats.from_buffer_copy(bytes(x.cpu().numpy().tobytes())).cycles for x in cyc]
        out[arm] = {"value": 4096 * 2048 / (ms * 1e-3) / 1e6, "ms_per_step": ms,
                    "mg_cycles_mean": statistics.mean(c)}
    head = "nn" if "nn" in out else "extrap"
    print(json.dumps({
        "metric": "Mcell-steps/s, 4096x2048 three-cylinder dynamic-LES step",
        "value": out[head]["value"], "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": out[head]["ms_per_step"],
        "higher_is_better": True, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": case["name"], "arms": out,
                   "l2": "working set (~1 GB) above the L2 size (no flush)"}}))


def parity_workload(args, dev, st):
    """The reference's own algorithm on the GPU: the GUI MAC step
    (step_handlers.py:62-301) with the reference multigrid, 5 V-cycles (the
    GUI default), on the 2048x512 NACA 0012 workload, configured like the
    CPU port that is timed beside it (Smagorinsky 0.17, eta 1e-4, CFL 0.5)."""
    import torch
    from dataclasses import replace
    import aerojax_gb300 as aj
    from aerojax_gb300 import _lib, configs
    nx, ny = args.nx, args.ny
    case = configs.naca_mac_2048x512(device=dev, nx=nx, ny=ny, mg_mode="parity")
    cfg = replace(case["cfg"], v_cycles=5, brinkman_eta=1e-4, nu_hyper_ratio=0.0,
                  warm_start=False)
    plan = aj.Plan(cfg, dev)
    plan.prepare(case["mask"])
    mask = case["mask"]
    bufs = [(case["u"].clone(), case["v"].clone(), torch.zeros((nx, ny), device=dev))
            for _ in range(2)]
    flush = torch.empty(FLUSH_BYTES, dtype=torch.uint8, device=dev)
    cur = [0]

    def step():
        src, dst = bufs[cur[0]], bufs[1 - cur[0]]
        aj.run_step(plan, src[0], src[1], mask, out=dst)
        cur[0] = 1 - cur[0]

    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()
    ev, cyc = [], []
    for _ in range(args.steps):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        step()
        e1.record(st)
        ev.append((e0, e1))
        cyc.append(plan.stats_buf.clone())
    torch.cuda.synchronize()
    ms = sum(a.elapsed_time(b) for a, b in ev) / args.steps
    cycles = [_lib.AjStats.from_buffer_copy(bytes(c.cpu().numpy().tobytes())).cycles for c in cyc]
    L = _lib.lib()
    kc = int(L.aj_kernel_count(ctypes.byref(plan.params), 0))
    cpu = None
    if not args.no_cpu_baseline and not args.quick:
        n = args.cpu_sample_steps
        cval, info = cpu_replicas(nx, ny, n, 1, "reference")
        cpu = {"value": cval, "unit": UNIT, "cores": info["procs"], "kind": "port",
               "sample": f"{info['procs']} concurrent replicas x {n} full {nx}x{ny} MAC steps "
                         f"({info['seconds']:.1f} s), NumPy float32 port of the reference GUI "
                         "step with 5 reference V-cycles"}
    print(json.dumps({
        "metric": "Mcell-steps/s, reference GUI step with the reference multigrid (5 V-cycles), "
                  f"{nx}x{ny} MAC",
        "value": nx * ny / (ms * 1e-3) / 1e6, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "dtype": "f32",
        "data": "synthetic (seeded NACA 0012 flow)",
        "config": {"workload": f"naca0012_{nx}x{ny}_mac_gui_parity_mg5", "v_cycles": 5,
                   "mg_cycles_mean": statistics.mean(cycles), "kernels_per_step": kc,
                   "l2": "flushed before every step (256 MiB write outside the timed events)"},
        "cpu_baseline": cpu,
        "gpu_launches": kc * args.steps}))


# algorithmic bytes per cell of one aj_step_vjp (RK3, one V-cycle, four
# coarser levels): each array read or written once per kernel, FP32
#   forward predictor: stage 1 reads u, v, chi, writes 2; stages 2, 3 read
#     the stage state, u, v, chi, write 2                              20+28+28
#   correction: reads gu, gv, mask, writes gu*, gv*, gdpx, gdpy            28
#   gradient transpose: reads gdpx, gdpy, gp, writes pbar                  16
#   level-0 multigrid: two sweep pairs (read 1, update b 2, write 1; the
#     down pair also reads the coarse b: 1/4), prolongation read 1 + 1/4  38
#   levels 1-4 of the V-cycle: a third of level 0 (1/4 + 1/16 + ...)      13
#   divergence transpose: reads b, mask, updates gu*, gv*                  24
#   output stage: reads gu*, gv*, mask, chi, u*, v*, writes 5 fields       44
#   three reversed stages: read slope 2, state 2, chi, update w1 2 and
#     den 1, write slope 2 (the last writes gu, gv, updates gsdf)   52+52+52
VJP_BYTES_PER_CELL = 20 + 28 + 28 + 28 + 16 + 38 + 13 + 24 + 44 + 3 * 52


def adjoint_workload(args, dev, st):
    """Reverse mode of step_pure (aj_step_vjp) on a 2048x512 collocated
    cylinder channel: RK3, one parity V-cycle (the defaults of the
    reference's differentiable rollout), gradients w.r.t. u, v, the SDF, nu
    and U_inf.  The forward step is timed beside it."""
    import torch
    from aerojax_gb300 import _lib
    from aerojax_gb300.adjoint import StepVjp, _config
    nx, ny, dx, dt = 2048, 512, 1.0 / 128, 2e-4
    cells = nx * ny
    g = torch.Generator(device=dev).manual_seed(0)
    X = (torch.arange(nx, device=dev, dtype=torch.float32)[:, None] + 0.5) * dx
    Y = (torch.arange(ny, device=dev, dtype=torch.float32)[None, :] + 0.5) * dx
    sdf = torch.sqrt((X - 0.28 * nx * dx) ** 2 + (Y - 0.5 * ny * dx) ** 2) - 0.08 * ny * dx
    mask = 1.0 - torch.sigmoid(-sdf / (0.5 * dx))
    u = 1.0 + 0.3 * torch.randn((nx, ny), device=dev, generator=g)
    v = 0.3 * torch.randn((nx, ny), device=dev, generator=g)
    op = StepVjp(_config(nx, ny, dx, dx, 1e-3, 1.0, dt, True), dev)
    op.prepare(mask, sdf)
    op.u_in.copy_(u)
    op.v_in.copy_(v)
    for t in op.g_in:
        t.copy_(torch.randn((nx, ny), device=dev, generator=g))
    flush = torch.empty(FLUSH_BYTES, dtype=torch.uint8, device=dev)
    L = _lib.lib()
    P = op.plan
    uo, vo, po = (torch.empty((nx, ny), device=dev) for _ in range(3))

    def fwd():
        rc = L.aj_step(ctypes.byref(P.params), op.u_in.data_ptr(), op.v_in.data_ptr(),
                       mask.data_ptr(), None, uo.data_ptr(), vo.data_ptr(), po.data_ptr(),
                       P.ws.data_ptr(), P.nbytes, P.stats_buf.data_ptr(), st.cuda_stream)
        assert rc == 0, rc

    def vjp():
        op(op.u_in, op.v_in, mask, op.g_in[0], op.g_in[1], op.g_in[2], stream=st)

    def timed(fn, k):
        ev = []
        for _ in range(k):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            fn()
            e1.record(st)
            ev.append((e0, e1))
        torch.cuda.synchronize()
        return sum(a.elapsed_time(b) for a, b in ev) / k

    for _ in range(max(3, args.warmup)):
        fwd()
        vjp()
    torch.cuda.synchronize()
    fwd_ms = timed(fwd, args.steps)
    vjp_ms = timed(vjp, args.steps)
    kc = int(L.aj_step_vjp_kernel_count(ctypes.byref(P.params)))
    # a gradient through a rollout, as grad_design_loss runs it
    # (solver/solver.py:34-114): the forward scan keeping the history, then the
    # reverse scan, through the public Python API (one graph launch per step
    # each, plus the staging copies); no L2 flush inside the rollout
    from aerojax_gb300 import adjoint as ADJ
    from aerojax_gb300.params import SimState
    n_roll = 50
    state = SimState(u=u, v=v, p=None, u_prev=None, v_prev=None, c=None, dt=dt, iteration=0)
    params = {"dx": dx, "dy": dx, "nu": 1e-3, "U_inf": 1.0, "sdf": sdf}
    ADJ.rollout_vjp(state, mask, params, 3, op.g_in[0], op.g_in[1])   # warm-up (graphs)
    torch.cuda.synchronize()
    r0, r1, r2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    r0.record(st)
    _, hist = ADJ.differentiable_rollout(state, mask, params, n_roll)
    r1.record(st)
    ADJ.rollout_vjp(state, mask, params, n_roll, op.g_in[0], op.g_in[1], history=hist)
    r2.record(st)
    torch.cuda.synchronize()
    roll_fwd_ms, roll_rev_ms = r0.elapsed_time(r1) / n_roll, r1.elapsed_time(r2) / n_roll
    hbm = 6800.0
    if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")):
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            hbm = float(json.load(f)["hbm_gbs"])
    gbs = VJP_BYTES_PER_CELL * cells / (vjp_ms * 1e-3) / 1e9
    cpu = None
    if not args.no_cpu_baseline and not args.quick:
        import numpy as np
        from oracle import adjoint_np as A
        h = lambda t: t.detach().cpu().numpy().astype(np.float64)
        t0 = time.perf_counter()
        A.step_pure_vjp(h(op.u_in), h(op.v_in), dt, h(mask), h(sdf), dx, dx, 1e-3, 1.0,
                        h(op.g_in[0]), h(op.g_in[1]), h(op.g_in[2]))
        el = time.perf_counter() - t0
        cpu = {"value": cells / el / 1e6, "unit": UNIT, "cores": 1, "kind": "port",
               "sample": f"one 2048x512 reverse-mode step ({el:.1f} s), NumPy FP64 oracle "
                         "(forward recomputation included)"}
    print(json.dumps({
        "metric": "Mcell-steps/s of the reverse-mode step_pure (aj_step_vjp), 2048x512",
        "value": cells / (vjp_ms * 1e-3) / 1e6, "unit": UNIT, "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": vjp_ms,
        "higher_is_better": True, "dtype": "f32", "data": "synthetic (seeded cylinder channel)",
        "config": {"workload": "step_pure_vjp_cylinder_2048x512", "rk": "rk3", "v_cycles": 1,
                   "gradients": ["u", "v", "sdf", "nu", "U_inf"],
                   "forward_ms_per_step": fwd_ms, "vjp_over_forward": vjp_ms / fwd_ms,
                   "kernels_per_vjp": kc, "algorithmic_bytes_per_cell": VJP_BYTES_PER_CELL,
                   "rollout": {"steps": n_roll, "forward_ms_per_step": roll_fwd_ms,
                               "reverse_ms_per_step": roll_rev_ms,
                               "gradient_mcell_steps_per_s":
                                   cells / ((roll_fwd_ms + roll_rev_ms) * 1e-3) / 1e6,
                               "api": "adjoint.differentiable_rollout + adjoint.rollout_vjp"},
                   "achieved_gbs": gbs, "frac_of_measured_hbm": gbs / hbm,
                   "l2": "flushed before every call (256 MiB write outside the timed events)"},
        "cpu_baseline": cpu,
        "gpu_launches": kc * args.steps}))


def main():
    args = parse()
    if args.impl == "reference":
        reference_arm(args)
    elif args.workload != "naca":
        side_workload(args)
    else:
        gpu_arm(args)


if __name__ == "__main__":
    main()
