#!/usr/bin/env python
"""Throughput of the 2D shallow-water RK2 step (cell-updates/s) on GB300.

Workload: the wet/dry hill terrain at 4096 x 4096 (Δ = 1 m; 64 seeded Gaussian
hills + 1e-3 slope; w = max(1.5, B_cell); Manning-type friction n = 0.03 via
friction_bsa2012; rain 1e-5 m/s; infiltration 2e-6 m/s; wall BCs; RK2; CFL
0.25), Float64 (the parity precision) with the Float32 variant reported
beside it. One step = one full RK2 step of every interior cell; a
cell-update = one interior cell advanced by one step.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

`value` is device throughput with the state resident in HBM (CUDA events on the
library's stream, max over ranks); `e2e` is the same metric through the public
API with the state copied from pinned host memory and back every step.
`--impl reference` times the reference's CPU path (the oracle's restatement of
it; VolumeFluxes.jl itself is Julia and no Julia toolchain exists on the box)
on all host cores. Multi-GPU runs are independent replicas (weak scaling).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "volumefluxes.jl_gb300"))
sys.path.insert(0, str(ROOT))

METRIC = "cell-updates/s"
WORDS_PER_CELL_STEP = 17        # stage 1: U0(3)+B(1) in, U1(3) out; stage 2: U1(3)+U0(3)+B(1) in, U2(3) out
WORDS_STAGE_PASS = 10           # the stage-2 share of those words
WORDS_FLUX_PASS = 7             # the stage-1 share


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000, help="timed RK2 steps (the configuration runs 1000)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--n", "--grid", dest="n", type=int, default=4096, help="side of the square grid")
    ap.add_argument("--dtype", choices=("f64", "f32"), default="f64")
    ap.add_argument("--no-variant", action="store_true", help="skip the Float32 variant")
    ap.add_argument("--no-faithful", action="store_true", help="skip the faithful-arithmetic Float64 variant")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--start-steps", type=int, default=0,
                    help="untimed steps on the measured simulator before the timed ones (profiling a developed flow)")
    ap.add_argument("--state-out", default=None,
                    help="save the measured simulator's interior state (after --start-steps) to this .npz and exit")
    ap.add_argument("--state-in", default=None, help="start from an interior state saved with --state-out")
    ap.add_argument("--cpu-budget", type=float, default=60.0,
                    help="seconds of oracle stepping the reference arm may spend (it runs min(K, budget) steps)")
    ap.add_argument("--no-ensemble", action="store_true", help="skip the batched-ensemble measurement")
    ap.add_argument("--ensemble-members", type=int, default=256)
    ap.add_argument("--ensemble-sample-every", type=int, default=8,
                    help="the plain baseline runs every m-th member (all of them), and so does a batch of that sample")
    ap.add_argument("--no-autotune", action="store_true", help="ensemble with the library's default granularity")
    ap.add_argument("--ensemble-wide-cells", type=int, default=None,
                    help="members with at least this many cells run the whole-grid kernels (default: autotuned)")
    ap.add_argument("--ensemble-endtime-cap", type=float, default=None,
                    help="cap every member's end time (small profiling runs only; the metric uses the full times)")
    ap.add_argument("--serving", action="store_true", help="measure the serving loop (the default; ~2 min)")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving loop")
    ap.add_argument("--serving-requests", type=int, default=24)
    ap.add_argument("--serving-rates", default="10,100,1000", help="Poisson arrival rates [req/s]")
    ap.add_argument("--serving-budget-gb", type=float, default=120.0)
    ap.add_argument("--serving-time-scale", type=float, default=0.1,
                    help="end times are U[10,600] s times this factor (1.0: the configuration's own times)")
    ap.add_argument("--adjoint", action="store_true", help="measure the differentiation workload (the default)")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the differentiation workload")
    ap.add_argument("--adjoint-n", type=int, default=512)
    ap.add_argument("--adjoint-steps", type=int, default=400)
    ap.add_argument("--adjoint-fd-dirs", type=int, default=64)
    return ap.parse_args()


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_table(tag: str):
    """Per-cell figures from the committed ncu summaries: lines '<tag>: <pass> <dtype> <value>'."""
    out = {}
    for f in sorted((ROOT / "profiles").glob("*.md")):
        for line in f.read_text().splitlines():
            if line.startswith(tag + ":"):
                parts = line.split()
                if len(parts) == 4:
                    out[(parts[1], parts[2])] = float(parts[3])
    return out


def kernel_names(dtype: str) -> dict:
    """Kernels the library runs for this precision (TMA-staged tiles for Float64,
    marching for Float32; VF_KERNELS and VF_TMA=0 override)."""
    variant = os.environ.get("VF_KERNELS", "tile" if dtype == "f64" else "march")
    t = "double" if dtype == "f64" else "float"
    if variant == "march":  # template arguments: rows per segment of each pass
        return {"flux": f"k_flux_march<{t},40>", "stage": f"k_stage_march<{t},24>"}
    if dtype == "f64" and os.environ.get("VF_TMA", "1") != "0":
        return {"flux": "k_flux_tma<double>", "stage": "k_stage2_tma<double>"}
    return {"flux": f"k_flux<{t}>", "stage": f"k_stage2<{t}>"}


# FP64 pipe peak: 2 DFMA-class thread instructions per clock per SM (ncu's
# sm__sass_thread_inst_executed_op_dfma_pred_on.peak_sustained on GB300), 152 SMs.
FP64_INST_PER_CLK_SM = 2.0
N_SMS = 152


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during a timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            time.sleep(0.15)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return None
        rows = [l.split(",") for l in open(self.path).read().strip().splitlines() if l.count(",") >= 8]
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].strip() == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows)}


def dist_setup(backend: str):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group(backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(world, x: float, device=None) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def oracle_sim(sc, real_bytes=8):
    from oracle import vf_oracle as O
    src = [(O.SRC_BOTTOM, 0.0), (O.SRC_CONST_RAIN, sc.rain_m_per_h), (O.SRC_CONST_INFIL, sc.infiltration_m_per_s)]
    o = O.OracleSim(nx=sc.nx, ny=sc.ny, extent=sc.extent, real_bytes=real_bytes, theta=sc.theta, sources=src,
                    friction=O.FRICTION_BSA2012, friction_Cz=sc.manning_n ** 2, stepper=O.STEPPER_RK2, cfl=sc.cfl,
                    B=sc.B)
    o.set_interior(sc.w0, sc.hu0, sc.hv0)
    return o


def cpu_rate(sc, warmup: int, steps: int | None, budget_s: float = 12.0, max_steps: int = 30,
             threads: int | None = None, o=None):
    """Oracle (the restated reference CPU path) on all host threads (or the
    given number): cell-updates/s.

    With steps=None the number of steps is chosen to fit budget_s (at most
    max_steps, at least one). `o` continues an existing oracle simulator."""
    from oracle import vf_oracle as O
    threads = O.set_threads(threads or os.cpu_count() or 1)
    o = o if o is not None else oracle_sim(sc)
    for _ in range(warmup):
        o.perform_step(math.inf)
    if steps is None:
        t0 = time.perf_counter()
        o.perform_step(math.inf)
        one = time.perf_counter() - t0
        steps = max(1, min(max_steps, int(budget_s / max(one, 1e-6))))
    t0 = time.perf_counter()
    for _ in range(steps):
        o.perform_step(math.inf)
    el = time.perf_counter() - t0
    return sc.nx * sc.ny * steps / el, threads, steps, el


def workload_name(sc, dtype):
    return (f"hills_wet_dry {sc.nx}x{sc.ny} RK2 {dtype.upper()}: 64 seeded Gaussian hills + 1e-3 slope, "
            f"w=max(1.5,B), Manning n=0.03 (bsa2012), rain 1e-5 m/s, infiltration 2e-6 m/s, wall BCs, CFL 0.25")


def bench_config(sc, dtype, world):
    """The `config` object of both arms' lines (identical keys and values)."""
    cells = sc.nx * sc.ny
    return {"workload": workload_name(sc, dtype), "nx": sc.nx, "ny": sc.ny, "seed": sc.meta["seed"],
            "parallelism": "replicas" if world > 1 else "single",
            "l2": "inputs larger than L2 (state %.0f MB per volume)" % (3 * cells * (8 if dtype == "f64" else 4) / 1e6)}


def run_reference(args):
    world, rank, local = dist_setup("gloo")
    if rank != 0:
        return
    from volumefluxes_sm103 import scenarios
    sc = scenarios.hills_wet_dry(args.n)
    value, threads, steps, el = cpu_rate(sc, args.warmup, None, budget_s=args.cpu_budget, max_steps=args.steps)
    sample = (f"{steps} full RK2 steps (of {args.steps} requested; time budget {args.cpu_budget:.0f} s) of the "
              f"{sc.nx}x{sc.ny} Float64 workload from its initial state after {args.warmup} warm-up steps")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": args.gpus,
        "steps": steps, "warmup": args.warmup, "ms_per_step": el / steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": bench_config(sc, "f64", world),
        "cpu_baseline": {"value": value, "unit": METRIC, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "VolumeFluxes.jl is Julia and no Julia toolchain exists on the box; the reference arm runs the "
                "oracle's C++ restatement of its CPU path (same passes, OpenMP over rows)",
    }
    print(json.dumps(line), flush=True)


FULL_STEPS = 1000        # the configuration's run length
FD_EPS = 1e-7            # central-difference step of the gradient check
DEVELOPED_STEPS = 20     # per-kernel timing window after the full run (the developed flow)


def _time_steps(sim, n):
    import ctypes as C
    import volumefluxes_sm103 as vf
    ms = C.c_float()
    vf._native.check(sim._lib, sim.handle, sim._lib.vf_time_steps(sim.handle, int(n), C.byref(ms)))
    return float(ms.value)


def _time_kernels(sim, n):
    import ctypes as C
    import volumefluxes_sm103 as vf
    mf, mst = C.c_float(), C.c_float()
    vf._native.check(sim._lib, sim.handle, sim._lib.vf_time_kernels(sim.handle, int(n), C.byref(mf), C.byref(mst)))
    return mf.value / n, mst.value / n


def _state(sim):
    import volumefluxes_sm103 as vf
    g = vf.current_interior_state(sim)
    return tuple(np.asarray(a, dtype=np.float64) for a in (g.h, g.hu, g.hv))


def measure_gpu(sc, dtype, args, world, local, arithmetic="reference"):
    """Device throughput of one precision (and Float64 arithmetic mode).

    headline: K steps back to back from the initial state (after W warm-up
    steps on a throwaway simulator), CUDA events on the library's stream.
    kernels: the same K steps on a second simulator with events between the
    two kernels of every step. full: when K < 1000 (the configuration's run)
    the 1000 steps on a third simulator. developed: per-kernel times of the 20
    steps after step 1000, the developed flow the ncu captures describe."""
    import volumefluxes_sm103 as vf
    real = np.float64 if dtype == "f64" else np.float32
    be = vf.SM103Backend(real, device=local, arithmetic=arithmetic)
    if args.warmup > 0:
        warm = sc.build(be)
        _time_steps(warm, args.warmup)
        warm.close()
    sim = sc.build(be)
    if args.start_steps > 0:
        _time_steps(sim, args.start_steps)
    if args.state_out:
        st = vf.current_interior_state(sim)
        np.savez(args.state_out, h=st.h, hu=st.hu, hv=st.hv)
        sys.exit(0)
    barrier(world)
    n0 = sim.launch_count()
    with Clocks(local) as clk:
        ms = _time_steps(sim, args.steps)
    launches = sim.launch_count() - n0
    barrier(world)
    ms_total = allmax(world, ms)
    out = {"sim": sim, "ms_total": ms_total, "launches": launches, "clocks": clk.summary(), "state": _state(sim)}
    prof = sc.build(be)
    if args.start_steps > 0:
        _time_steps(prof, args.start_steps)
    out["ms_flux"], out["ms_stage"] = _time_kernels(prof, args.steps)
    prof.close()
    fresh = args.start_steps == 0 and not args.state_in  # the timed window starts at the initial state
    if fresh and args.steps < FULL_STEPS:
        full = sc.build(be)
        out["full_ms"] = _time_steps(full, FULL_STEPS)
        out["full_state"] = _state(full)
    elif fresh and args.steps == FULL_STEPS:
        full = None
        out["full_ms"] = ms_total
        out["full_state"] = out["state"]
    else:
        full = None
    if "full_ms" in out:
        dev = full if full is not None else sim
        out["dev_flux"], out["dev_stage"] = _time_kernels(dev, DEVELOPED_STEPS)
        if full is not None:
            full.close()
    return out


def field_errors(got, ref):
    """Max-norm errors of (w, hu, hv) against a reference state: per field
    relative to the field's own max-norm, and relative to max |w|."""
    scale_w = float(np.abs(ref[0]).max())
    out = {}
    for name, a, b in zip(("w", "hu", "hv"), got, ref):
        d = float(np.abs(a - b).max())
        out[name] = {"max_abs": d, "rel_field": d / max(float(np.abs(b).max()), 1e-300), "rel_state": d / scale_w}
    return out


def e2e_rate(sim, steps: int):
    """Public API with host buffers: upload state (pinned), one step, download state (pinned)."""
    import volumefluxes_sm103 as vf
    g = sim.grid
    try:
        import torch
        bufs = [torch.empty((g.ny, g.nx), dtype=torch.float64 if sim.dtype == np.float64 else torch.float32,
                            pin_memory=True).numpy() for _ in range(3)]
    except Exception:
        bufs = [np.empty((g.ny, g.nx), dtype=sim.dtype) for _ in range(3)]
    view = vf.StateView(*(b.T for b in bufs))
    vf.current_interior_state(sim, out=view)
    t0 = time.perf_counter()
    for _ in range(steps):
        vf.set_current_state(sim, view)
        vf.perform_step(sim, math.inf)
        vf.current_interior_state(sim, out=view)
    el = time.perf_counter() - t0
    nbytes = 3 * g.nx * g.ny * sim.dtype.itemsize
    return g.nx * g.ny * steps / el, nbytes, nbytes, el


def roofline(sc, dtype, ms_flux, ms_stage, peak, peak_kind, traffic):
    e = 8 if dtype == "f64" else 4
    cells = sc.nx * sc.ny
    which, dom_ms, words = ("stage", ms_stage, WORDS_STAGE_PASS) if ms_stage >= ms_flux else \
        ("flux", ms_flux, WORDS_FLUX_PASS)
    alg = words * e * cells
    ach = alg / (dom_ms * 1e-3) / 1e9
    tb = traffic.get((which, dtype))
    return {
        "bound": "hbm", "kernel": kernel_names(dtype)[which], "achieved": ach, "peak": peak, "unit": "GB/s",
        "frac": ach / peak, "peak_kind": peak_kind, "traffic": (tb * cells) if tb is not None else None,
        "traffic_source": "ncu dram bytes per cell of a 3072^2 developed-flow capture, scaled to this launch"
                          if tb is not None else None,
        "algorithmic_bytes": alg, "launch_ms": dom_ms,
    }


def fp64_roofline(sc, ms_stage_developed, clk_mhz, inst):
    """Compute bound of the Float64 stage pass in the developed flow: FP64-pipe
    thread instructions per second against the pipe's peak. The instruction
    count per cell comes from the ncu capture of a developed-flow launch, so it
    is applied to the stage pass's time in the same flow state (the steps after
    step 1000), never to an early window (at rest, friction is skipped and far
    fewer instructions run)."""
    n = inst.get(("stage", "f64"))
    if n is None or ms_stage_developed is None:
        return None
    cells = sc.nx * sc.ny
    ach = n * cells / (ms_stage_developed * 1e-3)
    peak = FP64_INST_PER_CLK_SM * N_SMS * (clk_mhz or 2070.0) * 1e6
    return {"bound": "fp64_pipe", "kernel": kernel_names("f64")["stage"], "achieved": ach, "peak": peak,
            "unit": "FP64 thread-inst/s", "frac": ach / peak, "inst_per_cell": n, "launch_ms": ms_stage_developed,
            "window": f"the {DEVELOPED_STEPS} steps after step {FULL_STEPS} (developed flow)",
            "inst_source": "ncu DADD+DMUL+DFMA per cell of one stage-pass launch in the developed flow"}


def ensemble_workload(n):
    return (f"batched ensemble: {n} flood scenarios, Float32, square side log-uniform in [64,1024] (Δ = 1 m), "
            "8-32 seeded Gaussian hills (amplitude U[0.5,4] m, width U[50,400] m) + 1e-3 slope, uniform initial "
            "depth U[0,2] m, rain U[0,5e-5] m/s, Manning n U[0.01,0.08] (bsa2012), wall BCs, RK2, CFL 0.25, "
            "own CFL dt to an end time U[10,600] s each, depth_cutoff 8e-2 (examples/terrain.jl:92)")


def measure_ensemble(args, local):
    """The batched ensemble against the plain per-scenario drop-in on the same GPU.

    Batch: every member from its initial state to its end time in one vf_batch
    launch set, states resident on the device; latency of a member = time from
    the launch until the host sees its done flag. Measured on a sample (every
    m-th member, all of them): the plain drop-in, simulate_to_time per member
    one after the other, against the same members as a batch of their own.
    The plain figures for all members are extrapolated from the sample's mean
    time per member and labelled as estimates.
    """
    import volumefluxes_sm103 as vf
    from volumefluxes_sm103 import ensemble as E
    from volumefluxes_sm103 import scenarios as S
    real = np.float32
    specs = S.ensemble_specs(args.ensemble_members)
    scen = [S.ensemble_member(s) for s in specs]
    ends = [s.endtime if args.ensemble_endtime_cap is None else min(s.endtime, args.ensemble_endtime_cap)
            for s in specs]
    cells = np.array([sc.nx * sc.ny for sc in scen], dtype=np.float64)
    be = vf.SM103Backend(real, device=local)
    tuned, table = None, []
    if not args.no_autotune:
        probe = [sc.build(be) for sc in scen[::8]]
        tuned, table = E.autotune(probe, steps=60)
        for p in probe:
            p.close()
    if args.ensemble_wide_cells is not None:
        tuned = E.BatchOptions(**{**(tuned.__dict__ if tuned else {}), "wide_cells": args.ensemble_wide_cells})
    sims = [sc.build(be) for sc in scen]
    lib = sims[0]._lib
    n0 = sum(s.launch_count() for s in sims)
    done_at = [None] * len(sims)
    with Clocks(local) as clk:
        t0 = time.perf_counter()
        run = E.BatchRun(sims, ends, options=tuned)
        pending = set(range(len(sims)))
        while pending:
            for i in list(pending):
                if run.is_done(i):
                    done_at[i] = time.perf_counter() - t0
                    pending.discard(i)
            time.sleep(0.0005)
        res = run.finish()
        makespan = time.perf_counter() - t0
    launches = sum(s.launch_count() for s in sims) - n0
    steps = np.array([r.steps for r in res], dtype=np.float64)
    status = [E.STATUS_NAMES[r.status] for r in res]
    lat = np.array(done_at)
    batch = {
        "scenarios_per_s": len(sims) / makespan, "makespan_s": makespan,
        "cell_updates_per_s": float((cells * steps).sum() / makespan),
        "latency_s": {"p50": float(np.percentile(lat, 50)), "p95": float(np.percentile(lat, 95)),
                      "p99": float(np.percentile(lat, 99)), "max": float(lat.max())},
        "member_steps": {"min": int(steps.min()), "median": float(np.median(steps)), "max": int(steps.max()),
                         "total": int(steps.sum())},
        "status": {k: status.count(k) for k in sorted(set(status))},
        "gpu_launches": launches, "clocks": clk.summary(),
        "options": None if tuned is None else {k: v for k, v in tuned.__dict__.items() if v is not None},
        "autotune_top": [[{k: v for k, v in c.__dict__.items() if v is not None}, r] for c, r in table[:4]],
    }
    final_h = [vf.current_interior_state(x).h for x in sims[::args.ensemble_sample_every]]
    for x in sims:
        x.close()
    # the plain drop-in on a sample (every m-th member, all of them): one
    # simulate_to_time after the other, all arriving at once, served in index
    # order; and the same sample as a batch of its own
    m = args.ensemble_sample_every
    sample = list(range(0, len(scen), m))
    service, equal = [], 0
    for k, i in enumerate(sample):
        p = scen[i].build(be)
        t1 = time.perf_counter()
        vf.simulate_to_time(p, ends[i])
        service.append(time.perf_counter() - t1)
        equal += int(np.array_equal(vf.current_interior_state(p).h, final_h[k]))
        p.close()
    service = np.array(service)
    plain_lat = np.cumsum(service)
    sub = [scen[i].build(be) for i in sample]
    sub_done = [None] * len(sub)
    t0 = time.perf_counter()
    run = E.BatchRun(sub, [ends[i] for i in sample], options=tuned)
    pending = set(range(len(sub)))
    while pending:
        for i in list(pending):
            if run.is_done(i):
                sub_done[i] = time.perf_counter() - t0
                pending.discard(i)
        time.sleep(0.0005)
    run.finish()
    sub_make = time.perf_counter() - t0
    for x in sub:
        x.close()
    sub_lat = np.array(sub_done)

    def pct(a):
        return {"p50": float(np.percentile(a, 50)), "p95": float(np.percentile(a, 95)),
                "p99": float(np.percentile(a, 99)), "max": float(np.max(a))}

    sampled = {
        "members": f"{len(sample)} of {len(scen)} (every {m}th, all of them)",
        "plain_sequential": {"makespan_s": float(service.sum()), "scenarios_per_s": len(sample) / float(service.sum()),
                             "latency_s": pct(plain_lat),
                             "cell_updates_per_s": float((cells[sample] * steps[sample]).sum() / service.sum())},
        "batch": {"makespan_s": sub_make, "scenarios_per_s": len(sample) / sub_make, "latency_s": pct(sub_lat)},
        "speedup_scenarios_per_s": float(service.sum()) / sub_make,
        "bitwise_equal_plain_vs_batch": f"{equal} of {len(sample)}",
        "timing": "both arms measured: plain = simulate_to_time per member, one after the other, all arriving at "
                  "once (latency = finish time in index order); batch = the same members in one vf_batch launch set",
    }
    mean_t = float(service.mean())
    total_est = mean_t * len(scen)
    plain = {
        "scenarios_per_s_est": 1.0 / mean_t,
        "makespan_s_est": total_est,
        "latency_s_est": {"p50": 0.50 * total_est, "p95": 0.95 * total_est, "p99": 0.99 * total_est},
        "estimate": f"all {len(scen)} members one after the other, extrapolated from the measured sample's mean "
                    f"time per member ({mean_t:.2f} s)",
    }
    return {"workload": ensemble_workload(len(scen)), "dtype": "f32", "members": len(scen), "batch": batch,
            "sampled_measured": sampled, "plain_sequential_estimated": plain,
            "speedup_scenarios_per_s_est": batch["scenarios_per_s"] / plain["scenarios_per_s_est"],
            "timing": "host wall clock from vf_batch_launch to each member's done flag (pinned mapped memory), "
                      "states resident on the device"}


def serving_workload(n, scale):
    lo, hi = 10.0 * scale, 600.0 * scale
    cap = "" if scale == 1.0 else (f" (the configuration's U[10,600] s scaled by {scale:g}: at Float64's rate on this "
                                   "GPU one full-length pass of these requests takes ~6 min, and the measurement runs "
                                   "four passes)")
    return (f"serving: {n} flood requests drawn as the ensemble members but with sides log-uniform in [128,2048], "
            f"Float32 or Float64 with probability 1/2, end times U[{lo:g},{hi:g}] s{cap}; Poisson arrivals; "
            "HBM admission budget")


def measure_serving(args, local):
    """Continuous-batching server against a one-at-a-time plain server, same arrivals.

    Served: requests are submitted at their Poisson arrival times to the
    library's engine (vf_server_*: HBM-budget admission, one batch launch per
    poll beside the running ones); a request's latency runs from its arrival to
    the host holding its final state. Plain: one request at a time in arrival
    order through the drop-in API (build/upload, simulate_to_time, download);
    its service times are measured once back to back, and the FIFO latencies
    of each arrival sequence follow exactly from them (finish = max(arrival,
    previous finish) + service).
    """
    import volumefluxes_sm103 as vf
    from volumefluxes_sm103 import scenarios as S
    from volumefluxes_sm103.serving import Request, Server
    scale = args.serving_time_scale
    specs = S.serving_specs(args.serving_requests, endtime_range=(10.0 * scale, 600.0 * scale))
    reqs = [(S.ensemble_member(r.spec), np.float32 if r.real == "f32" else np.float64, r.spec.endtime)
            for r in specs]
    rates = [float(x) for x in args.serving_rates.split(",") if x]
    budget = int(args.serving_budget_gb * (1 << 30))
    rng = np.random.default_rng(20241204)
    gaps = rng.exponential(1.0, size=len(reqs))
    work = sum(sc.nx * sc.ny for sc, _, _ in reqs)
    out = {"workload": serving_workload(len(reqs), scale), "requests": len(reqs),
           "f64_requests": sum(r == np.float64 for _, r, _ in reqs), "hbm_budget_bytes": budget, "rates": []}
    # warm the kernels and the pool outside the timing
    with Server(budget, device=local) as srv:
        tk = [srv.submit(reqs[0][0], np.float32, 0.5), srv.submit(reqs[1][0], np.float64, 0.5)]
        while len(tk):
            for t in srv.poll():
                srv.result(t)
                tk.remove(t)
            time.sleep(0.001)
    ref_state = None
    for rate in rates:
        arrive = np.cumsum(gaps / rate)
        arrive -= arrive[0]
        prepared = [Request(sc, real, T, device=local) for sc, real, T in reqs]  # payloads ready before the clock
        lat = [None] * len(reqs)
        with Server(budget, device=local) as srv:
            t0 = time.perf_counter()
            nxt = 0
            ticket_of = {}
            first_submit = None
            while any(l is None for l in lat):
                now = time.perf_counter() - t0
                while nxt < len(reqs) and arrive[nxt] <= now:
                    ticket_of[srv.submit(prepared[nxt])] = nxt
                    nxt += 1
                for tk in srv.poll():
                    i = ticket_of[tk]
                    r = srv.result(tk)
                    if i == 0:
                        first_submit = r.submit_s
                    lat[i] = r  # engine clock
                    if i == 0:
                        ref_state = r.state.h.copy() if ref_state is None else ref_state
                        same0 = bool(np.array_equal(ref_state, r.state.h))
                time.sleep(0.0002)
            launches = srv.stats()["launches"]
        done = np.array([r.done_s for r in lat]) - first_submit
        lat = np.array([r.done_s - r.submit_s for r in lat])
        makespan = float(done.max())
        lat = np.array(lat)
        out["rates"].append({"rate_per_s": rate, "makespan_s": makespan, "throughput_req_per_s": len(reqs) / makespan,
                             "latency_s": {"p50": float(np.percentile(lat, 50)), "p95": float(np.percentile(lat, 95)),
                                           "p99": float(np.percentile(lat, 99))},
                             "batch_launches": launches, "request0_same_as_first_rate": same0})
    # one at a time through the drop-in API
    service = []
    for sc, real, T in reqs:
        t1 = time.perf_counter()
        sim = sc.build(vf.SM103Backend(real, device=local))
        vf.simulate_to_time(sim, T)
        st = vf.current_interior_state(sim)
        sim.close()
        service.append(time.perf_counter() - t1)
    for row in out["rates"]:
        rate = row["rate_per_s"]
        arrive = np.cumsum(gaps / rate)
        arrive -= arrive[0]
        fin, lat = 0.0, []
        for a, sv in zip(arrive, service):
            fin = max(a, fin) + sv
            lat.append(fin - a)
        lat = np.array(lat)
        row["plain_one_at_a_time"] = {"makespan_s": fin, "throughput_req_per_s": len(reqs) / fin,
                                      "latency_s": {"p50": float(np.percentile(lat, 50)),
                                                    "p95": float(np.percentile(lat, 95)),
                                                    "p99": float(np.percentile(lat, 99))}}
    # Float32 error against Float64 on the three smallest Float32 requests
    small = sorted([i for i, (sc, r, _) in enumerate(reqs) if r == np.float32], key=lambda i: reqs[i][0].nx)[:3]
    errs = []
    for i in small:
        sc, _, T = reqs[i]
        a = sc.build(vf.SM103Backend(np.float32, device=local))
        b = sc.build(vf.SM103Backend(np.float64, device=local))
        vf.simulate_to_time(a, T)
        vf.simulate_to_time(b, T)
        errs.append(float(np.abs(vf.current_interior_state(a).h - vf.current_interior_state(b).h).max()))
        a.close()
        b.close()
    out["f32_error_vs_f64"] = {"max_abs_w_m": max(errs), "members": [f"{reqs[i][0].nx}^2 to {reqs[i][2]:.2f} s"
                                                                      for i in small]}
    out["timing"] = ("engine clock (steady_clock in the library): latency from submission at the arrival time to "
                     "the final interior state copied to the caller's buffer; makespan from the first submission")
    return out


def adjoint_workload(n, steps):
    return (f"differentiation: {n}x{n} cells (Δ = 1 m), 16 seeded hills (amplitude U[0.2,1] m, width U[50,200] m) + "
            f"1e-3 slope, depth 1 m, Manning n = 0.03, rain 2e-5 m/s, wall BCs, RK2, CFL 0.25, {steps} steps with the "
            "dt sequence frozen from the forward pass; loss = sum over 32 seeded gauges of (w - w_target)^2, "
            "w_target from the same steps on a perturbed terrain; gradient w.r.t. every bottom corner "
            f"({(n + 5) ** 2} values) and Manning n")


def measure_adjoint(args, local):
    """Gradient of the gauge loss by the GPU reverse sweep, checked against
    central differences on the device (smooth random directions). The checks
    against the oracle on dual numbers and against extended-precision
    differences run in the GPU tests."""
    import volumefluxes_sm103 as vf
    from volumefluxes_sm103 import adjoint as AD
    from volumefluxes_sm103 import scenarios as S
    case = S.differentiation_case(args.adjoint_n)
    sc, gauges, steps = case.scenario, case.gauges, args.adjoint_steps
    out = {"workload": adjoint_workload(args.adjoint_n, steps), "checkpoint_every": int(round(math.sqrt(steps)))}
    grads = {}
    dts = None
    for real in (np.float64, np.float32):
        name = "f64" if real == np.float64 else "f32"
        sim = sc.build(vf.SM103Backend(real, device=local))
        adj = AD.GaugeAdjoint(sim, steps)
        t0 = time.perf_counter()
        d = adj.forward(dts)
        t1 = time.perf_counter()
        if dts is None:
            dts = d
            target = AD.gauge_values(sc, np.float64, gauges, dts, B=case.B_target)
        t2 = time.perf_counter()
        loss, gB, gCz = adj.backward(gauges, target)
        t3 = time.perf_counter()
        adj.close()
        sim.close()
        gn = gCz * 2 * sc.manning_n
        grads[name] = (loss, gB, gCz)
        out[name] = {"loss": loss, "dloss_dn": gn, "grad_B_norm": float(np.linalg.norm(gB)),
                     "forward_s": t1 - t0, "backward_s": t3 - t2,
                     "backward_cell_steps_per_s": sc.nx * sc.ny * steps / (t3 - t2)}
    loss, gB, gCz = grads["f64"]
    out["f32_vs_f64_grad_rel_l2"] = float(np.linalg.norm(grads["f32"][1] - gB) / np.linalg.norm(gB))
    # central differences on random smooth directions (random Gaussian bumps) and a random n component
    grid = sc.grid()
    f = vf.cell_faces(grid, interior=False)
    rng = np.random.default_rng(20241206)
    rel = []
    for k in range(args.adjoint_fd_dirs):
        v = np.zeros_like(sc.B)
        for _ in range(3):
            cx, cy = rng.uniform(0, sc.nx), rng.uniform(0, sc.ny)
            s = rng.uniform(10.0, 80.0)
            v += rng.standard_normal() * np.exp(-((f[:, :, 0] - cx) ** 2 + (f[:, :, 1] - cy) ** 2) / (2 * s * s))
        vn = float(rng.standard_normal()) * 1e-3
        got = float(np.sum(gB * v)) + gCz * 2 * sc.manning_n * vn
        fd = AD.central_difference(sc, np.float64, gauges, target, dts, v, vn, FD_EPS)
        rel.append(abs(fd - got) / max(abs(got), 1e-300))
    rel = np.array(rel)
    if len(rel):
        out["fd"] = {"directions": len(rel), "eps": FD_EPS, "rel_err_median": float(np.median(rel)),
                     "rel_err_p90": float(np.percentile(rel, 90)), "rel_err_max": float(rel.max()),
                     "within_1e-6": int((rel <= 1e-6).sum()),
                     "note": "Float64 central differences on the device: at this step some directions cross "
                             "branch switches (minmod, dry faces, the dry clamp) and rounding of the gauge depths "
                             "bounds the rest near 1e-7; the GPU tests compare the gradient with extended-precision "
                             "differences on directions whose perturbed runs take the same branches (1e-6)",
                     "directions_kind": "sums of 3 random Gaussian bumps (width U[10,80] m) on B plus a random n "
                                        "component"}
    return out


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    world, rank, local = dist_setup("nccl")
    from volumefluxes_sm103 import scenarios
    sc = scenarios.hills_wet_dry(args.n)
    if args.state_in:
        d = np.load(args.state_in)
        sc.w0, sc.hu0, sc.hv0 = d["h"], d["hu"], d["hv"]
    peak, peak_kind = peaks()
    traffic = profile_table("traffic")
    fp64_inst = profile_table("fp64_inst_per_cell")
    cells = sc.nx * sc.ny
    dtypes = [args.dtype] + ([] if args.no_variant else [d for d in ("f64", "f32") if d != args.dtype])
    results = {}
    states = {}
    modes = [(dt, "reference") for dt in dtypes]
    if "f64" in dtypes and not args.no_faithful:
        modes.append(("f64", "faithful"))
    if "f32" in dtypes and not args.no_faithful:
        modes.append(("f32", "no_near_dry"))
    for dt, mode in modes:
        key = {"reference": dt, "faithful": "f64_faithful", "no_near_dry": "f32_no_near_dry"}[mode]
        if mode == "no_near_dry":  # every Float32 velocity division by the fast reciprocal
            os.environ["VF_F32_NEAR_DRY"] = "0"
        try:
            m = measure_gpu(sc, dt, args, world, local, arithmetic="faithful" if mode == "faithful" else "reference")
        finally:
            os.environ.pop("VF_F32_NEAR_DRY", None)
        sim, ms_total = m["sim"], m["ms_total"]
        value = world * cells * args.steps / (ms_total * 1e-3)
        if args.e2e_steps > 0 and mode == "reference":
            e2e_v, h2d, d2h, _ = e2e_rate(sim, args.e2e_steps)
            e2e_v = world * e2e_v  # replicas
        else:
            e2e_v, h2d, d2h = None, 0, 0
        e = 8 if dt == "f64" else 4
        step_ach = WORDS_PER_CELL_STEP * e * cells / (ms_total / args.steps * 1e-3) / 1e9
        r = {
            "value": value, "ms_per_step": ms_total / args.steps, "gpu_launches": m["launches"], "clocks": m["clocks"],
            "roofline": roofline(sc, dt, m["ms_flux"], m["ms_stage"], peak, peak_kind, traffic),
            "roofline_step": {"bound": "hbm", "achieved": step_ach, "peak": peak, "unit": "GB/s",
                              "frac": step_ach / peak, "words_per_cell": WORDS_PER_CELL_STEP},
            "kernel_ms": {kernel_names(dt)["flux"]: m["ms_flux"], kernel_names(dt)["stage"]: m["ms_stage"]},
            "e2e": {"value": e2e_v, "unit": METRIC, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        }
        if mode == "faithful":
            r["arithmetic"] = "faithful quotients and fused multiply-adds (VF_ARITH_FAITHFUL)"
        if dt == "f32":
            r["near_dry_division"] = ("the Float64 quotient's bits (correctly rounded Float32 division) where "
                                      "|h| < 2 kappa" if mode != "no_near_dry" else "fast reciprocal everywhere")
        if "full_ms" in m:
            full_ms = m["full_ms"]
            r["full_config"] = {
                "steps": FULL_STEPS, "ms_per_step": full_ms / FULL_STEPS,
                "value": world * cells * FULL_STEPS / (full_ms * 1e-3), "unit": METRIC,
                "window": f"the configuration's {FULL_STEPS} RK2 steps from the initial state",
                "developed_kernel_ms": {kernel_names(dt)["flux"]: m["dev_flux"], kernel_names(dt)["stage"]: m["dev_stage"]},
                "developed_roofline": roofline(sc, dt, m["dev_flux"], m["dev_stage"], peak, peak_kind, traffic),
            }
            if dt == "f64" and mode == "reference":
                r["compute_roofline"] = fp64_roofline(sc, m["dev_stage"], (m["clocks"] or {}).get("sm_mhz"), fp64_inst)
        if args.steps < FULL_STEPS and args.start_steps == 0 and not args.state_in:
            r["window_note"] = (f"{args.steps} steps from the initial state: the flow starts at rest (no friction work "
                                f"for the first ~15 steps), so this window runs faster per step than the "
                                f"configuration's {FULL_STEPS} steps; see full_config")
        states[key] = (m["state"], m.get("full_state"))
        results[key] = r
        sim.close()
    # errors against the reference-rounded Float64 run, at the end of each window
    if "f64" in states:
        ref_k, ref_full = states["f64"]
        for key, (st_k, st_full) in states.items():
            if key == "f64":
                continue
            err = {"window_steps": args.steps, "at_window_end": field_errors(st_k, ref_k)}
            if st_full is not None and ref_full is not None:
                err["at_step_%d" % FULL_STEPS] = field_errors(st_full, ref_full)
            err["definition"] = ("max |x - x_f64| per field; rel_field divides by the Float64 field's max-norm, "
                                 "rel_state by max |w| (the state's max-norm)")
            results[key]["error_vs_f64"] = err
    states.clear()
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        o = oracle_sim(sc)
        v, threads, steps, el = cpu_rate(sc, 0, None, o=o)
        v1, _, steps1, el1 = cpu_rate(sc, 0, None, budget_s=6.0, threads=1, o=o)
        cpu = {"value": v, "unit": METRIC, "cores": threads, "kind": "port",
               "sample": f"{steps} RK2 steps of the {sc.nx}x{sc.ny} Float64 workload from its initial state "
                         f"({el:.1f} s, OpenMP over rows)",
               "single_core": {"value": v1, "unit": METRIC, "cores": 1,
                               "sample": f"the next {steps1} RK2 step(s) on one thread ({el1:.1f} s)"}}
    ens = serving = None
    if rank == 0 and world == 1 and not args.no_ensemble:
        ens = measure_ensemble(args, local)
    if rank == 0 and world == 1 and not args.no_serving:
        serving = measure_serving(args, local)
    adjoint = None
    if rank == 0 and world == 1 and not args.no_adjoint:
        adjoint = measure_adjoint(args, local)
    if rank != 0:
        return
    head = results[args.dtype]
    line = {
        "metric": METRIC, "value": head["value"], "unit": METRIC, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": head["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": args.dtype, "data": "synthetic",
        "config": bench_config(sc, args.dtype, world),
        "roofline": head["roofline"], "roofline_step": head["roofline_step"], "kernel_ms": head["kernel_ms"],
        "compute_roofline": head.get("compute_roofline"), "full_config": head.get("full_config"),
        "window_note": head.get("window_note"),
        "cpu_baseline": cpu, "e2e": head["e2e"], "gpu_launches": head["gpu_launches"], "clocks": head["clocks"],
        "variants": {k: v for k, v in results.items() if k != args.dtype},
        "ensemble": ens,
        "serving": serving,
        "adjoint": adjoint,
    }
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
