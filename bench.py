#!/usr/bin/env python3
"""Benchmark of the GB300 RAM kinetic step.

Headline workload: the four-species step on the standard RAM grid
(e-, H+, He+, O+; NR=20 x NT=25 x NE=35 x NPA=72 = 1,260,000 cells per
species; dipole field, Volland-Stern potential with Kp rising 1->6 over
4320 DTs steps, DTs = 5 s).  One bench step is one ram_run call: the Strang
pair R,P,E,MU,CEX,ATMOL | ATMOL,CEX,MU,E,P,R for every species, the periodic
copy, the magnetopause mask, DtsNext and the ANISCH moments -- two DTs
steps, i.e. 2 x 4 x 1.26e6 = 10.08e6 cell-updates.

Sections of the same line: the single-species step (H+, Kp 3, L2-resident),
the refined 40x49x70x144 four-species grid (its F2 exceeds L2), WPADIF on
the electrons, the 256-member uneven ensemble run from its first step to
the last retirement (members split over the ranks under torchrun), and the
2-hour adjoint window with checkpoints every 64 steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Prints one JSON line (rank 0).  Under torchrun every rank advances its own
replica of the headline workload on its own GPU (the path has no exchange
step); the ensemble's members are partitioned over the ranks.
"""
from __future__ import annotations

import argparse
import hashlib
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "ram-scb_gb300"))

METRIC = "FP64 cell-updates/s"
UNIT = "cell-updates/s"

# Figures of one ncu capture of the four-species step, labelled with the
# digest of the sweep sources they were taken from: DRAM bytes (read + write)
# per launch and FP64 instructions per cell (DADD + DFMA + DMUL thread
# instructions / cells), each the mean of the sweep's forward and reverse
# launch.  The line reports whether the current sources still have that
# digest; a changed kernel makes the figures stale until the next capture.
NCU_CAPTURE = {
    # ncu on the sources named by sources_sha16 (profiles/sweeps_four_sp.md,
    # profiles/driftr_refined.md, profiles/sweeps_l2.md): one kernel per
    # command, each captured launch advances one species, so a four-species
    # launch of the timing pass is scaled by 4.
    "sources_sha16": "8faa21e4265be355",
    "command": ("ncu --metrics gpu__time_duration.sum,dram__bytes_read.sum,dram__bytes_write.sum,lts__t_bytes.sum,"
                "smsp__sass_thread_inst_executed_op_{dadd,dfma,dmul}_pred_on.sum --clock-control none "
                "-k regex:k_sweep_<r|p|e|mu> -c 2 python bench.py --steps 2 --warmup 1 --sections headline "
                "--no-cpu-baseline --no-e2e --no-autotune [--workload refined|single_h]"),
    "dram_bytes": {"four_sp": {"driftr": 4 * 11.02e6, "driftp": 4 * 10.39e6,
                               "drifte": 4 * 0.5 * (11.34e6 + 29.98e6), "driftmu": 4 * 0.5 * (20.47e6 + 10.52e6)},
                   "single_h": {"driftr": 11.03e6, "driftp": 10.40e6,
                                "drifte": 0.5 * (11.33e6 + 29.98e6), "driftmu": 0.5 * (20.47e6 + 10.52e6)},
                   "refined": {"driftr": 4 * 0.5 * (268.51e6 + 267.80e6)}},
    # lts__t_bytes.sum per launch of the timing pass (profiles/sweeps_l2.md)
    "l2_bytes": {"four_sp": {"driftr": 4 * 0.5 * (112.45e6 + 112.11e6), "driftp": 4 * 0.5 * (39.40e6 + 39.16e6),
                             "drifte": 4 * 0.5 * (70.01e6 + 70.05e6), "driftmu": 4 * 0.5 * (78.02e6 + 58.62e6)},
                 "single_h": {"driftr": 0.5 * (112.54e6 + 111.96e6), "driftp": 0.5 * (39.44e6 + 39.26e6),
                              "drifte": 0.5 * (70.63e6 + 70.04e6), "driftmu": 0.5 * (78.13e6 + 58.64e6)},
                 "refined": {"driftr": 4 * 0.5 * (2156.6e6 + 2314.6e6)}},
    "fp64_ops_per_cell": {"driftr": 5.02, "driftp": 4.64, "drifte": 0.5 * (6.70 + 4.78),
                          "driftmu": 0.5 * (6.62 + 5.69)},
}
SWEEP_SOURCES = ["ram-scb_gb300/csrc/sweeps.cu", "ram-scb_gb300/csrc/ramgpu_internal.cuh",
                 "ram-scb_gb300/csrc/kernels.cuh"]
SECTIONS = ("headline", "single", "refined", "padif", "ensemble", "adjoint")


def sources_sha16():
    h = hashlib.sha256()
    for p in SWEEP_SOURCES:
        h.update((ROOT / p).read_bytes())
    return h.hexdigest()[:16]


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="four_sp", choices=["four_sp", "single_h", "refined"])
    ap.add_argument("--sections", default=",".join(SECTIONS),
                    help="comma-separated subset of " + ",".join(SECTIONS))
    ap.add_argument("--cpu-seconds", type=float, default=6.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--flush-mb", type=int, default=256)
    ap.add_argument("--no-graph", action="store_true")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--no-coef-store", action="store_true",
                    help="recompute the face coefficients in the reverse half instead of storing them")
    ap.add_argument("--members", type=int, default=256, help="ensemble members")
    ap.add_argument("--ensemble-calls", type=int, default=0,
                    help="ram_run calls of the ensemble run (0: until the last member retires)")
    ap.add_argument("--loop-members", type=int, default=16)
    ap.add_argument("--adj-calls", type=int, default=720,
                    help="adjoint window in ram_run calls (720 = 1440 DTs steps = 2 h)")
    ap.add_argument("--adj-ckpt", type=int, default=32, help="checkpoint spacing in calls (32 = 64 steps)")
    ap.add_argument("--adj-fd", type=int, default=16, help="finite-difference directions on the full window")
    ap.add_argument("--adj-members", type=int, default=64, help="batched-gradient members (0: skip)")
    ap.add_argument("--adj-member-calls", type=int, default=36)
    # internal: one CPU-oracle timing in a fresh process (see cpu_leg_fresh)
    ap.add_argument("--cpu-leg", default=None, help=argparse.SUPPRESS)
    ap.add_argument("--cpu-outer", type=int, default=1, help=argparse.SUPPRESS)
    ap.add_argument("--cpu-inner", type=int, default=1, help=argparse.SUPPRESS)
    ap.add_argument("--cpu-calls", type=int, default=0, help=argparse.SUPPRESS)
    ap.add_argument("--cpu-warmup", type=int, default=1, help=argparse.SUPPRESS)
    ap.add_argument("--cpu-impl", default="port", choices=["port", "ref"], help=argparse.SUPPRESS)
    args = ap.parse_args()
    args.sections = {s.strip() for s in args.sections.split(",") if s.strip()}
    bad = args.sections - set(SECTIONS)
    if bad:
        ap.error(f"unknown sections {sorted(bad)}")
    return args


def workload_desc(wl):
    g = wl.grid
    kp = "Kp 3" if wl.name == "single_h" else "Kp ramp 1->6"
    return (f"{wl.name}: {len(g.species)} species ({','.join(wl.meta['species'])}) "
            f"{g.nr}x{g.nt}x{g.ne}x{g.npa}, {kp} (VOLS), DTs={wl.dts}s")


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d.get("hbm_gbs", 6800.0)), "measured (MEASURED_PEAKS.json hbm_gbs)"
    return 6800.0, "fallback (6.8 TB/s)"


# --------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def max_over_ranks(value: float, device=None) -> float:
    """The largest value over all ranks (the job's time is its slowest rank)."""
    import torch

    t = torch.tensor([value], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(values, device=None):
    import torch

    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t)
    return [float(x) for x in t.tolist()]


# ------------------------------------------------------------ CPU legs
def cpu_threads(ns):
    """(species threads, line threads per species) using every host core:
    the reference's OpenMP loop over species, each species' independent
    lines threaded inside it."""
    cores = os.cpu_count() or 1
    outer = max(1, min(ns, cores))
    return outer, max(1, cores // outer)


def cpu_time_oracle(wl, seconds, nthreads, inner=1, calls=None, warmup=1):
    """Time the CPU oracle (the reference's routines restated in C, species
    loop under OpenMP like the reference, `inner` threads over independent
    lines inside each routine) on this workload: `warmup` untimed calls,
    then `calls` timed ones (or as many as fit in `seconds`); returns
    (cell-updates/s, calls, elapsed)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import numpy as np
    import pyoracle

    pyoracle.set_inner_threads(inner)
    o = pyoracle.Oracle(wl.grid, wl.fields)
    f2 = [np.asfortranarray(a).copy(order="F") for a in wl.f2]
    cells = 2 * wl.grid.ncell * len(wl.grid.species)
    for w in range(max(0, warmup)):
        o.ram_run(f2, wl.fgeos, wl.dts, kp=wl.kp(2 * w), nthreads=nthreads)
    n, t0 = 0, time.perf_counter()
    while True:
        o.ram_run(f2, wl.fgeos, wl.dts, kp=wl.kp(2 * (warmup + n)), nthreads=nthreads)
        n += 1
        el = time.perf_counter() - t0
        if (calls is not None and n >= calls) or (calls is None and (el >= seconds or n >= 1000)):
            break
    pyoracle.set_inner_threads(1)
    return cells * n / el, n, el


REF_DESC = ("the reference's own Fortran routines (src/ModRamDrift.f90, src/ModRamLoss.f90, src/ModRamRun.f90) "
            "translated to C by oracle/f90c.py and built by gcc -O3 -ffp-contract=off (no Fortran compiler here), "
            "run through its own ram_run with its own OpenMP loop over species")


def cpu_time_ref(wl, seconds, nthreads, calls=None, warmup=1):
    """Time the reference's own ram_run (translated, oracle/_ref) on this
    workload with nthreads OpenMP threads on its species loop (the only
    parallelism the reference has): `warmup` untimed calls, then `calls`
    timed ones (or as many as fit in `seconds`); returns (cell-updates/s,
    calls, elapsed).  The state stays in the reference's module arrays."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import refrun

    ref = refrun.RefRam(wl.grid, wl.fields, threads=nthreads)
    ref.load_state(wl.f2, wl.fgeos)
    cells = 2 * wl.grid.ncell * len(wl.grid.species)
    for w in range(max(0, warmup)):
        ref.step(wl.dts, wl.kp(2 * w))
    n, t0 = 0, time.perf_counter()
    while True:
        ref.step(wl.dts, wl.kp(2 * (warmup + n)))
        n += 1
        el = time.perf_counter() - t0
        if (calls is not None and n >= calls) or (calls is None and (el >= seconds or n >= 1000)):
            break
    return cells * n / el, n, el


def ref_available():
    sys.path.insert(0, str(ROOT / "oracle"))
    try:
        import refrun

        return refrun.build() is not None
    except Exception:  # noqa: BLE001 -- no compiler or no sources: the port stands in
        return False


def cpu_leg_main(args):
    """--cpu-leg: time a CPU leg in this process (which never imports torch
    or the CUDA library) and print one JSON object: the translated reference
    (--cpu-impl ref) or the C oracle (--cpu-impl port)."""
    from ramgpu import workload as W

    wl = W.make_workload(args.cpu_leg)
    calls = args.cpu_calls if args.cpu_calls > 0 else None
    if args.cpu_impl == "ref":
        v, n, el = cpu_time_ref(wl, args.cpu_seconds, args.cpu_outer, calls=calls, warmup=args.cpu_warmup)
    else:
        v, n, el = cpu_time_oracle(wl, args.cpu_seconds, args.cpu_outer, args.cpu_inner, calls=calls,
                                   warmup=args.cpu_warmup)
    print(json.dumps({"value": v, "calls": n, "elapsed_s": el, "outer": args.cpu_outer, "inner": args.cpu_inner}),
          flush=True)


def cpu_leg_fresh(workload, outer, inner, calls=0, seconds=10.0, warmup=1, impl="port"):
    """A CPU leg timed in a fresh interpreter that imports neither torch
    nor the CUDA library, so the figure is the one a reference run on the
    same cores sees.  (Timed inside the GPU process after its GPU sections,
    the line threads inside each species did not run: that leg measured the
    species-threads-only rate.)"""
    cmd = [sys.executable, str(ROOT / "bench.py"), "--cpu-leg", workload, "--cpu-outer", str(outer),
           "--cpu-inner", str(inner), "--cpu-calls", str(calls), "--cpu-seconds", str(seconds),
           "--cpu-warmup", str(warmup), "--cpu-impl", impl]
    r = subprocess.run(cmd, capture_output=True, text=True, check=True)
    return json.loads(r.stdout.strip().splitlines()[-1])


def cpu_baseline_fresh(workload, ns, seconds, calls=0, warmup=1, ref_calls=None, ref_warmup=None):
    """The CPU legs, each in a fresh process:
    reference: the reference's own routines (translated), OpenMP over
      species as the reference (at most nS threads) -- the line's value;
    port_species_threads / port_all_cores: the C oracle with the same
      species threads, and with every host core (line threads inside each
      routine), as reported before the reference could be run here.
    Without the translated reference the port's all-cores leg is the value
    (kind "port")."""
    cores = os.cpu_count() or 1
    o2, i2 = cpu_threads(ns)
    ot = min(ns, cores)
    v1 = cpu_leg_fresh(workload, ot, 1, calls=calls, seconds=seconds, warmup=warmup)
    v2 = cpu_leg_fresh(workload, o2, i2, calls=calls, seconds=seconds, warmup=warmup)
    variants = {"port_species_threads": {"value": v1["value"], "threads": v1["outer"], "calls": v1["calls"],
                                         "elapsed_s": v1["elapsed_s"]},
                "port_all_cores": {"value": v2["value"], "threads": o2 * i2, "calls": v2["calls"],
                                   "elapsed_s": v2["elapsed_s"]}}
    if ref_available():
        rc = calls if ref_calls is None else ref_calls
        rw = warmup if ref_warmup is None else ref_warmup
        vr = cpu_leg_fresh(workload, ot, 1, calls=rc, seconds=seconds, warmup=rw, impl="ref")
        variants["reference"] = {"value": vr["value"], "threads": ot, "calls": vr["calls"],
                                 "elapsed_s": vr["elapsed_s"]}
        return {"value": vr["value"], "unit": UNIT, "cores": ot, "kind": "reference",
                "sample": (f"{vr['calls']} ram_run calls of the workload in {vr['elapsed_s']:.1f} s after {rw} "
                           f"warm-up call(s), fresh process; {REF_DESC}, {ot} threads"),
                "variants": variants}
    return {"value": v2["value"], "unit": UNIT, "cores": o2 * i2, "kind": "port",
            "sample": (f"{v2['calls']} ram_run calls of the workload in {v2['elapsed_s']:.1f} s after {warmup} "
                       f"warm-up call(s), fresh process; C restatement of the reference routines (-O3 "
                       f"-ffp-contract=off, no Fortran compiler), OpenMP over {o2} species x {i2} line threads"),
            "variants": variants}


def run_reference(args, rank, world):
    """The reference arm: the reference's own ram_run (translated to C, with
    its own OpenMP loop over species, so at most nS threads) on this arm's
    workload; the C oracle on every host core where the translated reference
    is not available."""
    from ramgpu import workload as W

    if rank != 0:
        return
    wl = W.make_workload(args.workload)
    ns = len(wl.grid.species)
    # W untimed warm-up steps, then exactly K timed steps; a step is one
    # ram_run call of the workload
    if ref_available():
        threads = min(ns, os.cpu_count() or 1)
        v, n, el = cpu_time_ref(wl, 0.0, threads, calls=max(1, args.steps), warmup=args.warmup)
        kind, cores = "reference", threads
        sample = (f"{n} ram_run calls of the workload ({workload_desc(wl)}) after {args.warmup} warm-up "
                  f"calls, {el:.1f} s; {REF_DESC}, {threads} threads")
    else:
        outer, inner = cpu_threads(ns)
        v, n, el = cpu_time_oracle(wl, 0.0, outer, inner, calls=max(1, args.steps), warmup=args.warmup)
        kind, cores = "port", outer * inner
        sample = (f"{n} ram_run calls of the workload ({workload_desc(wl)}) after {args.warmup} warm-up "
                  f"calls, {el:.1f} s; C restatement of the reference routines (-O3 -ffp-contract=off, no Fortran "
                  f"compiler), OpenMP over {outer} species x {inner} line threads")
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": n, "warmup": args.warmup, "ms_per_step": 1e3 * el / n, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": workload_desc(wl), "step": "one ram_run call (2 DTs steps)"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": kind, "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------ GPU pieces
def new_model(abi, wl, stream, members=1):
    gpu = abi.RamGpu(wl.grid, wl.fields, n_members=members)
    gpu.set_stream(stream.cuda_stream)
    for m in range(members):
        for s in range(len(wl.grid.species)):
            gpu.upload_f2(m, s, wl.f2[s])
            gpu.set_boundary(m, s, wl.fgeos[s])
    return gpu


def timed_steps(torch, gpu, stream, wl, steps, flush, start=0):
    """`steps` graph-replayed ram_run calls along the workload's Kp driver,
    L2 flushed (a write larger than L2) before each, each bracketed by CUDA
    events on the launching stream; returns the per-call ms and the number
    of kernel launches."""
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    l0 = gpu.launch_count()
    for k in range(steps):
        with torch.cuda.stream(stream):
            flush.fill_(k & 0xFF)
        gpu.set_kp(-1, wl.kp(2 * (start + k)))
        ev[k][0].record(stream)
        gpu.ram_run_async(wl.dts)
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    return [a.elapsed_time(b) for a, b in ev], gpu.launch_count() - l0


def kernel_pass(torch, gpu, stream, wl, flush, n):
    """Per-kernel durations: n calls with events around every launch group
    on the launching stream (timing mode runs direct launches on one
    stream); returns ({class: (ms, launches)}, mean call ms)."""
    gpu.set_timing(True)
    gpu.kernel_times()
    ms = []
    for k in range(n):
        with torch.cuda.stream(stream):
            flush.fill_(k & 0xFF)
        gpu.set_kp(-1, wl.kp(2 * k))
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        gpu.ram_run_async(wl.dts)
        b.record(stream)
        torch.cuda.synchronize()
        ms.append(a.elapsed_time(b))
    kt = gpu.kernel_times()
    gpu.set_timing(False)
    return kt, statistics.mean(ms)


def roofline(kt, wl, nitems, hbm_peak, peak_kind, fp64_peak, workload, l2_peak=None):
    """HBM view of the dominant sweep: 16 B per cell (F2 read + write once)
    over its event-timed launch; the FP64 view and the L2 view (the ncu L2
    bytes of the same launch against the live L2 probe) beside it."""
    sweep = {k: v for k, v in kt.items() if k.startswith("drift")}
    dom = max(sweep, key=lambda k: sweep[k][0])
    dom_ms = sweep[dom][0] / sweep[dom][1]
    cells = wl.grid.ncell * nitems
    achieved = 16.0 * cells / (dom_ms / 1e3) / 1e9
    current = sources_sha16() == NCU_CAPTURE["sources_sha16"]
    ops = NCU_CAPTURE["fp64_ops_per_cell"][dom]
    fp64 = ops * cells / (dom_ms / 1e3) / 1e9
    traffic = NCU_CAPTURE["dram_bytes"].get(workload, {}).get(dom)
    return {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak,
            "traffic": traffic if current else None, "kernel": dom, "kernel_ms": dom_ms, "peak_kind": peak_kind,
            "traffic_source": {"capture": NCU_CAPTURE["command"], "sources_sha16": NCU_CAPTURE["sources_sha16"],
                               "current_sources_sha16": sources_sha16(), "matches_current_sources": current,
                               "workload": workload if traffic is not None else None},
            "algorithmic_bytes_per_launch": 16.0 * cells,
            "fp64": {"achieved": fp64, "peak": fp64_peak, "unit": "G lane-ops/s", "frac": fp64 / fp64_peak,
                     "ops_per_cell": ops, "ops_per_cell_from_current_sources": current,
                     "peak_kind": "measured live (fma loop, ramgpu_probe_fp64)"},
            "sweeps_GBps": {k: 16.0 * cells / (v[0] / v[1] / 1e3) / 1e9 for k, v in sweep.items()},
            "l2": l2_view(sweep, dom, workload, current, l2_peak)}


def l2_view(sweep, dom, workload, current, l2_peak):
    """L2 traffic of the sweeps (ncu lts__t_bytes of the capture, per launch
    of the timing pass) over their event-timed launches, against the live
    L2 read-bandwidth probe; null when the capture is not of the current
    sources or of this workload."""
    l2b = NCU_CAPTURE.get("l2_bytes", {}).get(workload)
    if not current or not l2b or l2_peak is None:
        return None
    gbps = {k: l2b[k] / (v[0] / v[1] / 1e3) / 1e9 for k, v in sweep.items() if k in l2b}
    return {"achieved": gbps.get(dom), "peak": l2_peak, "unit": "GB/s",
            "frac": gbps[dom] / l2_peak if dom in gbps else None, "kernel": dom,
            "bytes_per_launch": l2b.get(dom), "sweeps_GBps": gbps,
            "peak_kind": "measured live (L1-bypassing 16-byte loads over 32 MB held in L2, ramgpu_probe_l2)"}


def e2e_section(torch, np, abi, gpu, wl, steps):
    """The metric end to end through the C ABI with host buffers, full F2 in
    and out every call, as the reference's host array F2 is: the per-species
    pipelined call from page-locked and from ordinary memory, the same
    traffic serialised on one stream, and the call on F2 in the reference's
    own layout F2(NS,NR,NT,NE,NPA) (page-locked and ordinary)."""
    g = wl.grid
    ns = len(g.species)
    cells_per_step = 2 * g.ncell * ns
    nm2 = g.nr * g.nt
    pin = [torch.empty(g.ncell, dtype=torch.float64, pin_memory=True) for _ in range(ns)]
    host = [np.reshape(p.numpy(), (g.nr, g.nt, g.ne, g.npa), order="F") for p in pin]
    mom_t = torch.empty(2 * ns * nm2, dtype=torch.float64, pin_memory=True)
    mom = mom_t.numpy()
    pe_h = [mom[s * nm2:(s + 1) * nm2] for s in range(ns)]
    pa_h = [mom[(ns + s) * nm2:(ns + s + 1) * nm2] for s in range(ns)]
    for s in range(ns):
        host[s][...] = gpu.download_f2(0, s)
    host_pg = [np.asfortranarray(a).copy(order="F") for a in host]
    pe_pg = [np.zeros(nm2) for _ in range(ns)]
    pa_pg = [np.zeros(nm2) for _ in range(ns)]
    ref_pin_t = torch.empty(ns * g.ncell, dtype=torch.float64, pin_memory=True)
    ref_pin = np.reshape(ref_pin_t.numpy(), (ns, g.nr, g.nt, g.ne, g.npa), order="F")
    ref_pin[...] = np.stack([np.asarray(a) for a in host], axis=0)
    mref_t = torch.empty(2 * ns * nm2, dtype=torch.float64, pin_memory=True)
    mref = mref_t.numpy()
    pe_ref, pa_ref = mref[:ns * nm2], mref[ns * nm2:]
    ref_pg = ref_pin.copy(order="F")
    pe_ref_pg, pa_ref_pg = np.zeros(ns * nm2), np.zeros(ns * nm2)
    lib, h = gpu.lib, gpu.h
    hp = [a.ctypes.data_as(abi._P) for a in host]

    def pipelined(k):
        gpu.set_kp(-1, wl.kp(2 * k))
        gpu.ram_run_host(wl.dts, host, pe_h, pa_h)

    def pageable(k):
        gpu.set_kp(-1, wl.kp(2 * k))
        gpu.ram_run_host(wl.dts, host_pg, pe_pg, pa_pg)

    def serial(k):
        for s in range(ns):
            gpu._ck(lib.ramgpu_upload_f2_async(h, 0, s, hp[s]), "upload")
        gpu.set_kp(-1, wl.kp(2 * k))
        gpu.ram_run_async(wl.dts)
        for s in range(ns):
            gpu._ck(lib.ramgpu_download_f2_async(h, 0, s, hp[s]), "download")
            gpu._ck(lib.ramgpu_moments_async(h, 0, s, pe_h[s].ctypes.data_as(abi._P),
                                             pa_h[s].ctypes.data_as(abi._P)), "moments")
        gpu._ck(lib.ramgpu_synchronize(h), "synchronize")

    def ref_layout(k):
        gpu.set_kp(-1, wl.kp(2 * k))
        gpu.ram_run_ref(wl.dts, [ref_pin], [pe_ref], [pa_ref])

    def ref_layout_pageable(k):
        gpu.set_kp(-1, wl.kp(2 * k))
        gpu.ram_run_ref(wl.dts, [ref_pg], [pe_ref_pg], [pa_ref_pg])

    med = {}

    def run(fn):
        # three warm-up calls (the first creates the group streams and
        # captures the graph; the first few also touch the host buffers)
        for w in range(3):
            fn(w)
        torch.cuda.synchronize()
        ts = []
        t0 = time.perf_counter()
        for k in range(steps):
            t1 = time.perf_counter()
            fn(k)
            ts.append(time.perf_counter() - t1)
        med[fn.__name__] = 1e3 * statistics.median(ts)
        return cells_per_step * steps / max(time.perf_counter() - t0, 1e-9)

    out = {"value": None, "unit": UNIT, "h2d_bytes_per_step": 8 * g.ncell * ns,
           "d2h_bytes_per_step": 8 * g.ncell * ns + 16 * nm2 * ns,
           "path": (f"ramgpu_set_kp + ramgpu_ram_run_host (page-locked host F2 of {ns} species in and out, "
                    f"moments of {ns} species out; pipelined over species groups), every step")}
    out["value"] = run(pipelined)
    out["pageable_value"] = run(pageable)
    out["serial_value"] = run(serial)
    out["ref_layout_value"] = run(ref_layout)
    out["ref_layout_pageable_value"] = run(ref_layout_pageable)
    out["ms_per_step_median"] = dict(med)
    out["pageable_path"] = "ramgpu_ram_run_host with ordinary (pageable) host arrays"
    out["serial_path"] = ("ramgpu_upload_f2_async x NS + ramgpu_ram_run_async + ramgpu_download_f2_async x NS "
                          "+ ramgpu_moments_async x NS + ramgpu_synchronize on one stream")
    out["ref_layout_path"] = ("ramgpu_ram_run_ref on F2(NS,NR,NT,NE,NPA) and PPERT/PPART(NS,NR,NT) as RAM holds "
                              "them (page-locked; _pageable: ordinary memory), transposed on the device")
    del pin, mom_t, ref_pin_t, mref_t
    return out


def measure(args, torch, np, abi, W, stream, name, steps, warmup, world=1, clocks=False, e2e_steps=0,
            kernel_steps=3):
    """One workload: autotune, graph-replayed timed calls (L2 flushed), the
    per-kernel pass, the roofline and optionally the end-to-end figures."""
    wl = W.make_workload(name)
    g = wl.grid
    ns = len(g.species)
    gpu = new_model(abi, wl, stream)
    gpu.set_kp(-1, wl.kp(0))
    if args.no_coef_store:
        gpu.set_coef_store(0)
    if args.no_autotune:
        shapes, trials = gpu.launch_shape(), None
    else:
        shapes, _ = gpu.autotune(wl.dts)
        pl, pe = gpu.autotune_trials()
        trials = {"plain_ms": [round(x, 5) for x in pl], "persistent_ms": [round(x, 5) for x in pe]}
    groups = gpu.step_groups()
    gpu.set_graph(not args.no_graph)
    flush = torch.empty(max(1, args.flush_mb) << 20, dtype=torch.uint8, device="cuda")
    for w in range(warmup):
        gpu.set_kp(-1, wl.kp(2 * w))
        gpu.ram_run(wl.dts)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    sampler = ClockSampler(torch.cuda.current_device()) if clocks else None
    if sampler:
        sampler.start()
        time.sleep(0.3)
    # an NVTX range marks the timed steps, so that a profiler can select
    # exactly their launches (ncu --nvtx --nvtx-include "ram_run_timed_four_sp/")
    nvtx = getattr(torch.cuda, "nvtx", None)
    if nvtx is not None:
        nvtx.range_push(f"ram_run_timed_{name}")
    wall0 = time.perf_counter()
    ms, launches = timed_steps(torch, gpu, stream, wl, steps, flush, start=warmup)
    wall = time.perf_counter() - wall0
    if nvtx is not None:
        nvtx.range_pop()
    clk = sampler.stop() if sampler else None
    total_ms = sum(ms)
    if world > 1:
        total_ms = max_over_ranks(total_ms, torch.device("cuda"))
    cells_per_step = 2 * g.ncell * ns
    kt, kt_ms = kernel_pass(torch, gpu, stream, wl, flush, max(3, kernel_steps))
    hbm_peak, peak_kind = measured_peaks()
    fp64_peak = abi.probe_fp64() / 1e9
    l2_peak = abi.probe_l2() / 1e9
    out = {"workload": workload_desc(wl), "cells_per_step": cells_per_step,
           "value": world * cells_per_step * steps / (total_ms / 1e3), "ms_per_step": total_ms / steps,
           "steps": steps, "warmup": warmup, "launches": launches, "wall_s": wall, "clocks": clk,
           "launch_shapes": shapes, "autotune_trials": trials, "item_groups": groups,
           "kernels_ms": {k: round(v[0] / v[1], 5) for k, v in kt.items()}, "kernel_pass_ms_per_step": kt_ms,
           "roofline": roofline(kt, wl, ns, hbm_peak, peak_kind, fp64_peak, name, l2_peak)}
    per_gpu = out["value"] / world
    out["roofline"]["step"] = {"fused_min_GBps": per_gpu * 16 / 1e9, "fused_min_frac": per_gpu * 16 / 1e9 / hbm_peak,
                               "unfused_GBps": per_gpu * 80 / 1e9, "unfused_frac": per_gpu * 80 / 1e9 / hbm_peak}
    if e2e_steps:
        e = e2e_section(torch, np, abi, gpu, wl, e2e_steps)
        for k in ("value", "pageable_value", "serial_value", "ref_layout_value", "ref_layout_pageable_value"):
            e[k] *= world
        out["e2e"] = e
    gpu.close()
    return out


def run_padif(torch, abi, W, stream, args):
    """The four-species step with WPADIF on the electrons (both halves),
    per-kernel timed."""
    wl = W.make_workload("four_sp")
    g = wl.grid
    gpu = new_model(abi, wl, stream)
    flush = torch.empty(max(1, args.flush_mb) << 20, dtype=torch.uint8, device="cuda")
    # each measured pass follows an untimed one, so that the once-per-DTs
    # tables (and, with WPADIF on, its elimination tables) are built outside it
    kernel_pass(torch, gpu, stream, wl, flush, 1)
    _, base_ms = kernel_pass(torch, gpu, stream, wl, flush, 3)
    gpu.set_pa_diffusion(0, W.pa_diffusion(g, wl.fields))
    kernel_pass(torch, gpu, stream, wl, flush, 1)
    kt, step_ms = kernel_pass(torch, gpu, stream, wl, flush, 3)
    gpu.close()
    pk = kt.get("padif", (0.0, 1))
    per = pk[0] / max(pk[1], 1)
    # algorithmic bytes of the two launches per step: the electrons' solve
    # reads F2 and the three elimination tables and writes F2 (40 B per
    # cell) in both; the first also applies the loss factor to the other
    # three species (F2 and factor in, F2 out: 24 B per cell)
    byts = 0.5 * (40.0 + 40.0 + 3 * 24.0) * g.ncell
    return {"species": "Electron (WPADIF after the drifts and before the reverse drifts)",
            "step_ms": step_ms, "step_ms_without": base_ms, "kernel_ms_per_launch": per, "launches": pk[1],
            "algorithmic_GBps": byts / (per / 1e3) / 1e9 if per > 0 else None}


def run_ensemble(args, torch, np, abi, W, stream, rank, world):
    """Config 4: 256 members on the standard grid (1-4 species, Kp drivers
    piecewise linear on a 30-min cadence drawn uniform 1-7, density scale
    lognormal sigma 0.5, lengths uniform 360-1440 DTs steps), run from step
    0 until the last member retires, batched in one graph-replayed ram_run
    per call; members partitioned over the ranks by work.  Against: the
    plain single-member step looped, and sampled members' solo runs."""
    from ramgpu import shard

    ens = W.make_ensemble(args.members)
    base = ens.base
    g = base.grid
    parts = shard.partition_members(shard.member_work(ens.species, ens.length), world)
    mine = parts[rank]
    nm = len(mine)
    gpu = abi.RamGpu(g, base.fields, n_members=nm)
    gpu.set_stream(stream.cuda_stream)

    def load(model, members):
        for i, m in enumerate(members):
            model.set_member_species(i, ens.species[m])
            for s in ens.species[m]:
                model.upload_f2(i, s, base.f2[s] * ens.scale[m])
                model.set_boundary(i, s, base.fgeos[s] * ens.scale[m])

    load(gpu, mine)
    gpu.set_kp_all(ens.kp(0)[mine])
    shapes, _ = gpu.autotune(base.dts)
    pl, pe = gpu.autotune_trials()
    groups = gpu.step_groups()
    gpu.set_graph(True)
    gpu.ram_run(base.dts)  # captures the graph; the run then starts from the initial state
    load(gpu, mine)
    flush = torch.empty(max(1, args.flush_mb) << 20, dtype=torch.uint8, device="cuda")
    length = np.asarray(ens.length)[mine]
    ncalls = int(math.ceil(length.max() / 2)) if args.ensemble_calls <= 0 else args.ensemble_calls
    active = np.ones(nm, dtype=bool)
    nspec = np.array([len(ens.species[m]) for m in mine])
    last_call = np.zeros(nm, dtype=int)
    ev = []
    member_steps = 0
    cell_updates = 0
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    wall0 = time.perf_counter()
    for c in range(ncalls):
        step = 2 * c
        for i in np.nonzero(active & (step >= length))[0]:  # finished members retire
            gpu.set_member_active(int(i), False)
            active[i] = False
        if not active.any():
            break
        member_steps += 2 * int(active.sum())
        cell_updates += 2 * g.ncell * int(nspec[active].sum())
        last_call[active] = c
        gpu.set_kp_all(ens.kp(step)[mine])
        if c % 8 == 0:  # the state (GBs) is far larger than L2; flush now and then as well
            with torch.cuda.stream(stream):
                flush.fill_(c & 0xFF)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        gpu.ram_run_async(base.dts)
        b.record(stream)
        ev.append((a, b))
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    batched_s = sum(a.elapsed_time(b) for a, b in ev) / 1e3
    # per-member diagnostics: the sum of PPERT of each species after the
    # member's last call, gathered on every rank
    rows = {m: [float(np.sum(gpu.moments(i, s)[0])) for s in ens.species[m]] for i, m in enumerate(mine)}
    allrows = shard.gather_member_rows(rows, world, rank, ens.members, torch.distributed if world > 1 else None)
    if world > 1:
        batched_s = max_over_ranks(batched_s, torch.device("cuda"))
        member_steps, cell_updates = sum_over_ranks([member_steps, cell_updates], torch.device("cuda"))
    # the persistent grids the configuration names, forced on every sweep
    # (2 CTAs per SM looping over the work units), against the tuned shapes,
    # a few calls with every member active again
    for i in range(nm):
        gpu.set_member_active(i, True)
    gpu.set_kp_all(ens.kp(0)[mine])

    def sample(n=4):
        gpu.ram_run(base.dts)  # recapture for the shapes
        t = []
        for k in range(n):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            gpu.ram_run_async(base.dts)
            b.record(stream)
            torch.cuda.synchronize()
            t.append(a.elapsed_time(b))
        return statistics.median(t)

    tuned_ms = sample()
    nsm = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    for w, (thr, _) in enumerate(shapes):
        gpu.set_launch_shape(w, thr, 2 * nsm)
    persistent_ms = sample()
    for w, (thr, pc) in enumerate(shapes):
        gpu.set_launch_shape(w, thr, pc)
    # looped: the plain single-member step (direct launches), one member at a time
    gpu.set_graph(False)
    sub = list(range(0, nm, max(1, nm // args.loop_members)))[:args.loop_members]
    for i in range(nm):
        gpu.set_member_active(i, False)
    lev = []
    for i in sub:
        gpu.set_member_active(i, True)
        gpu.set_kp_all(ens.kp(0)[mine])
        gpu.ram_run(base.dts)  # warm (rebuilds the work list)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            flush.fill_(i & 0xFF)
        a.record(stream)
        gpu.ram_run_async(base.dts)
        b.record(stream)
        torch.cuda.synchronize()
        lev.append(a.elapsed_time(b) / 1e3)
        gpu.set_member_active(i, False)
    gpu.close()
    # solo runs of a few members over their whole length equal the batched run
    solo_diff = 0.0
    solo_members = [mine[i] for i in sub[:3]]
    for m in solo_members:
        solo = abi.RamGpu(g, base.fields, n_members=1)
        solo.set_stream(stream.cuda_stream)
        load(solo, [m])
        solo.set_graph(True)
        for c in range(int(last_call[mine.index(m)]) + 1):
            solo.set_kp(0, float(ens.kp(2 * c)[m]))
            solo.ram_run_async(base.dts)
        torch.cuda.synchronize()
        got = [float(np.sum(solo.moments(0, s)[0])) for s in ens.species[m]]
        for x, y in zip(got, rows[m]):
            solo_diff = max(solo_diff, abs(x - y) / max(abs(y), 1e-300))
        solo.close()
    looped = 2.0 / statistics.mean(lev)
    batched = member_steps / batched_s
    return {"members": ens.members, "member_species": int(sum(len(x) for x in ens.species)),
            "ranks": world, "members_per_rank": [len(p) for p in parts],
            "calls": len(ev), "dts_steps": 2 * len(ev), "member_steps": int(member_steps),
            "batched_s": batched_s, "wall_s": wall,
            "member_steps_per_s_batched": batched, "member_steps_per_s_looped": looped,
            "batched_over_looped": batched / looped,
            "cell_updates_per_s_batched": cell_updates / batched_s,
            "looped_sample_members": len(sub), "launch_shapes": shapes, "item_groups": groups,
            "autotune_trials": {"plain_ms": [round(x, 4) for x in pl], "persistent_ms": [round(x, 4) for x in pe]},
            "persistent_all_sweeps_ms_per_call": persistent_ms, "tuned_ms_per_call": tuned_ms,
            "solo_members": solo_members, "solo_vs_batched_max_rel_diff": solo_diff,
            "diagnostics_gathered": sum(r is not None for r in allrows),
            "notes": ("batched: the whole uneven run, from step 0 until the last member retires, one graph-replayed "
                      "ram_run per call for all active members; looped: the plain direct-launch step of one member "
                      "at a time; persistent: one persistent grid per sweep (2 CTAs per SM) with every member "
                      "active, against the tuned shapes in the same state")}


def _truth_observations(gpu, wl, kp, obs, ncalls, species, seed):
    """Fill log_obs from a seed-perturbed forward run sampled by the
    virtual-spacecraft flyer; kp: (ncalls, members)."""
    import numpy as np

    rng = np.random.Generator(np.random.PCG64(seed))
    for m in range(gpu.n_members):
        gpu.set_member_species(m, species[m])
        for s in species[m]:
            gpu.upload_f2(m, s, np.asarray(wl.f2[s]) * rng.lognormal(0.0, 0.05, size=wl.f2[s].shape))
            gpu.set_boundary(m, s, wl.fgeos[s])
    gpu.set_graph(True)
    bycall = {}
    for o in obs:
        bycall.setdefault(o["call"], []).append(o)
    for c in range(ncalls):
        gpu.set_kp_all(kp[c])
        gpu.ram_run(wl.dts)
        if c in bycall:
            sf, _ = gpu.fly_sats([(o["member"], o["lshell"], o["mlt"]) for o in bycall[c]])
            for t, o in enumerate(bycall[c]):
                o["log_obs"] = math.log(sf[t, o["s"], o["k"], o["l"]])


def _event_timer(torch, stream):
    """Seconds on the device between this point of the stream and the point
    where the returned function is called."""
    a = torch.cuda.Event(enable_timing=True)
    a.record(stream)

    def stop():
        b = torch.cuda.Event(enable_timing=True)
        b.record(stream)
        b.synchronize()
        return a.elapsed_time(b) / 1e3
    return stop


def run_adjoint(args, torch, np, abi, W, stream):
    """Config 5: adjoint window on the four-species standard grid, 1440 DTs
    steps (720 ram_run calls, Kp 1->6 ramp), 50 virtual-spacecraft samples on
    circular equatorial orbits at L = 4-6, 10-200 keV, pitch-angle bin 2.
    Forward and adjoint are timed with CUDA events on the same stream."""
    from ramgpu import sats

    wl = W.make_workload("four_sp")
    g = wl.grid
    ns = len(g.species)
    nc, kc = args.adj_calls, args.adj_ckpt
    kp = np.array([[wl.kp(2 * c)] for c in range(nc)])
    obs = sats.orbit_observations(g, nc, wl.dts, 50, seed=505)
    truth = abi.RamGpu(g, wl.fields)
    truth.set_stream(stream.cuda_stream)
    _truth_observations(truth, wl, kp, obs, nc, [list(range(ns))], seed=606)
    truth.close()
    gpu = abi.RamGpu(g, wl.fields)
    gpu.set_stream(stream.cuda_stream)

    def reset():
        for s in range(ns):
            gpu.upload_f2(0, s, wl.f2[s])
            gpu.set_boundary(0, s, wl.fgeos[s])
        torch.cuda.synchronize()

    reset()
    gpu.autotune(wl.dts)
    gpu.set_graph(True)
    for c in range(2):
        gpu.set_kp(-1, kp[c, 0])
        gpu.ram_run(wl.dts)
    reset()
    stop = _event_timer(torch, stream)
    for c in range(nc):
        gpu.set_kp(-1, kp[c, 0])
        gpu.ram_run_async(wl.dts)
    fwd_s = stop()

    def window(k_ckpt, budget):
        """A warm-up window (allocations) and a timed one: J, gradients,
        forward and backward seconds, segments and kept segments."""
        gpu.set_adj_record_budget(budget)
        reset()
        gpu.adj_forward(nc, wl.dts, kp, k_ckpt, obs)
        gpu.adj_backward()
        reset()
        stop = _event_timer(torch, stream)
        J = gpu.adj_forward(nc, wl.dts, kp, k_ckpt, obs)[0]
        tf = stop()
        stop = _event_timer(torch, stream)
        gf, gb = gpu.adj_backward()
        tb = stop()
        nseg, nkeep = gpu.adj_segments()
        return J, gf, gb, tf, tb, nseg, nkeep

    # checkpoints every kc calls with the smallest record ring, two segments:
    # every earlier segment is recomputed from its checkpoint on a second
    # stream while the next one is transposed (the configuration's policy,
    # and the one for windows whose records do not fit in HBM)
    J, gfr, gbr, tfr, tbr, nseg, nkeep_r = window(kc, 0)
    # the same without the overlap: a one-segment ring, each segment
    # recomputed and then transposed on the same streams
    gpu.set_adj_overlap(False)
    _, gfs, gbs, tfs, tbs, _, nkeep_s = window(kc, 0)
    gpu.set_adj_overlap(True)
    # the same checkpoints, the ring keeping as many segments as half of the
    # free HBM holds (here all: nothing recomputed)
    _, gf, gb, tfk, tbk, _, nkeep = window(kc, -1)
    gpu.set_adj_record_budget(-1)

    def rel(a, b):
        return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))

    same_r = max(rel(gfr, gf), rel(gbr, gb))
    same_s = max(rel(gfs, gf), rel(gbs, gb))
    # one segment (k = ncalls): the record of every call, for the replays
    reset()
    gpu.adj_forward(nc, wl.dts, kp, nc, obs)
    gf2, gb2 = gpu.adj_backward()
    same = max(rel(gf2, gf), rel(gb2, gb))
    rng = np.random.Generator(np.random.PCG64(707))

    def fd_f2(r, eps, frozen):
        jj = []
        for sign in (1.0, -1.0):
            for s in range(ns):
                gpu.upload_f2(0, s, np.asarray(wl.f2[s]) * (1.0 + sign * eps * r[s]))
            jj.append(gpu.adj_replay()[0] if frozen else gpu.adj_forward(nc, wl.dts, kp, nc, obs)[0])
        return (jj[0] - jj[1]) / (2 * eps)

    # finite differences of the frozen-limiter scheme (the record of the base
    # run replayed, affine in F2): the exact check of the adjoint on the whole
    # window, one central difference per direction (J is the log of affine
    # fluxes: truncation ~ eps^2, rounding ~ 1e-16/eps)
    fd = []
    for d in range(max(0, args.adj_fd)):
        r = [rng.uniform(-1.0, 1.0, size=wl.f2[s].shape) for s in range(ns)]
        ad = sum(float(np.sum(gf2[0, s] * np.asarray(wl.f2[s]) * r[s])) for s in range(ns))
        fd.append(abs(fd_f2(r, 1e-6, True) - ad) / abs(ad))
    # unfrozen: perturbed runs re-decide every limiter branch (kinks crossed)
    unfrozen = {}
    if args.adj_fd > 0:
        r = [rng.uniform(-1.0, 1.0, size=wl.f2[s].shape) for s in range(ns)]
        ad = sum(float(np.sum(gf2[0, s] * np.asarray(wl.f2[s]) * r[s])) for s in range(ns))
        for eps in (1e-6, 1e-8):
            unfrozen[f"{eps:.0e}"] = abs(fd_f2(r, eps, False) - ad) / abs(ad)
    reset()
    gpu.close()
    out = {"window_calls": nc, "window_dts_steps": 2 * nc, "checkpoint_calls": kc, "observations": len(obs),
           "J": J, "forward_s": fwd_s, "timing": "CUDA events on the context's stream for forward and adjoint",
           "adj_forward_s": tfr, "adj_backward_s": tbr, "adjoint_over_forward": (tfr + tbr) / fwd_s,
           "segments": nseg, "segments_kept": nkeep_r, "segments_recomputed": nseg - nkeep_r,
           "policy": ("checkpoints every checkpoint_calls calls; the branch-record ring keeps two segments; the "
                      "forward pass records only those and runs the plain step elsewhere; the backward pass "
                      "recomputes every earlier segment from its checkpoint, recording, on a second stream "
                      "while the following segment is transposed"),
           "sequential_recompute": {"segments_kept": nkeep_s, "adj_forward_s": tfs, "adj_backward_s": tbs,
                                    "adjoint_over_forward": (tfs + tbs) / fwd_s,
                                    "gradient_vs_kept_max_rel_diff": same_s,
                                    "policy": ("one-segment ring; each earlier segment recomputed, then "
                                               "transposed, on the same streams")},
           "records_kept": {"segments_kept": nkeep, "adj_forward_s": tfk, "adj_backward_s": tbk,
                            "adjoint_over_forward": (tfk + tbk) / fwd_s,
                            "record_bytes": 4 * g.ncell * ns * nc,
                            "policy": "the ring keeps as many segments as half of the free HBM holds: none recomputed"},
           "gradient_recompute_vs_kept_max_rel_diff": same_r,
           "single_segment_gradient_max_rel_diff": same,
           "fd_frozen_directions": len(fd), "fd_frozen_max_rel_err": max(fd) if fd else None,
           "fd_frozen_eps": "central difference, eps = 1e-6", "fd_unfrozen_rel_err": unfrozen}
    if args.adj_members > 0:
        out["batched"] = run_adjoint_batched(args, torch, np, abi, W, stream)
    return out


def run_adjoint_batched(args, torch, np, abi, W, stream):
    from ramgpu import sats

    ens = W.make_ensemble(args.adj_members, seed=808)
    base = ens.base
    g = base.grid
    nm, nc = ens.members, args.adj_member_calls
    kc = max(1, nc // 3)
    kp = np.stack([ens.kp(2 * c) for c in range(nc)])
    obs = sats.orbit_observations(g, nc, base.dts, 10 * nm, seed=909, members=nm, species=ens.species)
    truth = abi.RamGpu(g, base.fields, n_members=nm)
    truth.set_stream(stream.cuda_stream)
    _truth_observations(truth, base, kp, obs, nc, ens.species, seed=910)
    truth.close()
    gpu = abi.RamGpu(g, base.fields, n_members=nm)
    gpu.set_stream(stream.cuda_stream)

    def reset(model, members):
        for mi, m in enumerate(members):
            model.set_member_species(mi, ens.species[m])
            for s in ens.species[m]:
                model.upload_f2(mi, s, np.asarray(base.f2[s]) * ens.scale[m])
                model.set_boundary(mi, s, base.fgeos[s] * ens.scale[m])
        torch.cuda.synchronize()

    reset(gpu, range(nm))
    gpu.set_graph(True)
    gpu.set_kp_all(kp[0])
    gpu.ram_run(base.dts)
    reset(gpu, range(nm))
    stop = _event_timer(torch, stream)
    for c in range(nc):
        gpu.set_kp_all(kp[c])
        gpu.ram_run_async(base.dts)
    fwd_s = stop()
    reset(gpu, range(nm))
    gpu.adj_forward(nc, base.dts, kp, kc, obs)  # warm-up (allocations)
    gpu.adj_backward()
    reset(gpu, range(nm))
    stop = _event_timer(torch, stream)
    gpu.adj_forward(nc, base.dts, kp, kc, obs)
    gf, gb = gpu.adj_backward()
    batched_s = stop()
    nseg, nkeep = gpu.adj_segments()
    gpu.close()
    # looped: the same gradients one member at a time
    sub = list(range(0, nm, max(1, nm // 4)))[:4]
    solo = abi.RamGpu(g, base.fields, n_members=1)
    solo.set_stream(stream.cuda_stream)
    loop_s, agree = [], 0.0
    for m in sub:
        obs_m = [dict(o, member=0) for o in obs if o["member"] == m]
        reset(solo, [m])
        solo.adj_forward(nc, base.dts, kp[:, m], kc, obs_m)  # warm-up
        solo.adj_backward()
        reset(solo, [m])
        stop = _event_timer(torch, stream)
        solo.adj_forward(nc, base.dts, kp[:, m], kc, obs_m)
        gfm, _ = solo.adj_backward()
        loop_s.append(stop())
        for s in ens.species[m]:
            agree = max(agree, float(np.max(np.abs(gfm[0, s] - gf[m, s])) / max(np.max(np.abs(gf[m, s])), 1e-300)))
    solo.close()
    looped = 1.0 / statistics.mean(loop_s)
    return {"members": nm, "member_species": int(sum(len(x) for x in ens.species)), "window_calls": nc,
            "checkpoint_calls": kc, "observations": len(obs), "segments": nseg, "segments_kept": nkeep,
            "forward_s": fwd_s, "adjoint_s": batched_s,
            "adjoint_over_forward": batched_s / fwd_s,
            "member_gradients_per_s_batched": nm / batched_s, "member_gradients_per_s_looped": looped,
            "batched_over_looped": (nm / batched_s) / looped,
            "solo_vs_batched_max_rel_diff": agree, "looped_sample_members": len(sub)}


def run_gb300(args, rank, world, local_rank):
    import numpy as np
    import torch

    from ramgpu import abi, workload as W

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    stream = torch.cuda.Stream(device=dev)
    sec = args.sections
    head = measure(args, torch, np, abi, W, stream, args.workload, args.steps, args.warmup, world=world,
                   clocks=True, e2e_steps=0 if args.no_e2e else max(3, min(30, args.steps)),
                   kernel_steps=max(3, min(args.steps, 10)))
    single = refined = padif = ensemble = adjoint = None
    if rank == 0 and "single" in sec and args.workload != "single_h":
        # config 1: one species, 10 MB of F2, L2-resident between its sweeps
        single = measure(args, torch, np, abi, W, stream, "single_h", 20, 3)
        single["l2"] = ("working set (F2 10.1 MB + tables) inside the 129 MB L2: within a step the sweeps' "
                        "algorithmic traffic (roofline.sweeps_GBps, 16 B per cell) is served by L2; L2 is flushed "
                        "between steps")
    if rank == 0 and "refined" in sec and args.workload != "refined":
        # config 3: F2 of 632 MB, larger than L2: the HBM roofline case
        refined = measure(args, torch, np, abi, W, stream, "refined", 10, 2,
                          e2e_steps=0 if args.no_e2e else 5, kernel_steps=3)
    if rank == 0 and "padif" in sec:
        padif = run_padif(torch, abi, W, stream, args)
    if "ensemble" in sec and args.members > 0:
        ensemble = run_ensemble(args, torch, np, abi, W, stream, rank, world)
    if rank == 0 and "adjoint" in sec and args.adj_calls > 0:
        adjoint = run_adjoint(args, torch, np, abi, W, stream)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        ns = len(W.make_workload(args.workload).grid.species)
        cpu = cpu_baseline_fresh(args.workload, ns, args.cpu_seconds)
        if single is not None:
            single["cpu_baseline"] = cpu_baseline_fresh("single_h", 1, args.cpu_seconds)
        if refined is not None:
            # a bounded sample: one timed call per variant (a few seconds each)
            refined["cpu_baseline"] = cpu_baseline_fresh("refined", 4, 0.0, calls=1, warmup=1, ref_warmup=0)
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": head["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": head["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": head["workload"], "step": "one ram_run call = 2 DTs steps",
                   "cells_per_step": head["cells_per_step"], "l2": "flushed between timed steps (256 MB write)",
                   "graph": not args.no_graph, "launch_shapes": head["launch_shapes"],
                   "autotune_trials": head["autotune_trials"], "item_groups": head["item_groups"],
                   "coef_store": "none" if args.no_coef_store else "DRIFTE",
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU"},
        "roofline": head["roofline"], "kernels_ms": head["kernels_ms"],
        "kernel_pass_ms_per_step": head["kernel_pass_ms_per_step"],
        "e2e": head.get("e2e"), "cpu_baseline": cpu, "clocks": head["clocks"], "gpu_launches": head["launches"],
        "single_species": single, "refined": refined, "padif": padif, "ensemble": ensemble, "adjoint": adjoint,
        "wall_s": head["wall_s"],
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.cpu_leg:
        cpu_leg_main(args)
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch

        torch.distributed.init_process_group("nccl" if args.impl == "gb300" else "gloo")
    try:
        if args.impl == "reference":
            run_reference(args, rank, world)
        else:
            run_gb300(args, rank, world, local_rank)
    finally:
        if world > 1:
            import torch

            torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
