#!/usr/bin/env python3
"""Benchmark of the GB300 RAM kinetic step.

Workload (default): the four-species step on the standard RAM grid
(e-, H+, He+, O+; NR=20 x NT=25 x NE=35 x NPA=72 = 1,260,000 cells per
species; dipole field, Volland-Stern potential with Kp rising 1->6 over
4320 DTs steps, DTs = 5 s).  One bench step is one ram_run call: the Strang
pair R,P,E,MU,CEX,ATMOL | ATMOL,CEX,MU,E,P,R for every species, the periodic
copy, the magnetopause mask, DtsNext and the ANISCH moments -- two DTs
steps, i.e. 2 x 4 x 1.26e6 = 10.08e6 cell-updates.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Prints one JSON line (rank 0).  Under torchrun every rank advances its own
replica of the workload on its own GPU (the path has no exchange step).
"""
from __future__ import annotations

import argparse
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
# FP64 instructions per cell of each sweep kernel (csrc/sweeps.cu): ncu's
# sm__inst_executed_pipe_fp64 x 32 lanes / cells, the mean of its forward
# and reverse launches on the four-species standard grid (the forward E and
# MU carry the CFL quotient's multiply; DRIFTE's forward computes and stores
# its face coefficients, the reverse loads them).  Per face this is the
# formulation's own count: X, coefficient, a-term, face fma and the two
# update operations (beta*|X|, the CFL quotients and the flux C*FBND are
# formed on the integer pipe); DRIFTMU's lines are split between lane
# pairs, whose second lane recomputes the face at the split.
FP64_OPS_PER_CELL = {"driftr": 6.22, "driftp": 5.55, "drifte": 0.5 * (6.71 + 4.78), "driftmu": 0.5 * (6.81 + 5.84)}
# DRAM bytes (read + write) per launch of each sweep on the four-species
# standard grid, the mean of its forward and reverse launches in one ncu
# capture (profiles/sweeps_four_sp.md, current kernels): F2 is read once
# and the written lines stay in L2 within a launch; the forward MU also
# reads the fused CEX/ATMOL factor, and DRIFTE stores and reloads its face
# coefficients.
NCU_DRAM_BYTES = {"four_sp": {"driftr": 0.5 * (44.6e6 + 44.3e6), "driftp": 0.5 * (40.6e6 + 40.6e6),
                               "drifte": 0.5 * (111.0e6 + 129.8e6), "driftmu": 0.5 * (81.8e6 + 40.3e6)}}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="four_sp", choices=["four_sp", "single_h", "refined"])
    ap.add_argument("--cpu-seconds", type=float, default=6.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--flush-mb", type=int, default=256)
    ap.add_argument("--no-graph", action="store_true")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--no-padif", action="store_true", help="skip the step timed with WPADIF on")
    ap.add_argument("--no-coef-store", action="store_true",
                    help="recompute the face coefficients in the reverse half instead of storing them")
    ap.add_argument("--members", type=int, default=256, help="ensemble members (0: skip)")
    ap.add_argument("--ensemble-steps", type=int, default=6)
    ap.add_argument("--loop-members", type=int, default=16)
    ap.add_argument("--adj-calls", type=int, default=720,
                    help="adjoint window in ram_run calls (720 = 1440 DTs steps = 2 h); 0: skip")
    ap.add_argument("--adj-ckpt", type=int, default=32, help="checkpoint spacing in calls (32 = 64 steps)")
    ap.add_argument("--adj-fd", type=int, default=4, help="finite-difference directions on the full window")
    ap.add_argument("--adj-members", type=int, default=64, help="batched-gradient members (0: skip)")
    ap.add_argument("--adj-member-calls", type=int, default=36)
    ap.add_argument("--only", choices=["adjoint"], default=None,
                    help="run one section alone (profiling); prints its result as JSON")
    # internal: one CPU-oracle timing in a fresh process (see cpu_leg_fresh)
    ap.add_argument("--cpu-leg", default=None, help=argparse.SUPPRESS)
    ap.add_argument("--cpu-outer", type=int, default=1, help=argparse.SUPPRESS)
    ap.add_argument("--cpu-inner", type=int, default=1, help=argparse.SUPPRESS)
    ap.add_argument("--cpu-calls", type=int, default=0, help=argparse.SUPPRESS)
    ap.add_argument("--cpu-warmup", type=int, default=1, help=argparse.SUPPRESS)
    return ap.parse_args()


def workload_desc(wl):
    g = wl.grid
    return (f"{wl.name}: {len(g.species)} species ({','.join(wl.meta['species'])}) "
            f"{g.nr}x{g.nt}x{g.ne}x{g.npa}, Kp ramp 1->6 (VOLS), DTs={wl.dts}s")


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


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


def cpu_leg_main(args):
    """--cpu-leg: time the CPU oracle in this process (which never imports
    torch or the CUDA library) and print one JSON object."""
    from ramgpu import workload as W

    wl = W.make_workload(args.cpu_leg)
    v, n, el = cpu_time_oracle(wl, args.cpu_seconds, args.cpu_outer, args.cpu_inner,
                               calls=args.cpu_calls if args.cpu_calls > 0 else None, warmup=args.cpu_warmup)
    print(json.dumps({"value": v, "calls": n, "elapsed_s": el, "outer": args.cpu_outer, "inner": args.cpu_inner}),
          flush=True)


def cpu_leg_fresh(workload, outer, inner, calls=0, seconds=10.0, warmup=1):
    """The CPU oracle timed in a fresh interpreter: the measuring process
    holds no CUDA context, torch thread pool or GPU work of its own, so the
    figure is the one a reference run on the same cores would see (timed in
    the GPU process after its GPU sections, the line threads inside each
    species did not run: the leg measured the species-threads-only rate)."""
    cmd = [sys.executable, str(ROOT / "bench.py"), "--cpu-leg", workload, "--cpu-outer", str(outer),
           "--cpu-inner", str(inner), "--cpu-calls", str(calls), "--cpu-seconds", str(seconds),
           "--cpu-warmup", str(warmup)]
    r = subprocess.run(cmd, capture_output=True, text=True, check=True)
    return json.loads(r.stdout.strip().splitlines()[-1])


def cpu_baseline_fresh(workload, ns, seconds):
    """Both CPU variants of the reference's path, each in a fresh process:
    (1) OpenMP over species only, as the reference (at most nS threads);
    (2) every host core: species threads x line threads inside each routine.
    The line's value is variant 2."""
    cores = os.cpu_count() or 1
    o2, i2 = cpu_threads(ns)
    v1 = cpu_leg_fresh(workload, min(ns, cores), 1, seconds=seconds)
    v2 = cpu_leg_fresh(workload, o2, i2, seconds=seconds)
    return {"value": v2["value"], "unit": UNIT, "cores": o2 * i2, "kind": "port",
            "sample": (f"{v2['calls']} ram_run calls of the workload in {v2['elapsed_s']:.1f} s after 1 warm-up call, "
                       f"fresh process; C restatement of the reference routines (-O3 -ffp-contract=off, no Fortran "
                       f"compiler), OpenMP over {o2} species x {i2} line threads"),
            "variants": {"species_threads": {"value": v1["value"], "threads": v1["outer"], "calls": v1["calls"],
                                             "elapsed_s": v1["elapsed_s"]},
                         "all_cores": {"value": v2["value"], "threads": o2 * i2, "calls": v2["calls"],
                                       "elapsed_s": v2["elapsed_s"]}}}


def run_reference(args, rank, world):
    from ramgpu import workload as W

    if rank != 0:
        return
    wl = W.make_workload(args.workload)
    ns = len(wl.grid.species)
    outer, inner = cpu_threads(ns)
    # W untimed warm-up steps, then exactly K timed steps; a step is one
    # ram_run call of the workload (about 0.3 s on 16 host cores)
    v, n, el = cpu_time_oracle(wl, 0.0, outer, inner, calls=max(1, args.steps), warmup=args.warmup)
    sample = (f"{n} ram_run calls of the workload ({workload_desc(wl)}) after {args.warmup} warm-up "
              f"calls, {el:.1f} s; C restatement of the reference routines (no Fortran compiler), "
              f"OpenMP over {outer} species x {inner} line threads")
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": n, "warmup": args.warmup, "ms_per_step": 1e3 * el / n, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": workload_desc(wl), "step": "one ram_run call (2 DTs steps)"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": outer * inner, "kind": "port",
                             "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------ GPU leg
def run_ensemble(args, torch, dev, stream):
    """Batched ensemble (256 uneven members on the standard grid) against
    looping the plain single-member GPU step; returns a dict for the line."""
    import numpy as np

    from ramgpu import abi, workload as W

    ens = W.make_ensemble(args.members)
    base = ens.base
    g = base.grid
    gpu = abi.RamGpu(g, base.fields, n_members=ens.members)
    gpu.set_stream(stream.cuda_stream)
    for m in range(ens.members):
        gpu.set_member_species(m, ens.species[m])
        for s in ens.species[m]:
            gpu.upload_f2(m, s, base.f2[s] * ens.scale[m])
            gpu.set_boundary(m, s, base.fgeos[s] * ens.scale[m])
    t0 = 356  # sample from DTs step 356 on: members with length < t0 + 2K retire inside it
    gpu.set_kp_all(ens.kp(t0))
    shapes, _ = gpu.autotune(base.dts)
    gpu_groups = gpu.step_groups()
    gpu.set_graph(True)
    flush = torch.empty(max(1, args.flush_mb) << 20, dtype=torch.uint8, device=dev)
    for w in range(2):  # warm-up (captures the graph)
        gpu.ram_run(base.dts)
    K = max(2, min(args.ensemble_steps, 20))
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    member_steps = 0
    cell_updates = 0
    dead = set()
    for k in range(K):
        step = t0 + 2 * k
        for m in range(ens.members):  # finished members retire
            if step >= ens.length[m] and m not in dead:
                gpu.set_member_active(m, False)
                dead.add(m)
        active = [m for m in range(ens.members) if step < ens.length[m]]
        member_steps += 2 * len(active)
        cell_updates += 2 * g.ncell * sum(len(ens.species[m]) for m in active)
        gpu.set_kp_all(ens.kp(step))
        with torch.cuda.stream(stream):
            flush.fill_(k & 0xFF)
        ev[k][0].record(stream)
        gpu.ram_run_async(base.dts)
        ev[k][1].record(stream)
    torch.cuda.synchronize(dev)
    batched_s = sum(a.elapsed_time(b) for a, b in ev) / 1e3
    retired = len(dead)
    # looped: the plain single-member step (direct launches), one member at a time
    gpu.set_graph(False)
    sub = list(range(0, ens.members, max(1, ens.members // args.loop_members)))[:args.loop_members]
    for m in range(ens.members):
        gpu.set_member_active(m, False)
    lev = []
    for m in sub:
        gpu.set_member_active(m, True)
        gpu.set_kp_all(ens.kp(t0))
        gpu.ram_run(base.dts)  # warm (rebuilds the work list)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            flush.fill_(m & 0xFF)
        a.record(stream)
        gpu.ram_run_async(base.dts)
        b.record(stream)
        torch.cuda.synchronize(dev)
        lev.append(a.elapsed_time(b) / 1e3)
        gpu.set_member_active(m, False)
    looped_per_member = statistics.mean(lev)
    gpu.close()
    batched = member_steps / batched_s
    looped = 2.0 / looped_per_member
    return {"members": ens.members, "member_species": int(sum(len(x) for x in ens.species)),
            "steps": K, "retired_in_sample": retired,
            "member_steps_per_s_batched": batched, "member_steps_per_s_looped": looped,
            "batched_over_looped": batched / looped,
            "cell_updates_per_s_batched": cell_updates / batched_s,
            "looped_sample_members": len(sub), "launch_shapes": shapes,
            "item_groups": gpu_groups,
            "notes": "batched: one graph-replayed ram_run per step for all active members; "
                     "looped: the plain direct-launch step of one member at a time"}


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


def run_adjoint(args, torch, dev, stream):
    """Adjoint window on the four-species standard grid: 1440 DTs steps
    (720 ram_run calls, Kp 1->6 ramp), 50 virtual-spacecraft samples on
    circular equatorial orbits at L = 4-6, 10-200 keV, pitch-angle bin 2;
    checkpoints every 64 steps.  Reports adjoint cost over the plain forward,
    finite-difference checks on the full window, and a 64-member batched
    gradient against looping single-member gradients."""
    import numpy as np

    from ramgpu import abi, sats, workload as W

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

    reset()
    gpu.autotune(wl.dts)
    gpu.set_graph(True)
    for c in range(2):
        gpu.set_kp(-1, kp[c, 0])
        gpu.ram_run(wl.dts)
    reset()
    torch.cuda.synchronize(dev)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for c in range(nc):
        gpu.set_kp(-1, kp[c, 0])
        gpu.ram_run_async(wl.dts)
    b.record(stream)
    torch.cuda.synchronize(dev)
    fwd_s = a.elapsed_time(b) / 1e3
    reset()
    gpu.adj_forward(2, wl.dts, kp[:2], 1, [])  # warm-up of the adjoint buffers and kernels
    gpu.adj_backward()
    # the library's policy: checkpoints every kc calls, the record ring keeps
    # as many trailing segments as half of the free HBM holds (here all)
    reset()
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    J = gpu.adj_forward(nc, wl.dts, kp, kc, obs)[0]
    t1 = time.perf_counter()
    gf, gb = gpu.adj_backward()
    t2 = time.perf_counter()
    nseg, nkeep = gpu.adj_segments()
    # the same window with a one-segment ring: every earlier segment is
    # recomputed from its checkpoint (the policy for windows that do not fit)
    gpu.set_adj_record_budget(0)
    reset()
    torch.cuda.synchronize(dev)
    t3 = time.perf_counter()
    gpu.adj_forward(nc, wl.dts, kp, kc, obs)
    t4 = time.perf_counter()
    gfr, gbr = gpu.adj_backward()
    t5 = time.perf_counter()
    gpu.set_adj_record_budget(-1)
    same_r = max(float(np.max(np.abs(gfr - gf)) / np.max(np.abs(gf))),
                 float(np.max(np.abs(gbr - gb)) / max(np.max(np.abs(gb)), 1e-300)))
    # and as one segment (k = ncalls): the record of every call, no checkpoints
    reset()
    gpu.adj_forward(nc, wl.dts, kp, nc, obs)
    gf2, gb2 = gpu.adj_backward()
    same = max(float(np.max(np.abs(gf2 - gf)) / np.max(np.abs(gf))),
               float(np.max(np.abs(gb2 - gb)) / max(np.max(np.abs(gb)), 1e-300)))
    rng = np.random.Generator(np.random.PCG64(707))

    def fd_f2(r, eps, frozen):
        jj = []
        for sign in (1.0, -1.0):
            for s in range(ns):
                gpu.upload_f2(0, s, np.asarray(wl.f2[s]) * (1.0 + sign * eps * r[s]))
            jj.append(gpu.adj_replay()[0] if frozen else gpu.adj_forward(nc, wl.dts, kp, nc, obs)[0])
        return (jj[0] - jj[1]) / (2 * eps)

    # finite differences of the frozen-limiter scheme (the record of the base
    # run replayed): exact check of the adjoint on the whole window
    # (J is the log of affine fluxes: Richardson extrapolation of two central
    # differences removes the O(eps^2) term)
    fd = []
    for d in range(max(0, args.adj_fd)):
        r = [rng.uniform(-1.0, 1.0, size=wl.f2[s].shape) for s in range(ns)]
        ad = sum(float(np.sum(gf2[0, s] * np.asarray(wl.f2[s]) * r[s])) for s in range(ns))
        est = (4.0 * fd_f2(r, 1e-5, True) - fd_f2(r, 2e-5, True)) / 3.0
        fd.append(abs(est - ad) / abs(ad))
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
           "J": J, "forward_s": fwd_s, "adj_forward_s": t1 - t0, "adj_backward_s": t2 - t1,
           "adjoint_over_forward": (t2 - t0) / fwd_s,
           "segments": nseg, "segments_kept": nkeep, "record_bytes": 8 * g.ncell * ns * nc,
           "policy": "checkpoints every checkpoint_calls calls; the branch-record ring keeps the last "
                     "segments_kept segments (half of the free HBM as budget) and recomputes the rest",
           "recompute": {"segments_kept": 1, "segments_recomputed": nseg - 1,
                         "adj_forward_s": t4 - t3, "adj_backward_s": t5 - t4,
                         "adjoint_over_forward": (t5 - t3) / fwd_s,
                         "gradient_vs_kept_max_rel_diff": same_r},
           "single_segment_gradient_max_rel_diff": same,
           "fd_frozen_directions": len(fd), "fd_frozen_max_rel_err": max(fd) if fd else None,
           "fd_frozen_eps": "Richardson of 1e-5 and 2e-5", "fd_unfrozen_rel_err": unfrozen,
           "forward": "graph-replayed ram_run per call",
           "adjoint": "recording forward with checkpoints + recompute of the segments not kept + transposed sweeps"}
    if args.adj_members > 0:
        out["batched"] = run_adjoint_batched(args, torch, dev, stream)
    return out


def run_adjoint_batched(args, torch, dev, stream):
    import numpy as np

    from ramgpu import abi, sats, workload as W

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

    reset(gpu, range(nm))
    gpu.set_graph(True)
    gpu.set_kp_all(kp[0])
    gpu.ram_run(base.dts)
    reset(gpu, range(nm))
    torch.cuda.synchronize(dev)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for c in range(nc):
        gpu.set_kp_all(kp[c])
        gpu.ram_run_async(base.dts)
    b.record(stream)
    torch.cuda.synchronize(dev)
    fwd_s = a.elapsed_time(b) / 1e3
    reset(gpu, range(nm))
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    J = gpu.adj_forward(nc, base.dts, kp, kc, obs)
    gf, gb = gpu.adj_backward()
    batched_s = time.perf_counter() - t0
    gpu.close()
    # looped: the same gradients one member at a time
    sub = list(range(0, nm, max(1, nm // 4)))[:4]
    solo = abi.RamGpu(g, base.fields, n_members=1)
    solo.set_stream(stream.cuda_stream)
    loop_s, agree = [], 0.0
    for m in sub:
        reset(solo, [m])
        obs_m = [dict(o, member=0) for o in obs if o["member"] == m]
        solo.adj_forward(1, base.dts, kp[:1, m], 1, [])  # warm-up
        solo.adj_backward()
        reset(solo, [m])
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        Jm = solo.adj_forward(nc, base.dts, kp[:, m], kc, obs_m)
        gfm, _ = solo.adj_backward()
        loop_s.append(time.perf_counter() - t0)
        for s in ens.species[m]:
            agree = max(agree, float(np.max(np.abs(gfm[0, s] - gf[m, s])) / max(np.max(np.abs(gf[m, s])), 1e-300)))
    solo.close()
    looped = 1.0 / statistics.mean(loop_s)
    return {"members": nm, "member_species": int(sum(len(x) for x in ens.species)), "window_calls": nc,
            "checkpoint_calls": kc, "observations": len(obs), "forward_s": fwd_s, "adjoint_s": batched_s,
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
    if args.only == "adjoint":
        stream = torch.cuda.Stream(device=dev)
        print(json.dumps({"adjoint": run_adjoint(args, torch, dev, stream)}), flush=True)
        return
    wl = W.make_workload(args.workload)
    g = wl.grid
    ns = len(g.species)
    gpu = abi.RamGpu(g, wl.fields)
    stream = torch.cuda.Stream(device=dev)
    gpu.set_stream(stream.cuda_stream)
    for s in range(ns):
        gpu.upload_f2(0, s, wl.f2[s])
        gpu.set_boundary(0, s, wl.fgeos[s])
    cells_per_step = 2 * g.ncell * ns
    flush = torch.empty(max(1, args.flush_mb) << 20, dtype=torch.uint8, device=dev)  # > 129 MB L2

    def kp_at(step):
        return wl.kp(2 * step)

    gpu.set_kp(-1, kp_at(0))
    if args.no_coef_store:
        gpu.set_coef_store(0)
    shapes, _ = gpu.autotune(wl.dts) if not args.no_autotune else (gpu.launch_shape(), None)
    # species groups on concurrent streams (autotuned; ramgpu_set_step_groups)
    item_groups = gpu.step_groups()
    gpu.set_graph(not args.no_graph)
    # warm-up (builds the DTs tables, captures the graph)
    for w in range(args.warmup):
        gpu.set_kp(-1, kp_at(w))
        gpu.ram_run(wl.dts)
    torch.cuda.synchronize(dev)
    if world > 1:
        torch.distributed.barrier()
    clocks = ClockSampler(local_rank)
    clocks.start()
    time.sleep(0.3)
    launches0 = gpu.launch_count()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    torch.cuda.synchronize(dev)
    # an NVTX range marks the timed steps, so that a profiler can select
    # exactly their launches (ncu --nvtx --nvtx-include "ram_run_timed/")
    nvtx = getattr(torch.cuda, "nvtx", None)
    if nvtx is not None:
        nvtx.range_push("ram_run_timed")
    wall0 = time.perf_counter()
    for k in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(k & 0xFF)
        gpu.set_kp(-1, kp_at(args.warmup + k))
        ev[k][0].record(stream)
        gpu.ram_run_async(wl.dts)
        ev[k][1].record(stream)
    torch.cuda.synchronize(dev)
    wall = time.perf_counter() - wall0
    if nvtx is not None:
        nvtx.range_pop()
    launches = gpu.launch_count() - launches0
    clk = clocks.stop()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    total_ms = sum(step_ms)
    if world > 1:
        total_ms = max_over_ranks(total_ms, dev)
    value = world * cells_per_step * args.steps / (total_ms / 1e3)

    # per-kernel durations: a second timed pass with events around every
    # launch group on the launching stream (timing mode bypasses the graph)
    gpu.set_timing(True)
    gpu.kernel_times()
    kt_ms = []
    for k in range(max(3, min(args.steps, 10))):
        with torch.cuda.stream(stream):
            flush.fill_(k & 0xFF)
        gpu.set_kp(-1, kp_at(k))
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        gpu.ram_run_async(wl.dts)
        b.record(stream)
        torch.cuda.synchronize(dev)
        kt_ms.append(a.elapsed_time(b))
    ktimes = gpu.kernel_times()
    gpu.set_timing(False)

    # dominant kernel and its roofline (per launch)
    hbm_peak, peak_kind = measured_peaks()
    sweep = {k: v for k, v in ktimes.items() if k.startswith("drift")}
    dom = max(sweep, key=lambda k: sweep[k][0])
    dom_ms = sweep[dom][0] / sweep[dom][1]
    nitems = ns
    bytes_per_launch = 16.0 * g.ncell * nitems  # F2 read + write once per sweep
    achieved = bytes_per_launch / (dom_ms / 1e3) / 1e9
    nfaces = g.ncell * nitems
    fp64 = FP64_OPS_PER_CELL[dom] * nfaces / (dom_ms / 1e3) / 1e9
    fp64_peak = abi.probe_fp64() / 1e9

    # end-to-end through the C ABI with host buffers (pinned), full F2 in and
    # out every step, as the reference's host array F2 is
    e2e_steps = 0 if args.no_e2e else max(3, min(30, args.steps))
    nm2 = g.nr * g.nt
    pin = [torch.empty(g.ncell, dtype=torch.float64, pin_memory=True) for _ in range(ns)]
    host = [np.reshape(p.numpy(), (g.nr, g.nt, g.ne, g.npa), order="F") for p in pin]
    mom = torch.empty(2 * ns * nm2, dtype=torch.float64, pin_memory=True).numpy()
    pe_h = [mom[s * nm2:(s + 1) * nm2] for s in range(ns)]
    pa_h = [mom[(ns + s) * nm2:(ns + s + 1) * nm2] for s in range(ns)]
    for s in range(ns):
        host[s][...] = gpu.download_f2(0, s)
    lib, h = gpu.lib, gpu.h
    hp = [a.ctypes.data_as(abi._P) for a in host]

    def e2e_pipelined(k):
        # ramgpu_ram_run_host: uploads, sweeps and read-back of F2 and the
        # moments of every species, pipelined over species groups
        gpu.set_kp(-1, kp_at(k))
        gpu.ram_run_host(wl.dts, host, pe_h, pa_h)

    host_pg = [np.asfortranarray(a).copy(order="F") for a in host]  # ordinary (pageable) memory
    pe_pg = [np.zeros(nm2) for _ in range(ns)]
    pa_pg = [np.zeros(nm2) for _ in range(ns)]

    def e2e_pageable(k):
        # the same call from ordinary host arrays, as a Fortran caller's F2:
        # the SMs move them over the coherent host link
        gpu.set_kp(-1, kp_at(k))
        gpu.ram_run_host(wl.dts, host_pg, pe_pg, pa_pg)

    def e2e_serial(k):
        # the same traffic as one stream: uploads, ram_run, read-back, wait
        for s in range(ns):
            gpu._ck(lib.ramgpu_upload_f2_async(h, 0, s, hp[s]), "upload")
        gpu.set_kp(-1, kp_at(k))
        gpu.ram_run_async(wl.dts)
        for s in range(ns):
            gpu._ck(lib.ramgpu_download_f2_async(h, 0, s, hp[s]), "download")
            gpu._ck(lib.ramgpu_moments_async(h, 0, s, pe_h[s].ctypes.data_as(abi._P),
                                             pa_h[s].ctypes.data_as(abi._P)), "moments")
        gpu._ck(lib.ramgpu_synchronize(h), "synchronize")

    e2e_med = {}

    def e2e_time(fn):
        fn(0)  # warm (first use creates the group streams)
        torch.cuda.synchronize(dev)
        ts = []
        t0 = time.perf_counter()
        for k in range(e2e_steps):
            t1 = time.perf_counter()
            fn(k)
            ts.append(time.perf_counter() - t1)
        e2e_med[fn.__name__] = 1e3 * statistics.median(ts)
        return max(time.perf_counter() - t0, 1e-9)

    e2e = {"value": None, "unit": UNIT, "h2d_bytes_per_step": 8 * g.ncell * ns,
           "d2h_bytes_per_step": 8 * g.ncell * ns + 16 * nm2 * ns,
           "path": "ramgpu_set_kp + ramgpu_ram_run_host (page-locked host F2 of 4 species in and out, "
                   "moments of 4 species out; pipelined over 4 species groups), every step"}
    if e2e_steps:
        e2e["value"] = world * cells_per_step * e2e_steps / e2e_time(e2e_pipelined)
        e2e["pageable_value"] = world * cells_per_step * e2e_steps / e2e_time(e2e_pageable)
        e2e["serial_value"] = world * cells_per_step * e2e_steps / e2e_time(e2e_serial)
        e2e["ms_per_step_median"] = {"pipelined": e2e_med["e2e_pipelined"], "pageable": e2e_med["e2e_pageable"],
                                     "serial": e2e_med["e2e_serial"]}
        e2e["pageable_path"] = "ramgpu_ram_run_host with ordinary (pageable) host arrays"
        e2e["serial_path"] = ("ramgpu_upload_f2_async x4 + ramgpu_ram_run_async + ramgpu_download_f2_async x4 "
                              "+ ramgpu_moments_async x4 + ramgpu_synchronize on one stream")
    # the same step with WPADIF on the electrons (both halves), per-kernel timed
    padif = None
    if not args.no_padif:
        gpu.set_pa_diffusion(0, W.pa_diffusion(g, wl.fields))
        gpu.set_timing(True)
        gpu.kernel_times()
        pd_ms = []
        for k in range(3):
            with torch.cuda.stream(stream):
                flush.fill_(k & 0xFF)
            gpu.set_kp(-1, kp_at(k))
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            gpu.ram_run_async(wl.dts)
            b.record(stream)
            torch.cuda.synchronize(dev)
            pd_ms.append(a.elapsed_time(b))
        kt = gpu.kernel_times()
        gpu.set_timing(False)
        gpu.set_pa_diffusion(0, None)
        pk = kt.get("padif", (0.0, 1))
        per = pk[0] / max(pk[1], 1)
        # algorithmic bytes of the two launches per step: the electrons' solve
        # reads F2 and the three elimination tables and writes F2 (40 B per
        # cell) in both; the first also applies the loss factor to the other
        # three species (F2 and factor in, F2 out: 24 B per cell)
        byts = 0.5 * (40.0 + 40.0 + 3 * 24.0) * g.ncell
        padif = {"species": "Electron (WPADIF after the drifts and before the reverse drifts)",
                 "step_ms": statistics.mean(pd_ms), "step_ms_without": statistics.mean(kt_ms),
                 "kernel_ms_per_launch": per, "launches": pk[1],
                 "algorithmic_GBps": byts / (per / 1e3) / 1e9 if per > 0 else None}
    gpu.close()

    ensemble = None
    if rank == 0 and args.members > 0:
        ensemble = run_ensemble(args, torch, dev, stream)
    adjoint = None
    if rank == 0 and args.adj_calls > 0:
        adjoint = run_adjoint(args, torch, dev, stream)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline_fresh(args.workload, ns, args.cpu_seconds)
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": workload_desc(wl), "step": "one ram_run call = 2 DTs steps",
                   "cells_per_step": cells_per_step, "l2": "flushed between timed steps (256 MB write)",
                   "graph": not args.no_graph, "launch_shapes": shapes,
                   "item_groups": item_groups,
                   "coef_store": "none" if args.no_coef_store else "DRIFTE",
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved / hbm_peak,
                     "traffic": NCU_DRAM_BYTES.get(args.workload, {}).get(dom), "kernel": dom,
                     "kernel_ms": dom_ms, "peak_kind": peak_kind,
                     "fp64": {"achieved": fp64, "peak": fp64_peak, "unit": "G lane-ops/s",
                              "frac": fp64 / fp64_peak, "ops_per_cell": FP64_OPS_PER_CELL[dom],
                              "peak_kind": "measured live (fma loop, ramgpu_probe_fp64)"},
                     # whole-step views: the fused minimum (F2 read and written once per
                     # DTs step, 16 B per cell-update) and the unfused sweep sequence
                     # (4 sweeps x 16 B + CEX 16 B = 80 B per cell-update)
                     "step": {"fused_min_GBps": value * 16 / 1e9, "fused_min_frac": value * 16 / 1e9 / hbm_peak,
                              "unfused_GBps": value * 80 / 1e9, "unfused_frac": value * 80 / 1e9 / hbm_peak}},
        "kernels_ms": {k: round(v[0] / v[1], 5) for k, v in ktimes.items()},
        "kernel_pass_ms_per_step": statistics.mean(kt_ms),
        "e2e": e2e, "cpu_baseline": cpu, "clocks": clk, "gpu_launches": launches,
        "padif": padif, "ensemble": ensemble, "adjoint": adjoint, "wall_s": wall,
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
