"""Writes the golden fixtures of this directory from the reference's own code.

The reference's Fortran routines (src/ModRamDrift.f90, src/ModRamLoss.f90,
src/ModRamRun.f90) are translated to C by oracle/f90c.py and run by
oracle/refrun.py (RAM's own ram_run, src/ModRamRun.f90:16-225).  That needs
the reference's tree on the machine that runs this script; the fixtures
are committed so that tests elsewhere (the GPU machine) need neither.

  ram_run_tiny.json  : one ram_run call (Kp 3, DTs 5 s) of the four-species
                       workload on the non-dipole 6x9x35x72 test grid
                       (tiny_pert), given as per-species sums and 256
                       sampled cells of F2, the moments at 16 points, FLUX at
                       64 cells and DtsNext.
  ram_run_ramp.json  : three successive calls (Kp 1, 3.5, 6) on the 8x9x35x72
                       perturbed grid (tiny_pert8, stale DRIFTR ghosts and
                       clip events included), the same summaries per call.

Run:  python tests/golden/make_golden.py
"""
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path[:0] = [str(ROOT / "oracle"), str(ROOT / "ram-scb_gb300")]

import refrun  # noqa: E402
from ramgpu import workload as W  # noqa: E402

SEED = 20261203
SOURCE = "reference ram_run (src/ModRamRun.f90:16-225), translated by oracle/f90c.py"


def sample_indices(shape, n, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    return [tuple(int(rng.integers(d)) for d in shape) for _ in range(n)]


def summary(g, f2, out, seed):
    shp = (g.nr, g.nt, g.ne, g.npa)
    cells = sample_indices(shp, 256, seed)
    mom = sample_indices((g.nr, g.nt), 16, seed + 1)
    flx = sample_indices(shp, 64, seed + 2)
    sp = []
    for s in range(len(g.species)):
        sp.append({
            "sum": float(np.sum(f2[s])), "sum_sq": float(np.sum(f2[s] ** 2)),
            "cells": [[list(c), float(f2[s][c])] for c in cells],
            "ppert": [[list(c), float(out["ppert"][s][c])] for c in mom],
            "ppart": [[list(c), float(out["ppart"][s][c])] for c in mom],
            "flux": [[list(c), float(out["flux"][s][c])] for c in flx],
        })
    return sp


def make():
    if refrun.build() is None:
        raise SystemExit("the reference's tree (or a translated oracle/_ref/ramref.c) is needed")
    wl = W.make_workload("tiny_pert")
    g = wl.grid
    ref = refrun.RefRam(g, wl.fields)
    f2 = [np.asfortranarray(a).copy(order="F") for a in wl.f2]
    out = ref.ram_run(f2, wl.fgeos, wl.dts, 3.0)
    data = {"source": SOURCE, "workload": "tiny_pert", "kp": 3.0, "dts": wl.dts, "dts_next": out["dts_next"],
            "species": summary(g, f2, out, SEED)}
    (HERE / "ram_run_tiny.json").write_text(json.dumps(data, indent=1))

    wl = W.make_workload("tiny_pert8")
    g = wl.grid
    ref = refrun.RefRam(g, wl.fields)
    f2 = [np.asfortranarray(a).copy(order="F") for a in wl.f2]
    calls = []
    for c, kp in enumerate((1.0, 3.5, 6.0)):
        out = ref.ram_run(f2, wl.fgeos, wl.dts, kp)
        calls.append({"kp": kp, "dts_next": out["dts_next"],
                      "losses": [list(map(float, out["losses"][s])) for s in range(len(g.species))],
                      "species": summary(g, f2, out, SEED + 10 * (c + 1))})
    data = {"source": SOURCE, "workload": "tiny_pert8", "dts": wl.dts, "calls": calls}
    (HERE / "ram_run_ramp.json").write_text(json.dumps(data, separators=(",", ":")))


if __name__ == "__main__":
    make()
