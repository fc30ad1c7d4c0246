"""Writes the golden fixtures of this directory from the oracle.

The reference (Fortran 90) cannot be built here, so these vectors pin the
oracle's own results on seeded inputs -- a regression fixture for the
oracle and a compact target for the GPU path that needs no CPU run:

  ram_run_tiny.json : one ram_run call (Kp 3, DTs 5 s) of the four-species
                      workload on the non-dipole 6x9x35x72 test grid, given
                      as per-species sums and 256 sampled cells of F2, the
                      moments at 16 points, FLUX at 64 cells and DtsNext.

Run:  python tests/golden/make_golden.py
"""
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path[:0] = [str(ROOT / "oracle"), str(ROOT / "ram-scb_gb300")]

import pyoracle  # noqa: E402
from ramgpu import workload as W  # noqa: E402

KP = 3.0
SEED = 20261203


def sample_indices(shape, n, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    return [tuple(int(rng.integers(d)) for d in shape) for _ in range(n)]


def make():
    wl = W.make_workload("tiny_pert")
    g = wl.grid
    o = pyoracle.Oracle(g, wl.fields)
    f2 = [np.asfortranarray(a).copy(order="F") for a in wl.f2]
    out = o.ram_run(f2, wl.fgeos, wl.dts, kp=KP, want_flux=True)
    shp = (g.nr, g.nt, g.ne, g.npa)
    cells = sample_indices(shp, 256, SEED)
    mom = sample_indices((g.nr, g.nt), 16, SEED + 1)
    flx = sample_indices(shp, 64, SEED + 2)
    data = {"workload": "tiny_pert", "kp": KP, "dts": wl.dts, "dts_next": out["dts_next"], "species": []}
    for s in range(len(g.species)):
        data["species"].append({
            "sum": float(np.sum(f2[s])), "sum_sq": float(np.sum(f2[s] ** 2)),
            "cells": [[list(c), float(f2[s][c])] for c in cells],
            "ppert": [[list(c), float(out["ppert"][s][c])] for c in mom],
            "ppart": [[list(c), float(out["ppart"][s][c])] for c in mom],
            "flux": [[list(c), float(out["flux"][s][c])] for c in flx],
        })
    (HERE / "ram_run_tiny.json").write_text(json.dumps(data, indent=1))


if __name__ == "__main__":
    make()
