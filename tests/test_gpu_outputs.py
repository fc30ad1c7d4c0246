"""GPU output products against the oracle: virtual-spacecraft samples
(SatFlux/OmnFlux) and the ram_sum_pressure hand-off, after ram_run calls on
the non-dipole grid, for a full member and for members with species
subsets."""
import numpy as np
import pytest

import pyoracle
from ramgpu import abi, sats as S, workload as W

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def test_fly_sats_and_sum_pressure_match_oracle():
    wl = W.make_workload("tiny_pert")
    g = wl.grid
    ns = len(g.species)
    lists = [[0, 1, 2, 3], [1, 3], [2]]
    gpu = abi.RamGpu(g, wl.fields, n_members=3)
    o = pyoracle.Oracle(g, wl.fields)
    try:
        f_or = {}
        for m, sl in enumerate(lists):
            gpu.set_member_species(m, sl)
            f_or[m] = {s: np.asfortranarray(wl.f2[s] * (1.0 + 0.1 * m)) for s in range(ns)}
            for s in sl:
                gpu.upload_f2(m, s, f_or[m][s])
                gpu.set_boundary(m, s, wl.fgeos[s])
        res = {}
        for call in range(2):
            gpu.set_kp(-1, 3.0 + call)
            gpu.ram_run(wl.dts)
            for m, sl in enumerate(lists):
                res[m] = o.ram_run(f_or[m], wl.fgeos, wl.dts, kp=3.0 + call, want_flux=True, species=sl)
        tracks = [S.circular_orbit(4.3, 2.0), S.circular_orbit(5.8, 20.5), S.circular_orbit(6.4, 11.0)]
        sats = [(m, *tr.position(7200.0 * (m + 1))) for m in range(3) for tr in tracks]
        sf, om = gpu.fly_sats(sats)
        for t, (m, lsh, mlt) in enumerate(sats):
            ef, eo = pyoracle.sat_samples(g, res[m]["flux"], [(m, lsh, mlt)], species_of={m: lists[m]})
            bad = ef[0] == pyoracle.BAD_DATA
            assert np.array_equal(sf[t] == abi.BAD_DATA, bad)
            assert _rel(sf[t][~bad], ef[0][~bad]) <= TOL
            assert np.array_equal(om[t] == abi.BAD_DATA, eo[0] == pyoracle.BAD_DATA)
            good = eo[0] != pyoracle.BAD_DATA
            assert _rel(om[t][good], eo[0][good]) <= TOL
        for m, sl in enumerate(lists):
            pall, ppar = gpu.sum_pressure(m)
            epall, eppar = pyoracle.sum_pressure(res[m]["ppert"], res[m]["ppart"], sl)
            assert _rel(pall, epall) <= TOL and _rel(ppar, eppar) <= TOL
            assert np.all(pall[0] == 0.0)  # PPERT/PPART are defined for I >= 2
    finally:
        gpu.close()
