"""The C oracle against the reference's own routines, bit for bit.

oracle/f90c.py translates the reference's Fortran (src/ModRamDrift.f90,
src/ModRamLoss.f90, src/ModRamRun.f90 and their modules) to C and gcc
builds it (with array bounds checks in libramref_check.so);
oracle/refrun.py runs the reference's ram_run (src/ModRamRun.f90:16-225)
and its single routines on the same inputs as the oracle.  Every output is
compared for exact equality: F2, the moments, FLUX, VT, DtsNext, the
DtDrift minima, the SUMRC loss bookkeeping, CHARGE/ATLOS and the CDrift
coefficient arrays of each sweep; beside the step, the grid construction
(ARRAYS, src/ModRamInit.f90), the implicit pitch-angle diffusion (WPADIF,
src/ModRamWPI.f90; FLCscatter, src/ModRamLoss.f90) and ram_sum_pressure
(src/ModRamFunctions.f90).

Needs the reference's tree (to translate) or a translated oracle/_ref/ramref.c.
"""
import numpy as np
import pytest

import pyoracle
import refrun
from ramgpu import workload as W

pytestmark = pytest.mark.skipif(refrun.build() is None,
                                reason="translated reference unavailable (no reference tree, no oracle/_ref/ramref.c)")


def _runs(name, kps, check):
    wl = W.make_workload(name)
    g = wl.grid
    ref = refrun.RefRam(g, wl.fields, check=check)
    o = pyoracle.Oracle(g, wl.fields)
    f_ref = [np.asfortranarray(a).copy(order="F") for a in wl.f2]
    f_or = [np.asfortranarray(a).copy(order="F") for a in wl.f2]
    losses = {s: (0.0, 0.0, 0.0, 0.0) for s in range(len(g.species))}
    for kp in kps:
        r = ref.ram_run(f_ref, wl.fgeos, wl.dts, kp)
        out = o.ram_run(f_or, wl.fgeos, wl.dts, kp=kp, want_flux=True, losses=losses)
        losses = out["losses"]
        yield g, ref, r, out, f_ref, f_or


@pytest.mark.parametrize("name", ["tiny", "tiny_pert", "tiny_pert8"])
def test_ram_run_bit_for_bit(name):
    """Three calls along a Kp ramp (bounds-checked build of the reference)."""
    for g, ref, r, out, f_ref, f_or in _runs(name, (1.0, 3.5, 6.0), check=True):
        for s in range(len(g.species)):
            assert np.array_equal(f_ref[s], f_or[s]), s
            assert np.array_equal(r["ppert"][s], out["ppert"][s]), s
            assert np.array_equal(r["ppart"][s], out["ppart"][s]), s
            assert np.array_equal(r["flux"][s], out["flux"][s]), s
            assert r["losses"][s] == tuple(out["losses"][s]), s
        assert np.array_equal(r["vt"], out["vt"])
        assert r["dts_next"] == out["dts_next"]
        assert ref.stubs() == {"coulpara": len(g.species)}


def test_standard_grid_bit_for_bit():
    """The 20x25x35x72 four-species step (e-, H+, He+, O+), one call."""
    for g, ref, r, out, f_ref, f_or in _runs("four_sp", (3.0,), check=False):
        for s in range(len(g.species)):
            assert np.array_equal(f_ref[s], f_or[s]), s
            assert np.array_equal(r["ppert"][s], out["ppert"][s]), s
            assert np.array_equal(r["flux"][s], out["flux"][s]), s
        assert r["dts_next"] == out["dts_next"]


@pytest.mark.parametrize("which,routine", [("R", "driftr"), ("P", "driftp"), ("E", "drifte"), ("MU", "driftmu")])
def test_single_sweeps_and_coefficients(which, routine):
    """DRIFTPARA then one sweep of the reference on every species of the
    perturbed grid (stale DRIFTR ghosts included): F2, the CDrift array
    and the DtDrift minimum."""
    wl = W.make_workload("tiny_pert8")
    g = wl.grid
    ref = refrun.RefRam(g, wl.fields, check=True)
    o = pyoracle.Oracle(g, wl.fields)
    kp = 4.0
    vt = o.vt_vols(kp)
    ref.a["vt"][...] = vt
    ref.set("modramtiming::dts", wl.dts)
    for s in range(len(g.species)):
        ref.a["f2"][s] = wl.f2[s]
        ref.a["fgeos"][s] = wl.fgeos[s]
        ref.subroutine("driftpara", s)
        ref.subroutine(routine, s)
        f = np.asfortranarray(wl.f2[s]).copy(order="F")
        cd = np.zeros_like(f, order="F")
        dt = o.sweep(which, s, f, vt, wl.dts, fgeos=wl.fgeos[s], cdrift=cd)
        assert np.array_equal(ref.a["f2"][s], f), s
        assert np.array_equal(ref.view("modramdrift::cdrift" + which.lower()), cd), s
        assert ref.view("modramvariables::dtdrift" + which.lower())[s] == dt, s
        ref.call("driftend")


def test_cepara_tables():
    """CHARGE (analytic H+, He+, O+ cross sections; none for e-) and ATLOS."""
    wl = W.make_workload("tiny_pert")
    g = wl.grid
    ref = refrun.RefRam(g, wl.fields)
    o = pyoracle.Oracle(g, wl.fields)
    ref.set("modramtiming::dts", wl.dts)
    for s in range(len(g.species)):
        ref.subroutine("cepara", s)
        charge, atlos = o.cepara(s, wl.dts)
        assert np.array_equal(ref.a["charge"][s], charge), s
        assert np.array_equal(ref.a["atlos"][s], atlos), s
    assert np.all(ref.a["charge"][0] == 1.0)
    assert np.any(ref.a["charge"][1] < 1.0)


def test_stale_ghost_lines_occur():
    """The perturbed grid has DRIFTR lines that are outflow at NR and
    upwinded from the right at NR-1 (they read the previous inflow line's
    ghost), so the bit-for-bit sweeps above cover that quirk."""
    wl = W.make_workload("tiny_pert8")
    g = wl.grid
    ref = refrun.RefRam(g, wl.fields)
    o = pyoracle.Oracle(g, wl.fields)
    ref.a["vt"][...] = o.vt_vols(4.0)
    ref.set("modramtiming::dts", wl.dts)
    ref.a["f2"][1] = wl.f2[1]
    ref.a["fgeos"][1] = wl.fgeos[1]
    ref.subroutine("driftpara", 1)
    ref.subroutine("driftr", 1)
    cd = ref.view("modramdrift::cdriftr")
    assert ((cd[-1] >= 0) & (cd[-2] < 0)).any() and (cd[-1] < 0).any()
    ref.call("driftend")


@pytest.mark.parametrize("name", ["four_sp", "single_h"])
def test_arrays_grid_bit_for_bit(name):
    """The standard-grid construction of ramgpu/workload.py against the
    reference's ARRAYS (src/ModRamInit.f90:364-587) for every species:
    radial, MLT, energy and pitch-angle grids, the loss-cone index UPA,
    GREL/GRBND/V/VBND, FFACTOR, EPP, ERNH, CONF1/2, DL1, MDR, DPHI."""
    wl = W.make_workload(name)
    g = wl.grid
    ref = refrun.RefRam(g, wl.fields, check=True)
    out = ref.arrays()
    for k, v in out.items():
        mine = np.asarray(getattr(g, k), dtype=np.float64)
        assert mine.shape == np.shape(v), k
        assert np.array_equal(mine, np.asarray(v, dtype=np.float64)), k


def test_implicit_diffusion_bit_for_bit():
    """The oracle's implicit pitch-angle diffusion against the reference's
    WPADIF (electrons, src/ModRamWPI.f90:643-714) and FLCscatter (ions,
    src/ModRamLoss.f90:513-575)."""
    wl = W.make_workload("tiny_pert")
    g = wl.grid
    ref = refrun.RefRam(g, wl.fields, check=True)
    o = pyoracle.Oracle(g, wl.fields)
    for s, fn in ((0, "wpadif"), (1, "flcscatter"), (3, "flcscatter")):
        daa = W.pa_diffusion(g, wl.fields, seed=30 + s)
        f_ref = np.asfortranarray(wl.f2[s]).copy(order="F")
        f_or = f_ref.copy(order="F")
        getattr(ref, fn)(s, f_ref, daa, wl.dts)
        o.padif(f_or, daa, wl.dts)
        assert not np.array_equal(f_ref, wl.f2[s])
        assert np.array_equal(f_ref, f_or), (s, fn)


def test_sum_pressure_bit_for_bit():
    """pyoracle.sum_pressure against the reference's ram_sum_pressure
    (src/ModRamFunctions.f90:272-297)."""
    wl = W.make_workload("tiny")
    g = wl.grid
    ref = refrun.RefRam(g, wl.fields)
    rng = np.random.Generator(np.random.PCG64(5))
    pe = [np.asfortranarray(rng.random((g.nr, g.nt))) for _ in g.species]
    pa = [np.asfortranarray(rng.random((g.nr, g.nt))) for _ in g.species]
    pall, ppar = ref.sum_pressure(pe, pa)
    idx = list(range(len(g.species)))
    epall, eppar = pyoracle.sum_pressure(dict(enumerate(pe)), dict(enumerate(pa)), idx)
    assert np.array_equal(pall, epall) and np.array_equal(ppar, eppar)


def test_interpolated_potential_branch():
    """ram_run's non-VOLS branch, VT = VTOL + (VTN-VTOL)*(T-TOLV)/DtEfi
    (src/ModRamRun.f90:46-52): the reference's VT equals the same
    expression in NumPy, and the oracle given that VT equals the reference
    bit for bit."""
    wl = W.make_workload("tiny_pert8")
    g = wl.grid
    ref = refrun.RefRam(g, wl.fields, check=True)
    o = pyoracle.Oracle(g, wl.fields)
    rng = np.random.Generator(np.random.PCG64(3))
    vtol = np.asfortranarray(o.vt_vols(2.0) * (1 + 0.1 * rng.standard_normal((g.nr + 1, g.nt))))
    vtn = np.asfortranarray(o.vt_vols(5.0) * (1 + 0.1 * rng.standard_normal((g.nr + 1, g.nt))))
    f_ref = [np.asfortranarray(a).copy(order="F") for a in wl.f2]
    f_or = [np.asfortranarray(a).copy(order="F") for a in wl.f2]
    r = ref.ram_run(f_ref, wl.fgeos, wl.dts, 3.0, potential=(vtol, vtn, 450.0, 300.0, 300.0))
    assert np.array_equal(r["vt"], vtol + (vtn - vtol) * (450.0 - 300.0) / 300.0)
    out = o.ram_run(f_or, wl.fgeos, wl.dts, vt=r["vt"], want_flux=True)
    for s in range(len(g.species)):
        assert np.array_equal(f_ref[s], f_or[s]), s
        assert np.array_equal(r["ppert"][s], out["ppert"][s]), s
    assert r["dts_next"] == out["dts_next"]


def test_species_threads_bit_for_bit():
    """The reference's !$OMP PARALLEL DO over species (thread-local
    THREADPRIVATE arrays in the translation): four threads give the
    single-thread results bit for bit."""
    wl = W.make_workload("tiny_pert8")
    g = wl.grid
    outs = []
    for threads in (1, 4):
        ref = refrun.RefRam(g, wl.fields, threads=threads)
        f = [np.asfortranarray(a).copy(order="F") for a in wl.f2]
        r = [ref.ram_run(f, wl.fgeos, wl.dts, kp) for kp in (2.0, 5.0)]
        outs.append((f, r))
    (f1, r1), (f4, r4) = outs
    for s in range(len(g.species)):
        assert np.array_equal(f1[s], f4[s]), s
        assert np.array_equal(r1[1]["ppert"][s], r4[1]["ppert"][s]), s
        assert r1[1]["losses"][s] == r4[1]["losses"][s], s
    assert r1[1]["dts_next"] == r4[1]["dts_next"]


EDGE_CALLS = ((1.0, 5.0), (9.0, 200.0), (5.0, 5.0))  # (Kp, DTs)


def test_edge_states_bit_for_bit():
    """States built to reach every corner (workload.edge_state: zero blocks,
    1e-30 cells, spikes, a flat line) along Kp 1, then Kp 9 with DTs = 200 s
    (Courant numbers above 1: the CFL limit is below DTs and updates come
    out negative and are clipped), then Kp 5: the oracle equals the
    reference bit for bit, and clip events did occur."""
    wl = W.make_workload("tiny_pert8")
    g = wl.grid
    ref = refrun.RefRam(g, wl.fields, check=True)
    o = pyoracle.Oracle(g, wl.fields)
    f_ref = W.edge_state(wl.f2)
    f_or = [a.copy(order="F") for a in f_ref]
    # the corners are reached: every limiter case (0 upwind, 1 beta*R, 2 one,
    # 3 R, 4 beta) and clipped updates (bit 3) in the forward sweeps of the
    # Kp 9 / 200 s call, recorded by the oracle on a copy of the state
    rec_cases, clips = set(), 0
    vt = o.vt_vols(9.0)
    for s in range(len(g.species)):
        f = f_ref[s].copy(order="F")
        for which in ("R", "P", "E", "MU"):
            _, _, _, rec, _ = o.sweep_rec(which, s, f, vt, 200.0, fgeos=wl.fgeos[s])
            rec_cases |= set(np.unique(rec & 7).tolist())
            clips += int(np.count_nonzero(rec & 8))
    assert rec_cases >= {0, 1, 2, 3, 4} and clips > 0, (rec_cases, clips)
    for kp, dts in EDGE_CALLS:
        r = ref.ram_run(f_ref, wl.fgeos, dts, kp)
        out = o.ram_run(f_or, wl.fgeos, dts, kp=kp, want_flux=True)
        for s in range(len(g.species)):
            assert np.array_equal(f_ref[s], f_or[s]), (kp, s)
            assert np.array_equal(r["ppert"][s], out["ppert"][s]), (kp, s)
            assert np.array_equal(r["flux"][s], out["flux"][s]), (kp, s)
        assert r["dts_next"] == out["dts_next"]
        if dts > 100.0:
            assert min(min(v) for v in r["dtdrift"].values()) < dts
