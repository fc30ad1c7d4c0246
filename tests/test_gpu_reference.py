"""GPU: the CUDA ram_run against the reference's own routines.

Two sources, neither a restatement of this project:

* the committed fixtures of tests/golden (made by tests/golden/make_golden.py
  from the reference's ram_run, src/ModRamRun.f90:16-225, translated by
  oracle/f90c.py): the GPU advances alone along a three-call Kp ramp on the
  perturbed 8x9x35x72 grid and meets every call's sums, sampled cells,
  moments, FLUX and DtsNext;
* the translated reference itself, built on this machine from
  oracle/_ref/ramref.c: whole-array comparisons per call (each call started
  from the reference's state) on the test grids, on the standard
  20x25x35x72 four-species grid and on the refined 40x49x70x144 grid.

Bar: 1e-12 relative max-norm per call (FP64), as the rest of the parity suite.
"""
import json

import numpy as np
import pytest

from ramgpu import abi, workload as W
import refrun

pytestmark = pytest.mark.gpu
TOL = 1e-12


def rel(a, b):
    den = np.max(np.abs(b))
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / (den if den > 0 else 1.0))


def _gpu(wl, kp):
    g = wl.grid
    gpu = abi.RamGpu(g, wl.fields)
    for s in range(len(g.species)):
        gpu.upload_f2(0, s, wl.f2[s])
        gpu.set_boundary(0, s, wl.fgeos[s])
    gpu.set_kp(0, kp)
    return gpu


def _check_summary(gpu, sd_all, dts_next):
    assert abs(gpu.cfl(0, 0)[4] - dts_next) <= TOL * dts_next
    for s, sd in enumerate(sd_all):
        f = gpu.download_f2(0, s)
        assert abs(np.sum(f) - sd["sum"]) <= 1e-12 * abs(sd["sum"]), s
        scale = max(abs(v) for _, v in sd["cells"])
        for c, v in sd["cells"]:
            assert abs(f[tuple(c)] - v) <= TOL * scale, (s, c)
        pe, pa = gpu.moments(0, s)
        for arr, key in ((pe, "ppert"), (pa, "ppart")):
            sc = max(abs(v) for _, v in sd[key])
            for c, v in sd[key]:
                assert abs(arr[tuple(c)] - v) <= TOL * sc, (s, key, c)
        fl = gpu.flux(0, s)
        sc = max(abs(v) for _, v in sd["flux"])
        for c, v in sd["flux"]:
            assert abs(fl[tuple(c)] - v) <= TOL * sc, (s, c)


def test_follows_reference_ramp_fixture():
    from conftest import ROOT
    gd = json.loads((ROOT / "tests" / "golden" / "ram_run_ramp.json").read_text())
    wl = W.make_workload(gd["workload"])
    gpu = _gpu(wl, gd["calls"][0]["kp"])
    try:
        for call in gd["calls"]:
            gpu.set_kp(0, call["kp"])
            gpu.ram_run(gd["dts"])
            _check_summary(gpu, call["species"], call["dts_next"])
    finally:
        gpu.close()


@pytest.fixture(scope="module")
def have_ref():
    if refrun.build() is None:
        pytest.skip("translated reference not present (oracle/_ref/ramref.c)")
    return True


@pytest.mark.parametrize("name,kps", [("tiny_pert8", (1.0, 3.5, 6.0)), ("four_sp", (3.0,)), ("refined", (4.0,))])
def test_whole_arrays_against_translated_reference(have_ref, name, kps):
    """Each call from the reference's state: F2, PPERT/PPART, FLUX of every
    species and DtsNext within 1e-12."""
    wl = W.make_workload(name)
    g = wl.grid
    ref = refrun.RefRam(g, wl.fields, threads=len(g.species))  # its species loop, bitwise as one thread
    f_ref = [np.asfortranarray(a).copy(order="F") for a in wl.f2]
    gpu = _gpu(wl, kps[0])
    try:
        for kp in kps:
            for s in range(len(g.species)):
                gpu.upload_f2(0, s, f_ref[s])
            gpu.set_kp(0, kp)
            gpu.ram_run(wl.dts)
            r = ref.ram_run(f_ref, wl.fgeos, wl.dts, kp)
            assert abs(gpu.cfl(0, 0)[4] - r["dts_next"]) <= TOL * r["dts_next"]
            for s in range(len(g.species)):
                assert rel(gpu.download_f2(0, s), f_ref[s]) <= TOL, (kp, s)
                pe, pa = gpu.moments(0, s)
                assert rel(pe, r["ppert"][s]) <= TOL and rel(pa, r["ppart"][s]) <= TOL, (kp, s)
                assert rel(gpu.flux(0, s), r["flux"][s]) <= TOL, (kp, s)
    finally:
        gpu.close()


def test_implicit_diffusion_against_translated_reference(have_ref):
    """The CUDA WPADIF / FLCscatter (one application) against the reference's
    own WPADIF (electrons) and FLCscatter (ions)."""
    wl = W.make_workload("tiny_pert")
    g = wl.grid
    ref = refrun.RefRam(g, wl.fields)
    d = {0: W.pa_diffusion(g, wl.fields, seed=30), 2: W.pa_diffusion(g, wl.fields, seed=32)}
    gpu = _gpu(wl, 3.0)
    try:
        for s, a in d.items():
            gpu.set_pa_diffusion(s, a)
        gpu.apply_op(wl.dts, abi.OP_PADIF)
        for s, a in d.items():
            f = np.asfortranarray(wl.f2[s]).copy(order="F")
            (ref.wpadif if s == 0 else ref.flcscatter)(s, f, a, wl.dts)
            assert rel(gpu.download_f2(0, s), f) <= TOL, s
    finally:
        gpu.close()


def test_sum_pressure_against_translated_reference(have_ref):
    """The CUDA ram_sum_pressure hand-off after one ram_run, against the
    reference's ram_sum_pressure on the reference's own moments."""
    wl = W.make_workload("tiny_pert")
    g = wl.grid
    ref = refrun.RefRam(g, wl.fields)
    f_ref = [np.asfortranarray(a).copy(order="F") for a in wl.f2]
    gpu = _gpu(wl, 3.0)
    try:
        gpu.ram_run(wl.dts)
        r = ref.ram_run(f_ref, wl.fgeos, wl.dts, 3.0)
        pall, ppar = ref.sum_pressure([r["ppert"][s] for s in range(len(g.species))],
                                      [r["ppart"][s] for s in range(len(g.species))])
        gpall, gppar = gpu.sum_pressure(0)
        assert rel(gpall, pall) <= TOL and rel(gppar, ppar) <= TOL
    finally:
        gpu.close()


def test_interpolated_potential_against_translated_reference(have_ref):
    """ramgpu_set_potential (the non-VOLS branch) against the reference's
    ram_run with electric /= 'VOLS': VT interpolated between two potential
    tables (src/ModRamRun.f90:46-52), two calls."""
    wl = W.make_workload("tiny_pert8")
    g = wl.grid
    ref = refrun.RefRam(g, wl.fields)
    rng = np.random.Generator(np.random.PCG64(3))
    base = W.vols_vt(g, 3.0)
    vtol = np.asfortranarray(base * (1 + 0.1 * rng.standard_normal(base.shape)))
    vtn = np.asfortranarray(base * (1.5 + 0.1 * rng.standard_normal(base.shape)))
    f_ref = [np.asfortranarray(a).copy(order="F") for a in wl.f2]
    gpu = _gpu(wl, 3.0)
    try:
        for t in (350.0, 520.0):
            # each call from the reference's state; VT as the reference forms it
            for s in range(len(g.species)):
                gpu.upload_f2(0, s, f_ref[s])
            gpu.set_potential(0, np.asfortranarray(vtol + (vtn - vtol) * (t - 300.0) / 300.0))
            gpu.ram_run(wl.dts)
            r = ref.ram_run(f_ref, wl.fgeos, wl.dts, 3.0, potential=(vtol, vtn, t, 300.0, 300.0))
            assert abs(gpu.cfl(0, 0)[4] - r["dts_next"]) <= TOL * r["dts_next"]
            for s in range(len(g.species)):
                assert rel(gpu.download_f2(0, s), f_ref[s]) <= TOL, (t, s)
                pe, pa = gpu.moments(0, s)
                assert rel(pe, r["ppert"][s]) <= TOL and rel(pa, r["ppart"][s]) <= TOL, (t, s)
    finally:
        gpu.close()


def test_edge_states_against_translated_reference(have_ref):
    """States built to reach every corner (workload.edge_state: zero blocks,
    1e-30 cells, spikes, a flat line), Kp 1, then Kp 9 with DTs = 200 s
    (Courant numbers above 1, clipped updates), then Kp 5; each call from
    the reference's state, within 1e-12."""
    wl = W.make_workload("tiny_pert8")
    g = wl.grid
    ref = refrun.RefRam(g, wl.fields)
    f_ref = W.edge_state(wl.f2)
    gpu = _gpu(wl, 1.0)
    try:
        gpu.set_check(True)
        clips = 0
        for kp, dts in ((1.0, 5.0), (9.0, 200.0), (5.0, 5.0)):
            for s in range(len(g.species)):
                gpu.upload_f2(0, s, f_ref[s])
            gpu.set_kp(0, kp)
            gpu.ram_run(dts)
            clips += gpu.last_status()["clips"]
            r = ref.ram_run(f_ref, wl.fgeos, dts, kp)
            assert abs(gpu.cfl(0, 0)[4] - r["dts_next"]) <= TOL * r["dts_next"]
            for s in range(len(g.species)):
                assert rel(gpu.download_f2(0, s), f_ref[s]) <= TOL, (kp, s)
                pe, pa = gpu.moments(0, s)
                assert rel(pe, r["ppert"][s]) <= TOL and rel(pa, r["ppart"][s]) <= TOL, (kp, s)
                assert rel(gpu.flux(0, s), r["flux"][s]) <= TOL, (kp, s)
        assert clips > 0
    finally:
        gpu.close()
