"""GPU parity: every operator and the full ram_run against the CPU oracle.

Bar (from the specification of this path): FP64 results within 1e-12
relative max-norm per step, i.e. max|gpu - ref| / max|ref| <= 1e-12 for F2
of every species after one step started from the same state.  Moments,
FLUX and DtsNext use the same tolerance.
"""
import numpy as np
import pytest

from ramgpu import abi, workload as W
import pyoracle

pytestmark = pytest.mark.gpu
TOL = 1e-12


def rel(a, b):
    den = np.max(np.abs(b))
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / (den if den > 0 else 1.0))


@pytest.fixture(scope="module")
def single():
    return W.make_workload("single_h")


@pytest.fixture(scope="module")
def tiny():
    return W.make_workload("tiny")


@pytest.fixture(scope="module")
def four():
    return W.make_workload("four_sp")


def _setup(wl, kp, members=1, flags=0):
    g = wl.grid
    gpu = abi.RamGpu(g, wl.fields, n_members=members, flags=flags)
    for m in range(members):
        for s in range(len(g.species)):
            gpu.upload_f2(m, s, wl.f2[s])
            gpu.set_boundary(m, s, wl.fgeos[s])
        gpu.set_kp(m, kp)
    return gpu


SWEEPS = [("R", abi.OP_DRIFTR, 0), ("P", abi.OP_DRIFTP, 1), ("E", abi.OP_DRIFTE, 2),
          ("MU", abi.OP_DRIFTMU, 3)]


@pytest.mark.parametrize("name,op,slot", SWEEPS)
@pytest.mark.parametrize("kp", [3.0, 6.5])
def test_single_sweep(single, name, op, slot, kp):
    wl = single
    o = pyoracle.Oracle(wl.grid, wl.fields)
    gpu = _setup(wl, kp)
    vt = o.vt_vols(kp)
    ref = np.asfortranarray(wl.f2[0]).copy(order="F")
    dt_ref = o.sweep(name, 0, ref, vt, wl.dts, fgeos=wl.fgeos[0])
    gpu.apply_op(wl.dts, op, cfl=True)
    out = gpu.download_f2(0, 0)
    assert rel(out, ref) <= TOL, f"{name}: {rel(out, ref)}"
    dt_gpu = gpu.cfl(0, 0)[slot]
    assert abs(dt_gpu - dt_ref) <= 1e-12 * dt_ref, (dt_gpu, dt_ref)


@pytest.mark.parametrize("name,op,slot", SWEEPS)
@pytest.mark.parametrize("kp,dts", [(3.0, 5.0), (8.0, 1.0)])
def test_single_sweep_four_species(four, name, op, slot, kp, dts):
    """Each sweep for e-, H+, He+, O+ (charge sign and mass enter the
    gradient-curvature and energy terms)."""
    wl = four
    o = pyoracle.Oracle(wl.grid, wl.fields)
    gpu = _setup(wl, kp)
    vt = o.vt_vols(kp)
    gpu.apply_op(dts, op, cfl=True)
    for s in range(len(wl.grid.species)):
        ref = np.asfortranarray(wl.f2[s]).copy(order="F")
        dt_ref = o.sweep(name, s, ref, vt, dts, fgeos=wl.fgeos[s])
        e = rel(gpu.download_f2(0, s), ref)
        assert e <= TOL, (name, s, e)
        dt_gpu = gpu.cfl(0, s)[slot]
        assert abs(dt_gpu - dt_ref) <= 1e-12 * dt_ref, (name, s, dt_gpu, dt_ref)


@pytest.mark.parametrize("op,name", [(abi.OP_CHAREXCHANGE, "cex"), (abi.OP_ATMOL, "atmol")])
def test_losses_ops(tiny, op, name):
    wl = tiny
    g = wl.grid
    o = pyoracle.Oracle(g, wl.fields)
    gpu = _setup(wl, 3.0)
    gpu.apply_op(wl.dts, op)
    for s in range(len(g.species)):
        ref = np.asfortranarray(wl.f2[s]).copy(order="F")
        charge, atlos = o.cepara(s, wl.dts)
        if op == abi.OP_CHAREXCHANGE:
            o.lib.ro_charexchange(pyoracle.C.byref(o.rg), pyoracle._p(ref), pyoracle._p(charge))
        else:
            o.lib.ro_atmol(pyoracle.C.byref(o.rg), pyoracle._p(ref), pyoracle._p(atlos))
        assert rel(gpu.download_f2(0, s), ref) <= TOL, (name, s)


@pytest.mark.parametrize("order", [0, 1])
def test_half_step(tiny, order):
    wl = tiny
    g = wl.grid
    o = pyoracle.Oracle(g, wl.fields)
    gpu = _setup(wl, 4.0)
    vt = o.vt_vols(4.0)
    gpu.half_step(wl.dts, order)
    for s in range(len(g.species)):
        ref = np.asfortranarray(wl.f2[s]).copy(order="F")
        o.half_step(s, ref, vt, wl.fgeos[s], wl.dts, order)
        assert rel(gpu.download_f2(0, s), ref) <= TOL, (order, s)


def _compare_ram_run(wl, kp, steps=1, flags=0, dts=None, nthreads=1):
    g = wl.grid
    dts = wl.dts if dts is None else dts
    o = pyoracle.Oracle(g, wl.fields)
    gpu = _setup(wl, kp, flags=flags)
    ref = [np.asfortranarray(a).copy(order="F") for a in wl.f2]
    worst = 0.0
    for step in range(steps):
        # per-step parity: both start the step from the oracle's state
        for s in range(len(g.species)):
            gpu.upload_f2(0, s, ref[s])
        gpu.ram_run(dts)
        out = o.ram_run(ref, wl.fgeos, dts, kp=kp, want_flux=True, nthreads=nthreads)
        # the scheme is run inside its stability limit, as the reference's
        # driver ensures through DtsNext (src/ModRamScbRun.f90:49-61)
        assert dts <= out["dts_next"] / 0.8 + 1e-12
        for s in range(len(g.species)):
            e = rel(gpu.download_f2(0, s), ref[s])
            worst = max(worst, e)
            assert e <= TOL, (step, s, e)
            pe, pa = gpu.moments(0, s)
            assert rel(pe, out["ppert"][s]) <= TOL
            assert rel(pa, out["ppart"][s]) <= TOL
            assert rel(gpu.flux(0, s), out["flux"][s]) <= TOL
        dn = gpu.cfl(0, 0)[4]
        assert abs(dn - out["dts_next"]) <= 1e-12 * out["dts_next"], (dn, out["dts_next"])
    return worst


def test_ram_run_single_species(single):
    _compare_ram_run(single, 3.0, steps=3)


def test_ram_run_four_species_tiny(tiny):
    _compare_ram_run(tiny, 5.0, steps=3)


def test_ram_run_four_species_full(four):
    _compare_ram_run(four, 2.0, steps=2)


def test_ram_run_refined_grid():
    """The refined 40x49x70x144 grid (19.8 M cells per species, 632 MB of F2
    for the four species, larger than L2): one full ram_run step."""
    wl = W.make_workload("refined")
    pyoracle.set_inner_threads(4)
    try:
        _compare_ram_run(wl, 3.0, steps=1, nthreads=4)
    finally:
        pyoracle.set_inner_threads(1)


def test_strong_convection_inflow_mix(four):
    """Kp=8: strong E x B makes most outer-boundary lines inflow, exercising
    the ghost cells and the stale-ghost lines of DRIFTR.  DTs=1 s, the step
    the reference's driver takes for Kp>6 (src/ModRamScbRun.f90:57-59)."""
    _compare_ram_run(four, 8.0, steps=2, dts=1.0)


def test_no_nan_and_positive(tiny):
    gpu = _setup(tiny, 3.0)
    for _ in range(5):
        gpu.ram_run(tiny.dts)
    for s in range(len(tiny.grid.species)):
        f = gpu.download_f2(0, s)
        assert np.isfinite(f).all()
        assert (f >= 0).all()


def test_ram_run_matches_golden_fixture():
    """The GPU step against the committed fixture (tests/golden), with no
    CPU run: per-species sums, 256 sampled cells, moments, FLUX, DtsNext."""
    import json
    from conftest import ROOT
    gd = json.loads((ROOT / "tests" / "golden" / "ram_run_tiny.json").read_text())
    wl = W.make_workload(gd["workload"])
    gpu = _setup(wl, gd["kp"])
    try:
        gpu.ram_run(gd["dts"])
        assert abs(gpu.cfl(0, 0)[4] - gd["dts_next"]) <= 1e-12 * gd["dts_next"]
        for s, sd in enumerate(gd["species"]):
            f = gpu.download_f2(0, s)
            assert abs(np.sum(f) - sd["sum"]) <= 1e-12 * abs(sd["sum"])
            scale = max(abs(v) for _, v in sd["cells"])
            for c, v in sd["cells"]:
                assert abs(f[tuple(c)] - v) <= TOL * scale
            pe, pa = gpu.moments(0, s)
            for arr, key in ((pe, "ppert"), (pa, "ppart")):
                sc = max(abs(v) for _, v in sd[key])
                for c, v in sd[key]:
                    assert abs(arr[tuple(c)] - v) <= TOL * sc
            fl = gpu.flux(0, s)
            sc = max(abs(v) for _, v in sd["flux"])
            for c, v in sd["flux"]:
                assert abs(fl[tuple(c)] - v) <= TOL * sc
    finally:
        gpu.close()
