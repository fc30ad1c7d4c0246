"""GPU: the bounds-checked build (libramgpu_bounds.so, RAMGPU_BOUNDS_CHECK).

Its sweep and transposed-sweep kernels test every streamed line's index
ranges (work item, slot, first and last cell, table rows, coefficient-store
item) before touching it and count failures in the context's log.  On the
small test grids it must agree with the oracle per step within the parity
bar, give the release library's bits for the whole step, the adjoint and
the reference-layout call, and log no failure.
"""
import numpy as np
import pytest

from ramgpu import abi, build as B, workload as W
import pyoracle

pytestmark = pytest.mark.gpu
TOL = 1e-12


def rel(a, b):
    den = np.max(np.abs(b))
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / (den if den > 0 else 1.0))


@pytest.fixture(scope="module")
def blib():
    if not B.LIB_BOUNDS_PATH.exists():
        pytest.fail(f"{B.LIB_BOUNDS_PATH} is not built: run __graft_entry__.build()")
    return abi.load_library(B.LIB_BOUNDS_PATH)


def _model(wl, lib, members=1, species=None):
    g = wl.grid
    gpu = abi.RamGpu(g, wl.fields, n_members=members, lib=lib)
    for m in range(members):
        for s in range(len(g.species)):
            gpu.upload_f2(m, s, np.asarray(wl.f2[s]) * (1.0 + 0.25 * m))
            gpu.set_boundary(m, s, wl.fgeos[s])
        gpu.set_kp(m, 3.0 + m)
        if species is not None:
            gpu.set_member_species(m, species[m])
    return gpu


def _clean(gpu):
    rep = gpu.bounds_report()
    assert rep["checked"] == 1
    assert rep["failures"] == 0, rep


def test_only_the_checked_build_logs(blib):
    wl = W.make_workload("tiny")
    a = abi.RamGpu(wl.grid, wl.fields, lib=blib)
    b = abi.RamGpu(wl.grid, wl.fields)
    try:
        assert a.bounds_report() == {"checked": 1, "failures": 0, "check": 0, "value": 0}
        assert b.bounds_report()["checked"] == 0
    finally:
        a.close()
        b.close()


@pytest.mark.parametrize("name", ["tiny", "tiny_pert", "tiny_pert8"])
def test_ram_run_against_the_oracle(blib, name):
    """Per-step parity of the checked kernels with the oracle (each call
    starts from the oracle's state), three calls, no failed test."""
    wl = W.make_workload(name)
    g = wl.grid
    o = pyoracle.Oracle(g, wl.fields)
    gpu = _model(wl, blib)
    ref = [np.asfortranarray(a).copy(order="F") for a in wl.f2]
    try:
        for c in range(3):
            kp = 2.0 + 1.5 * c
            gpu.set_kp(0, kp)
            for s in range(len(g.species)):
                gpu.upload_f2(0, s, ref[s])
            gpu.ram_run(wl.dts)
            out = o.ram_run(ref, wl.fgeos, wl.dts, kp=kp, want_flux=True)
            for s in range(len(g.species)):
                assert rel(gpu.download_f2(0, s), ref[s]) <= TOL, (c, s)
                pe, pa = gpu.moments(0, s)
                assert rel(pe, out["ppert"][s]) <= TOL and rel(pa, out["ppart"][s]) <= TOL, (c, s)
        _clean(gpu)
    finally:
        gpu.close()


def _run_everything(wl, lib, persistent):
    """Uneven two-member ensemble: graph-replayed steps over item groups,
    both half steps, the reference-layout call and an adjoint window that
    recomputes segments on the second stream; returns every result."""
    g = wl.grid
    ns = len(g.species)
    species = [[0, 1, 2, 3], [3, 1]]
    gpu = _model(wl, lib, members=2, species=species)
    out = {}
    try:
        if persistent:
            for w in range(4):
                gpu.set_launch_shape(w, 64, 2 * 152)
        gpu.set_graph(True)
        gpu.set_step_groups(3)
        for c in range(3):
            gpu.set_kp(-1, 2.0 + c)
            gpu.ram_run(wl.dts)
        gpu.half_step(wl.dts, 0)
        gpu.half_step(wl.dts, 1)
        f2 = [np.asfortranarray(np.stack([gpu.download_f2(m, s) for s in range(ns)], axis=0)) for m in range(2)]
        pe = [np.zeros((ns, g.nr, g.nt), order="F") for _ in range(2)]
        pa = [np.zeros((ns, g.nr, g.nt), order="F") for _ in range(2)]
        gpu.ram_run_ref(wl.dts, f2, pe, pa)
        out["f2"] = [[gpu.download_f2(m, s) for s in species[m]] for m in range(2)]
        out["ref"] = (f2, pe, pa)
        kp = np.array([[2.0 + 0.5 * c, 3.0 + 0.25 * c] for c in range(4)])
        rng = np.random.Generator(np.random.PCG64(17))
        obs = []
        for t in range(12):
            m = t % 2
            obs.append({"member": m, "s": int(rng.choice(species[m])), "call": int(rng.integers(4)),
                        "k": int(rng.integers(8, 28)), "l": 1, "lshell": float(rng.uniform(2.6, 5.9)),
                        "mlt": float(rng.uniform(0.0, 24.0)), "log_obs": float(rng.normal(0.0, 1.0))})
        per_call = 4 * len(species[0] + species[1]) * g.ncell
        gpu.set_adj_record_budget(2 * per_call)  # two one-call segments kept, two recomputed
        out["J"] = gpu.adj_forward(4, wl.dts, kp, 1, obs)
        out["grad"] = gpu.adj_backward()
        rep = gpu.bounds_report()
    finally:
        gpu.close()
    return out, rep


@pytest.mark.parametrize("persistent", [False, True])
def test_whole_path_equals_release_bits(blib, persistent):
    wl = W.make_workload("tiny_pert8")
    chk, rep = _run_everything(wl, blib, persistent)
    rel_out, _ = _run_everything(wl, None, persistent)
    assert rep["checked"] == 1 and rep["failures"] == 0, rep
    for m in range(2):
        for a, b in zip(chk["f2"][m], rel_out["f2"][m]):
            assert np.array_equal(a, b)
        for a, b in zip(chk["ref"], rel_out["ref"]):
            assert np.array_equal(a[m], b[m])
    assert np.array_equal(chk["J"], rel_out["J"])
    # dJ/dF2 bit for bit; dJ/dFGEOS sums stale-ghost terms with atomics
    assert np.array_equal(chk["grad"][0], rel_out["grad"][0])
    gb, rb = chk["grad"][1], rel_out["grad"][1]
    assert np.max(np.abs(gb - rb)) <= 1e-13 * max(np.max(np.abs(rb)), 1e-300)
