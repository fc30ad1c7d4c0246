"""GPU: non-dipole fields, closed-face conservation, ensembles, SUMRC
bookkeeping and API error paths."""
import dataclasses

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
def pert():
    return W.make_workload("tiny_pert")


@pytest.fixture(scope="module")
def tiny():
    return W.make_workload("tiny")


def _gpu(wl, kp, members=1, flags=0, grid=None):
    g = grid or wl.grid
    gpu = abi.RamGpu(g, wl.fields, n_members=members, flags=flags)
    for m in range(members):
        for s in range(len(g.species)):
            gpu.upload_f2(m, s, wl.f2[s])
            gpu.set_boundary(m, s, wl.fgeos[s])
        gpu.set_kp(m, kp)
    return gpu


@pytest.mark.parametrize("op,name", [(abi.OP_DRIFTR, "R"), (abi.OP_DRIFTP, "P"),
                                     (abi.OP_DRIFTE, "E"), (abi.OP_DRIFTMU, "MU")])
@pytest.mark.parametrize("kp", [2.0, 4.0])
def test_sweeps_nondipole(pert, op, name, kp):
    """Every zero-in-dipole term, the stale-ghost lines and magnetopause cells."""
    wl = pert
    o = pyoracle.Oracle(wl.grid, wl.fields)
    gpu = _gpu(wl, kp)
    gpu.apply_op(wl.dts, op, cfl=True)
    vt = o.vt_vols(kp)
    for s in range(len(wl.grid.species)):
        ref = np.asfortranarray(wl.f2[s]).copy(order="F")
        dt = o.sweep(name, s, ref, vt, wl.dts, fgeos=wl.fgeos[s])
        assert rel(gpu.download_f2(0, s), ref) <= TOL, (name, s)
        slot = {"R": 0, "P": 1, "E": 2, "MU": 3}[name]
        assert abs(gpu.cfl(0, s)[slot] - dt) <= 1e-12 * dt


def test_ram_run_nondipole(pert):
    wl = pert
    g = wl.grid
    o = pyoracle.Oracle(g, wl.fields)
    gpu = _gpu(wl, 3.0)
    ref = [np.asfortranarray(a).copy(order="F") for a in wl.f2]
    for step in range(3):
        for s in range(len(g.species)):
            gpu.upload_f2(0, s, ref[s])
        gpu.ram_run(wl.dts)
        out = o.ram_run(ref, wl.fgeos, wl.dts, kp=3.0, want_flux=True)
        for s in range(len(g.species)):
            got = gpu.download_f2(0, s)
            assert rel(got, ref[s]) <= TOL, (step, s)
            # magnetopause mask (src/ModRamRun.f90:197-201)
            out_ij = wl.fields.outside == 1
            assert np.all(got[out_ij] == 1e-31)
            pe, pa = gpu.moments(0, s)
            assert rel(pe, out["ppert"][s]) <= TOL and rel(pa, out["ppart"][s]) <= TOL
        assert abs(gpu.cfl(0, 0)[4] - out["dts_next"]) <= 1e-12 * out["dts_next"]


def content_q(g, f2):
    w = g.we[None, None, 1:, None] * g.wmu[None, None, None, 1:-1]
    return float(np.sum(f2[1:, :-1, 1:, 1:-1] * w))


def test_closed_conservation(tiny):
    """Closed faces, no CEX/ATMOL/mask: sum F2*WE*WMU conserved to 1e-13."""
    wl = tiny
    g = dataclasses.replace(wl.grid, species=tuple(dataclasses.replace(s, cex_kind=W.CEX_NONE)
                                                   for s in wl.grid.species))
    gpu = _gpu(wl, 4.0, flags=abi.FLAG_CLOSED | abi.FLAG_NO_ATMOL, grid=g)
    q0 = [content_q(g, np.asfortranarray(a)) for a in wl.f2]
    for _ in range(20):
        gpu.ram_run(1.0)
    for s in range(len(g.species)):
        f = gpu.download_f2(0, s)
        assert abs(content_q(g, f) - q0[s]) <= 1e-13 * q0[s], s
        assert f.min() >= 0  # no clip events: the content is conserved exactly


def test_ensemble_equals_solo(tiny):
    """Batched members with uneven species sets, Kp and lengths advance
    bitwise like solo runs; retired members stop."""
    wl = tiny
    ns = len(wl.grid.species)
    plans = [([0, 1, 2, 3], 2.0, 3), ([1, 3], 5.0, 2), ([0], 3.5, 1), ([2, 1], 6.0, 3)]
    ens = _gpu(wl, 1.0, members=len(plans))
    for m, (sp, kp, _) in enumerate(plans):
        ens.set_member_species(m, sp)
        ens.set_kp(m, kp)
    for step in range(3):
        for m, (_, _, n) in enumerate(plans):
            ens.set_member_active(m, step < n)
        ens.ram_run(wl.dts)
    for m, (sp, kp, n) in enumerate(plans):
        solo = _gpu(wl, kp)
        solo.set_member_species(0, sp)
        for _ in range(n):
            solo.ram_run(wl.dts)
        for s in range(ns):
            a, b = ens.download_f2(m, s), solo.download_f2(0, s)
            assert np.array_equal(a, b), (m, s)
            if s not in sp:
                assert np.array_equal(a, np.asfortranarray(wl.f2[s]))
        solo.close()


def test_losses_bookkeeping(tiny):
    wl = tiny
    g = wl.grid
    o = pyoracle.Oracle(g, wl.fields)
    gpu = _gpu(wl, 3.0, flags=abi.FLAG_LOSSES)
    gpu.reset_losses()
    ref = [np.asfortranarray(a).copy(order="F") for a in wl.f2]
    losses = {s: (o.sumrc(ref[s]), 0.0, 0.0, 0.0) for s in range(len(g.species))}
    for _ in range(2):
        gpu.ram_run(wl.dts)
        out = o.ram_run(ref, wl.fgeos, wl.dts, kp=3.0, losses=losses)
        losses = out["losses"]
    for s in range(len(g.species)):
        got = gpu.losses(0, s)
        exp = losses[s]
        assert abs(got[0] - exp[0]) <= 1e-12 * exp[0], (s, got, exp)
        for k in (1, 2, 3):  # differences of nearly equal sums: compare to SETRC
            assert abs(got[k] - exp[k]) <= 1e-12 * exp[0], (s, k, got, exp)
        assert rel(gpu.download_f2(0, s), ref[s]) <= TOL


def test_api_errors(tiny):
    wl = tiny
    g = wl.grid
    lib = abi.load_library()
    cfg = abi.Config(g.nr, g.nt, g.ne, g.npa, len(g.species), 1, 1.5, 0.8, 0.1, 0)
    import ctypes
    h = ctypes.c_void_p()
    assert lib.ramgpu_create(ctypes.byref(cfg), ctypes.byref(h)) == 0
    # step before grid/fields: state error, not a crash
    assert lib.ramgpu_ram_run(h, 5.0) == -3
    buf = ctypes.create_string_buffer(256)
    lib.ramgpu_last_error(h, buf, 256)
    assert b"set_grid" in buf.value
    assert lib.ramgpu_set_species(h, 99, 1, 1) == -1
    assert lib.ramgpu_set_species(h, 0, 0, 1) == -1
    assert lib.ramgpu_set_kp(h, 5, 3.0) == -1
    lib.ramgpu_destroy(h)
    gpu = _gpu(wl, 3.0)
    with pytest.raises(abi.RamGpuError):
        gpu.ram_run(-1.0)
    with pytest.raises(abi.RamGpuError):
        gpu.download_f2(3, 0)
    with pytest.raises(abi.RamGpuError):
        gpu.set_member_species(0, [1, 1])
    gpu.ram_run(wl.dts)  # context still usable after the errors
    assert np.isfinite(gpu.download_f2(0, 1)).all()


def test_graph_replay_matches_direct(tiny):
    """ram_run from a captured CUDA graph equals direct launches bitwise, with
    Kp changing between steps (inputs are read when the graph runs)."""
    wl = tiny
    a = _gpu(wl, 2.0)
    b = _gpu(wl, 2.0)
    b.set_graph(True)
    for step, kp in enumerate([2.0, 3.0, 4.5, 4.5, 6.0]):
        a.set_kp(0, kp)
        b.set_kp(0, kp)
        a.ram_run(wl.dts)
        b.ram_run(wl.dts)
    for s in range(len(wl.grid.species)):
        assert np.array_equal(a.download_f2(0, s), b.download_f2(0, s)), s
        pa, pb = a.moments(0, s), b.moments(0, s)
        assert np.array_equal(pa[0], pb[0]) and np.array_equal(pa[1], pb[1])


@pytest.mark.parametrize("shape", [(32, 0), (256, 0), (64, 1), (128, 1)])
def test_launch_shapes_bitwise(tiny, shape):
    threads, persistent = shape
    wl = tiny
    ref = _gpu(wl, 3.0)
    alt = _gpu(wl, 3.0)
    for w in range(4):
        alt.set_launch_shape(w, threads, 2 * 152 if persistent else 0)
    for _ in range(2):
        ref.ram_run(wl.dts)
        alt.ram_run(wl.dts)
    for s in range(len(wl.grid.species)):
        assert np.array_equal(ref.download_f2(0, s), alt.download_f2(0, s))
    assert np.array_equal(ref.cfl(0, 1), alt.cfl(0, 1))


def test_autotune_restores_state_and_keeps_results(tiny):
    wl = tiny
    ref = _gpu(wl, 3.0)
    tun = _gpu(wl, 3.0)
    shapes, ms = tun.autotune(wl.dts, reps=2)
    assert all(t in (32, 64, 128, 256) for t, _ in shapes) and np.all(ms > 0)
    for s in range(len(wl.grid.species)):
        assert np.array_equal(tun.download_f2(0, s), np.asfortranarray(wl.f2[s]))
    ref.ram_run(wl.dts)
    tun.ram_run(wl.dts)
    for s in range(len(wl.grid.species)):
        assert np.array_equal(ref.download_f2(0, s), tun.download_f2(0, s))


@pytest.mark.parametrize("name", ["tiny_pert", "four_sp"])
def test_coefficient_store_is_bitwise_neutral(name):
    """Reading the forward sweeps' stored face coefficients in the reverse
    half gives the same bits as recomputing them (also with graph replay)."""
    wl = W.make_workload(name)
    outs = []
    for store, graph in ((0, False), (15, False), (4, True), (15, True)):
        gpu = _gpu(wl, 4.0)
        gpu.set_coef_store(store)
        gpu.set_graph(graph)
        for c in range(3):
            gpu.set_kp(-1, 3.0 + c)
            gpu.ram_run(wl.dts)
        outs.append([gpu.download_f2(0, s) for s in range(len(wl.grid.species))]
                    + [gpu.cfl(0, s) for s in range(len(wl.grid.species))])
        gpu.close()
    for o in outs[1:]:
        for a, b in zip(o, outs[0]):
            assert np.array_equal(a, b)


@pytest.mark.parametrize("name", ["tiny_pert", "four_sp"])
def test_mu_lanes_equal(name):
    """DRIFTMU with one lane per line and with 2 or 4 lanes per line (each
    lane but the first recomputing the flux at its split) gives the same F2,
    CFL and moments,
    in the plain step (graph and direct) and in the adjoint's recorded and
    transposed passes."""
    wl = W.make_workload(name)
    ns = len(wl.grid.species)
    outs = []
    for lanes, graph in ((1, False), (2, False), (2, True), (4, False), (4, True)):
        gpu = _gpu(wl, 4.0)
        gpu.set_mu_lanes(lanes)
        gpu.set_graph(graph)
        for c in range(3):
            gpu.set_kp(-1, 3.0 + c)
            gpu.ram_run(wl.dts)
        gpu.apply_op(wl.dts, abi.OP_DRIFTMU, cfl=True)
        outs.append([gpu.download_f2(0, s) for s in range(ns)] + [gpu.cfl(0, s) for s in range(ns)]
                    + [np.concatenate(gpu.moments(0, s)) for s in range(ns)])
        gpu.close()
    for o in outs[1:]:
        for a, b in zip(o, outs[0]):
            assert np.array_equal(a, b)
    if name != "tiny_pert":
        return
    grads = []
    kp = np.array([[3.0], [4.0], [5.0]])
    obs = [{"member": 0, "s": s, "call": c, "k": 10 + 3 * s, "l": 1 + c, "lshell": 3.0 + 0.5 * s,
            "mlt": 6.0 * c, "log_obs": 0.0} for s in range(ns) for c in range(3)]
    for lanes in (1, 2, 4):
        gpu = _gpu(wl, 4.0)
        gpu.set_mu_lanes(lanes)
        J = gpu.adj_forward(3, wl.dts, kp, 1, obs)
        gf, gb = gpu.adj_backward()
        grads.append((J, gf, gb))
        gpu.close()
    for k in (1, 2):
        assert np.array_equal(grads[0][0], grads[k][0])
        assert np.max(np.abs(grads[0][1] - grads[k][1])) <= 1e-13 * np.max(np.abs(grads[0][1]))
        assert np.max(np.abs(grads[0][2] - grads[k][2])) <= 1e-13 * max(np.max(np.abs(grads[0][2])), 1e-300)
    with pytest.raises(abi.RamGpuError):
        abi.RamGpu(wl.grid, wl.fields).set_mu_lanes(3)


def test_moments_with_non_separable_ffactor(pert):
    """FFACTOR that is not of the separable ARRAYS form takes the general
    moment sums; both forms match the oracle (the separable one is every
    other test's grid)."""
    wl = pert
    rng = np.random.Generator(np.random.PCG64(77))
    g = dataclasses.replace(wl.grid, ffactor=wl.grid.ffactor * rng.lognormal(0.0, 0.2, size=wl.grid.ffactor.shape))
    o = pyoracle.Oracle(g, wl.fields)
    gpu = _gpu(wl, 3.0, grid=g)
    ref = [np.asfortranarray(a).copy(order="F") for a in wl.f2]
    try:
        for step in range(2):
            gpu.ram_run(wl.dts)
            out = o.ram_run(ref, wl.fgeos, wl.dts, kp=3.0)
            for s in range(len(g.species)):
                assert rel(gpu.download_f2(0, s), ref[s]) <= TOL
                pe, pa = gpu.moments(0, s)
                assert rel(pe, out["ppert"][s]) <= TOL and rel(pa, out["ppart"][s]) <= TOL, (step, s)
    finally:
        gpu.close()
