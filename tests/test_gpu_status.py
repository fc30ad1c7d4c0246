"""GPU: the device status word (ramgpu_check, ramgpu_set_check).  The
reference stops when a moment is no longer finite (ANISCH,
src/ModRamRun.f90:410-413); the library reports the count of non-finite
F2 cells and moments, the first (member, species) holding one, and the
sweeps of the last call whose Courant number exceeded 1, against counts
taken with numpy on the downloaded state and against ramgpu_cfl."""
import numpy as np
import pytest

from ramgpu import abi, workload as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tiny():
    return W.make_workload("tiny_pert")


def _gpu(wl, members=1):
    g = wl.grid
    gpu = abi.RamGpu(g, wl.fields, n_members=members)
    for m in range(members):
        for s in range(len(g.species)):
            gpu.upload_f2(m, s, wl.f2[s])
            gpu.set_boundary(m, s, wl.fgeos[s])
        gpu.set_kp(m, 3.0)
    return gpu


def _cfl_over(gpu, wl, dts, members):
    """(item, sweep) pairs with DtDrift* below FracCFL*DTs (FracCFL*DTs is
    far below the DtDrift caps here, so that is a Courant number above 1)."""
    fr = gpu.fraccfl * dts
    n = 0
    for m in range(members):
        for s in gpu.member_species[m]:
            out = gpu.cfl(m, s)
            n += int(np.sum(np.asarray(out[:4]) < fr))
    return n


def test_healthy_state(tiny):
    gpu = _gpu(tiny)
    try:
        st = gpu.check()
        assert st == {"f2_nonfinite": 0, "moments_nonfinite": 0, "cfl_over": 0, "clips": 0,
                      "first_member": -1, "first_species": -1}
        gpu.ram_run(tiny.dts)
        st = gpu.check()
        assert st["f2_nonfinite"] == 0 and st["moments_nonfinite"] == 0
        assert st["cfl_over"] == _cfl_over(gpu, tiny, tiny.dts, 1)
    finally:
        gpu.close()


@pytest.mark.parametrize("graph", [False, True])
def test_nonfinite_is_reported(tiny, graph):
    """NaN and Inf planted in member 1, species 2: counted exactly before the
    call, spread by the sweeps after it (the count equals numpy's on the
    downloaded F2), and ram_run raises with the check on."""
    wl = tiny
    ns = len(wl.grid.species)
    gpu = _gpu(wl, members=2)
    gpu.set_graph(graph)
    try:
        bad = np.asfortranarray(np.array(wl.f2[2], copy=True))
        bad[3, 4, 5, 6] = np.nan
        bad[4, 2, 9, 30] = np.inf
        bad[1, 1, 1, 1] = -np.inf
        gpu.upload_f2(1, 2, bad)
        st = gpu.check()
        assert st["f2_nonfinite"] == 3 and st["moments_nonfinite"] == 0
        assert (st["first_member"], st["first_species"]) == (1, 2)
        with pytest.raises(abi.RamGpuError) as ei:
            gpu.set_check(True)
            gpu.ram_run(wl.dts)
        assert ei.value.code == -4
        st = gpu.last_status()
        count = sum(int(np.sum(~np.isfinite(gpu.download_f2(m, s)))) for m in range(2) for s in range(ns))
        assert st["f2_nonfinite"] == count > 3
        mom = sum(int(np.sum(~np.isfinite(np.asarray(gpu.moments(m, s))))) for m in range(2) for s in range(ns))
        assert st["moments_nonfinite"] == mom
        assert (st["first_member"], st["first_species"]) == (1, 2)
        assert gpu.check() == st
        # member 0 is untouched by member 1's values
        for s in range(ns):
            assert np.all(np.isfinite(gpu.download_f2(0, s)))
    finally:
        gpu.close()


def test_check_in_host_pipeline_and_courant(tiny):
    """With the check on, ram_run_host maps the word too; a DTs large enough
    to push Courant numbers above 1 is reported as ramgpu_cfl shows it."""
    wl = tiny
    ns = len(wl.grid.species)
    gpu = _gpu(wl)
    gpu.set_check(True)
    f2 = [np.asfortranarray(wl.f2[s]).copy(order="F") for s in range(ns)]
    try:
        gpu.ram_run_host(wl.dts, f2)
        st = gpu.last_status()
        assert st["f2_nonfinite"] == 0 and st["moments_nonfinite"] == 0
        big = 40.0 * wl.dts
        gpu.ram_run(big)
        st = gpu.last_status()
        want = _cfl_over(gpu, wl, big, 1)
        assert want > 0 and st["cfl_over"] == want
        f2[1][2, 3, 4, 5] = np.nan
        with pytest.raises(abi.RamGpuError) as ei:
            gpu.ram_run_host(wl.dts, f2)
        assert ei.value.code == -4
        assert gpu.last_status()["f2_nonfinite"] == int(np.sum(~np.isfinite(f2[1])))
        gpu.set_check(False)
        gpu.ram_run(wl.dts)  # no pass appended: the call itself does not raise
    finally:
        gpu.close()


def test_clip_count_matches_recorded_clip_bits(tiny):
    """The sweeps' clip count of a call (check on) equals the clip bits the
    adjoint's recording forward writes for the same call from the same
    state: one bit per updated cell that came out negative."""
    wl = tiny
    ns = len(wl.grid.species)
    gpu = _gpu(wl)
    big = 40.0 * wl.dts  # Courant numbers above 1: the update can undershoot
    try:
        gpu.adj_forward(1, big, [3.0], 1, [])
        rec = gpu.adj_record(0, ns)
        want = int(np.sum((rec & 8) != 0))
        for s in range(ns):
            gpu.upload_f2(0, s, wl.f2[s])
        gpu.set_check(True)
        gpu.set_kp(0, 3.0)
        gpu.ram_run(big)
        st = gpu.last_status()
        assert want > 0 and st["clips"] == want
        # with the check off the sweeps do not count
        gpu.set_check(False)
        gpu.ram_run(big)
        assert gpu.check()["clips"] == 0
    finally:
        gpu.close()


def test_check_needs_the_grid():
    """Before ramgpu_set_grid the pass has no grid to read: a state error."""
    import ctypes

    lib = abi.load_library()
    cfg = abi.Config(6, 9, 35, 72, 2, 1, 1.5, 0.8, 0.1, 0)
    h = ctypes.c_void_p()
    assert lib.ramgpu_create(ctypes.byref(cfg), ctypes.byref(h)) == abi.RAMGPU_OK
    try:
        st = abi.Status()
        assert lib.ramgpu_check(h, ctypes.byref(st)) == -3
    finally:
        lib.ramgpu_destroy(h)


def test_f2_stats_against_numpy(tiny):
    """ramgpu_f2_stats: exact min and max over all cells, the number content
    sum F2*WE*WMU over the updated cells within 1e-14 of numpy's, the same
    bits on a repeated call; negative and planted values are seen."""
    wl = tiny
    g = wl.grid
    gpu = abi.RamGpu(g, wl.fields)
    try:
        for s in range(len(g.species)):
            gpu.upload_f2(0, s, wl.f2[s])
            gpu.set_boundary(0, s, wl.fgeos[s])
        gpu.set_kp(0, 4.0)
        gpu.ram_run(wl.dts)
        w = g.we[None, None, 1:, None] * g.wmu[None, None, None, 1:-1]
        for s in range(len(g.species)):
            f = gpu.download_f2(0, s)
            lo, hi, q = gpu.f2_stats(0, s)
            assert lo == f.min() and hi == f.max()
            want = float(np.sum(f[1:, :-1, 1:, 1:-1] * w))
            assert abs(q - want) <= 1e-14 * abs(want), (q, want)
            assert gpu.f2_stats(0, s) == (lo, hi, q)
        f = gpu.download_f2(0, 2)
        f[3, 4, 5, 6] = -2.5
        f[1, 0, 0, 0] = 7.0e30
        gpu.upload_f2(0, 2, f)
        lo, hi, _ = gpu.f2_stats(0, 2)
        assert lo == -2.5 and hi == 7.0e30
    finally:
        gpu.close()
