"""GPU: ramgpu_ram_run_host, the call with F2 on the host pipelined over
item groups, gives the same bits as upload + ram_run + download, for every
group count, with the coefficient store, ensembles with uneven species
sets, resident (NULL) items, the loss bookkeeping and pitch-angle
diffusion; the resident ram_run over concurrent item groups gives the bits
of the single-stream step."""
import numpy as np
import pytest

from ramgpu import abi, workload as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tiny():
    return W.make_workload("tiny_pert")


def _gpu(wl, members=1, flags=0):
    g = wl.grid
    gpu = abi.RamGpu(g, wl.fields, n_members=members, flags=flags)
    for m in range(members):
        for s in range(len(g.species)):
            gpu.upload_f2(m, s, wl.f2[s])
            gpu.set_boundary(m, s, wl.fgeos[s])
        gpu.set_kp(m, 2.0 + m)
    return gpu


def _host_buffers(wl, members):
    ns = len(wl.grid.species)
    return [np.asfortranarray(wl.f2[k % ns]).copy(order="F") for k in range(members * ns)]


def _reference(wl, members=1, flags=0, calls=3, setup=None):
    """F2, moments and CFL after `calls` single-stream ram_run calls."""
    g = wl.grid
    ns = len(g.species)
    gpu = _gpu(wl, members, flags)
    gpu.set_step_groups(1)
    if setup:
        setup(gpu)
    for c in range(calls):
        gpu.set_kp(-1, 3.0 + c)
        gpu.ram_run(wl.dts)
    out = {"f2": [gpu.download_f2(m, s) for m in range(members) for s in range(ns)],
           "mom": [gpu.moments(m, s) for m in range(members) for s in range(ns)],
           "cfl": [gpu.cfl(m, s) for m in range(members) for s in range(ns)]}
    if flags & abi.FLAG_LOSSES:
        out["losses"] = [gpu.losses(m, s) for m in range(members) for s in range(ns)]
    gpu.close()
    return out


@pytest.mark.parametrize("groups", [1, 2, 3, 4, 8])
@pytest.mark.parametrize("store", [0, 4, 15])
def test_pipeline_equals_resident_run(tiny, groups, store):
    wl = tiny
    g = wl.grid
    ns = len(g.species)
    ref = _reference(wl, setup=lambda gp: gp.set_coef_store(store))
    gpu = _gpu(wl)
    gpu.set_coef_store(store)
    gpu.set_pipeline_groups(groups)
    f2 = _host_buffers(wl, 1)
    pe = [np.empty((g.nr, g.nt), order="F") for _ in range(ns)]
    pa = [np.empty((g.nr, g.nt), order="F") for _ in range(ns)]
    try:
        for c in range(3):
            gpu.set_kp(-1, 3.0 + c)
            gpu.ram_run_host(wl.dts, f2, pe, pa)
        for s in range(ns):
            assert np.array_equal(f2[s], ref["f2"][s]), s
            assert np.array_equal(gpu.download_f2(0, s), ref["f2"][s]), s
            assert np.array_equal(pe[s], ref["mom"][s][0]) and np.array_equal(pa[s], ref["mom"][s][1])
            assert np.array_equal(gpu.cfl(0, s), ref["cfl"][s])
    finally:
        gpu.close()


@pytest.mark.parametrize("graph", [False, True])
@pytest.mark.parametrize("groups", [2, 3, 4, 8])
def test_resident_groups_equal_single_stream(tiny, groups, graph):
    """ram_run with the items split over concurrent streams; an ensemble
    with uneven species sets, so groups hold items of several members."""
    wl = tiny
    ns = len(wl.grid.species)
    plans = [[0, 1, 2, 3], [1, 3], [0, 2]]

    def setup(gp):
        for m, sp in enumerate(plans):
            gp.set_member_species(m, sp)
        gp.set_coef_store(4)

    ref = _reference(wl, members=len(plans), setup=setup)
    gpu = _gpu(wl, members=len(plans))
    setup(gpu)
    gpu.set_graph(graph)
    gpu.set_step_groups(groups)
    assert gpu.step_groups() == groups
    try:
        for c in range(3):
            gpu.set_kp(-1, 3.0 + c)
            gpu.ram_run(wl.dts)
        for m in range(len(plans)):
            for s in range(ns):
                k = m * ns + s
                assert np.array_equal(gpu.download_f2(m, s), ref["f2"][k]), (m, s)
                if s not in plans[m]:
                    continue  # no moments or CFL for a species the member does not carry
                mom = gpu.moments(m, s)
                assert np.array_equal(mom[0], ref["mom"][k][0]) and np.array_equal(mom[1], ref["mom"][k][1])
                assert np.array_equal(gpu.cfl(m, s), ref["cfl"][k])
    finally:
        gpu.close()


def test_autotune_picks_groups(tiny):
    wl = tiny
    gpu = _gpu(wl)
    try:
        gpu.autotune(wl.dts, reps=1)
        assert 1 <= gpu.step_groups() <= min(8, len(wl.grid.species))
        assert gpu.pipeline_groups() == 4
    finally:
        gpu.close()


def test_pipeline_ensemble_and_resident_items(tiny):
    """Uneven member species sets; a NULL entry keeps that item resident (it
    is still advanced, and its host buffer is left alone)."""
    wl = tiny
    ns = len(wl.grid.species)
    plans = [[0, 1, 2, 3], [1, 3], [0], [2, 1]]

    def setup(gp):
        for m, sp in enumerate(plans):
            gp.set_member_species(m, sp)

    ref = _reference(wl, members=len(plans), setup=setup)
    gpu = _gpu(wl, members=len(plans))
    setup(gpu)
    gpu.set_pipeline_groups(3)
    f2 = _host_buffers(wl, len(plans))
    keep = f2[1].copy()
    f2_arg = list(f2)
    f2_arg[1] = None  # member 0, species 1 stays on the device
    try:
        for c in range(3):
            gpu.set_kp(-1, 3.0 + c)
            gpu.ram_run_host(wl.dts, f2_arg)
        for m, sp in enumerate(plans):
            for s in range(ns):
                k = m * ns + s
                assert np.array_equal(gpu.download_f2(m, s), ref["f2"][k]), (m, s)
                if f2_arg[k] is not None:
                    assert np.array_equal(f2[k], ref["f2"][k] if s in sp else np.asfortranarray(wl.f2[s]))
        assert np.array_equal(f2[1], keep)
    finally:
        gpu.close()


def test_pipeline_with_losses_and_diffusion(tiny):
    wl = tiny
    ns = len(wl.grid.species)
    d = W.pa_diffusion(wl.grid, wl.fields, seed=5)

    def setup(gp):
        gp.set_pa_diffusion(0, d)
        gp.reset_losses()

    ref = _reference(wl, flags=abi.FLAG_LOSSES, setup=setup)
    gpu = _gpu(wl, flags=abi.FLAG_LOSSES)
    setup(gpu)
    f2 = _host_buffers(wl, 1)
    try:
        for c in range(3):
            gpu.set_kp(-1, 3.0 + c)
            gpu.ram_run_host(wl.dts, f2)
        for s in range(ns):
            assert np.array_equal(f2[s], ref["f2"][s]), s
            assert np.array_equal(np.asarray(gpu.losses(0, s)), np.asarray(ref["losses"][s])), s
    finally:
        gpu.close()
    # diffusion without the bookkeeping runs in groups
    ref = _reference(wl, setup=lambda gp: gp.set_pa_diffusion(0, d))
    gpu = _gpu(wl)
    gpu.set_pa_diffusion(0, d)
    f2 = _host_buffers(wl, 1)
    try:
        for c in range(3):
            gpu.set_kp(-1, 3.0 + c)
            gpu.ram_run_host(wl.dts, f2)
        for s in range(ns):
            assert np.array_equal(f2[s], ref["f2"][s]), s
    finally:
        gpu.close()


def _pinned_like(arrs):
    torch = pytest.importorskip("torch")
    out = []
    for a in arrs:
        t = torch.empty(a.size, dtype=torch.float64, pin_memory=True).numpy()
        v = np.reshape(t, a.shape, order="F")
        v[...] = a
        out.append(v)
    return out


@pytest.mark.parametrize("groups", [1, 4])
def test_pipeline_graph_replay(tiny, groups):
    """With graphs on and page-locked buffers the pipeline is captured once
    per buffer set and replayed; alternating two buffer sets recaptures; a
    pageable set runs direct.  All give the resident run's bits."""
    wl = tiny
    g = wl.grid
    ns = len(g.species)
    ref = _reference(wl, calls=4)
    gpu = _gpu(wl)
    gpu.set_graph(True)
    gpu.set_pipeline_groups(groups)
    a = _pinned_like(_host_buffers(wl, 1))
    b = _pinned_like(_host_buffers(wl, 1))
    c = _host_buffers(wl, 1)  # pageable
    pe = _pinned_like([np.empty((g.nr, g.nt), order="F") for _ in range(ns)])
    pa = _pinned_like([np.empty((g.nr, g.nt), order="F") for _ in range(ns)])
    try:
        bufs = [a, a, b, c]
        for k in range(4):
            gpu.set_kp(-1, 3.0 + k)
            gpu.ram_run_host(wl.dts, bufs[k], pe, pa)
            nxt = bufs[k + 1] if k < 3 else None
            if nxt is not None and nxt is not bufs[k]:
                for s in range(ns):
                    nxt[s][...] = bufs[k][s]
        for s in range(ns):
            assert np.array_equal(c[s], ref["f2"][s]), s
            assert np.array_equal(pe[s], ref["mom"][s][0]) and np.array_equal(pa[s], ref["mom"][s][1])
    finally:
        gpu.close()


def test_pipeline_trace(tiny):
    """The traced call gives the same bits and a consistent timeline."""
    wl = tiny
    g = wl.grid
    ns = len(g.species)
    ref = _reference(wl, calls=2)
    gpu = _gpu(wl)
    gpu.set_graph(True)
    gpu.set_pipeline_groups(2)
    f2 = _host_buffers(wl, 1)
    try:
        with pytest.raises(abi.RamGpuError):
            gpu.pipeline_trace()
        gpu.set_pipeline_trace(True)
        for c in range(2):
            gpu.set_kp(-1, 3.0 + c)
            gpu.ram_run_host(wl.dts, f2)
        t = gpu.pipeline_trace()
        assert t.shape == (2, 3)
        assert np.all(t >= 0.0) and np.all(np.diff(t, axis=1) >= 0.0)
        assert t[1, 0] >= t[0, 0]  # uploads are chained in group order
        for s in range(ns):
            assert np.array_equal(f2[s], ref["f2"][s]), s
    finally:
        gpu.close()


def test_pipeline_argument_errors(tiny):
    wl = tiny
    gpu = _gpu(wl)
    try:
        with pytest.raises(abi.RamGpuError):
            gpu.set_pipeline_groups(0)
        with pytest.raises(abi.RamGpuError):
            gpu.set_step_groups(9)
        with pytest.raises(abi.RamGpuError):
            gpu.ram_run_host(wl.dts, [None])  # wrong number of entries
        bad = [np.zeros(5)] * len(wl.grid.species)
        with pytest.raises(abi.RamGpuError):
            gpu.ram_run_host(wl.dts, bad)
        with pytest.raises(abi.RamGpuError):
            gpu.ram_run_host(-1.0, _host_buffers(wl, 1))
    finally:
        gpu.close()


@pytest.mark.parametrize("chunks", [0, 1, 2, 3, 4, 8])
@pytest.mark.parametrize("graph", [False, True])
def test_plane_chunk_pipeline_equals_resident_run(tiny, chunks, graph):
    """ram_run_host over 0 (item groups), 1..8 chunks of L planes: the same
    F2, moments and CFL bits as the resident single-stream step, with the
    status pass (clip counts) on."""
    wl = tiny
    g = wl.grid
    ns = len(g.species)
    ref = _reference(wl)
    gpu = _gpu(wl)
    gpu.set_pipeline_chunks(chunks)
    gpu.set_graph(graph)
    gpu.set_check(True)
    f2 = _host_buffers(wl, 1)
    pe = [np.empty((g.nr, g.nt), order="F") for _ in range(ns)]
    pa = [np.empty((g.nr, g.nt), order="F") for _ in range(ns)]
    try:
        for c in range(3):
            gpu.set_kp(-1, 3.0 + c)
            gpu.ram_run_host(wl.dts, f2, pe, pa)
        for s in range(ns):
            assert np.array_equal(f2[s], ref["f2"][s]), s
            assert np.array_equal(gpu.download_f2(0, s), ref["f2"][s]), s
            assert np.array_equal(pe[s], ref["mom"][s][0]) and np.array_equal(pa[s], ref["mom"][s][1])
            assert np.array_equal(gpu.cfl(0, s), ref["cfl"][s])
        assert gpu.last_status()["f2_nonfinite"] == 0
    finally:
        gpu.close()
