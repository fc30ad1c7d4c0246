"""GPU: F2 in the reference's own layout F2(NS,NR,NT,NE,NPA)
(src/ModRamVariables.f90:31, species index fastest) and the moments as
PPERT/PPART(NS,NR,NT): the device-side transposes of ramgpu_upload_f2_all /
ramgpu_download_f2_all and the whole call ramgpu_ram_run_ref give the bits
of the per-species path, from page-locked and ordinary host memory, through
the copy engines (forced staging) and in place, with and without the CUDA
graph, for ensembles with uneven species sets."""
import numpy as np
import pytest

from ramgpu import abi, workload as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def wl():
    return W.make_workload("tiny_pert")


def _gpu(wl, members=1):
    g = wl.grid
    gpu = abi.RamGpu(g, wl.fields, n_members=members)
    for m in range(members):
        for s in range(len(g.species)):
            gpu.upload_f2(m, s, np.asarray(wl.f2[s]) * (1.0 + 0.25 * m))
            gpu.set_boundary(m, s, wl.fgeos[s])
        gpu.set_kp(m, 2.0 + m)
    return gpu


def _interleave(blocks):
    """Per-species (NR,NT,NE,NPA) arrays -> F2(NS,NR,NT,NE,NPA), Fortran order."""
    return np.asfortranarray(np.stack([np.asfortranarray(b) for b in blocks], axis=0))


def _pinned(shape):
    torch = pytest.importorskip("torch")
    n = int(np.prod(shape))
    t = torch.empty(n, dtype=torch.float64, pin_memory=True)
    return t, np.reshape(t.numpy(), shape, order="F")


@pytest.mark.parametrize("stage", [False, True])
def test_upload_download_all_bitwise(wl, stage):
    g = wl.grid
    ns = len(g.species)
    gpu = _gpu(wl, members=2)
    gpu.set_ref_staging(stage)
    rng = np.random.Generator(np.random.PCG64(5))
    blocks = [rng.random((g.nr, g.nt, g.ne, g.npa)) for _ in range(ns)]
    try:
        gpu.upload_f2_all(1, _interleave(blocks))
        for s in range(ns):
            assert np.array_equal(gpu.download_f2(1, s), blocks[s]), s
            # member 0 untouched
            assert np.array_equal(gpu.download_f2(0, s), np.asarray(wl.f2[s])), s
        back = gpu.download_f2_all(1)
        assert np.array_equal(back, _interleave(blocks))
        assert np.array_equal(gpu.download_f2_all(0), _interleave([np.asarray(a) for a in wl.f2]))
    finally:
        gpu.close()


def _reference(wl, members, species, calls):
    """Resident single-stream run: F2 and moments per (member, species)."""
    g = wl.grid
    ns = len(g.species)
    gpu = _gpu(wl, members)
    gpu.set_step_groups(1)
    for m in range(members):
        gpu.set_member_species(m, species[m])
    for c in range(calls):
        gpu.set_kp(-1, 3.0 + c)
        gpu.ram_run(wl.dts)
    out = ([[gpu.download_f2(m, s) for s in range(ns)] for m in range(members)],
           [[gpu.moments(m, s) for s in range(ns)] for m in range(members)])
    gpu.close()
    return out


@pytest.mark.parametrize("memory", ["pageable", "pinned"])
@pytest.mark.parametrize("graph,stage,groups,chunks", [(False, False, 1, 0), (True, False, 4, 0), (True, True, 2, 4),
                                                       (False, True, 3, 0), (False, False, 2, 3),
                                                       (True, False, 4, 4), (True, False, 1, 8),
                                                       (True, 2, 4, 4), (False, 2, 2, 3), (True, 2, 1, 8)])
def test_ram_run_ref_equals_per_species_path(wl, memory, graph, stage, groups, chunks):
    g = wl.grid
    ns = len(g.species)
    members = 2
    species = [[0, 1, 2, 3], [3, 1]]
    ref_f2, ref_mom = _reference(wl, members, species, calls=3)
    gpu = _gpu(wl, members)
    for m in range(members):
        gpu.set_member_species(m, species[m])
    gpu.set_graph(graph)
    gpu.set_ref_staging(stage)
    gpu.set_step_groups(groups)
    gpu.set_pipeline_chunks(chunks)
    keep = []
    f2, pe, pa = [], [], []
    for m in range(members):
        start = _interleave([gpu.download_f2(m, s) for s in range(ns)])
        if memory == "pinned":
            t, a = _pinned(start.shape)
            a[...] = start
            keep.append(t)
            tp, p = _pinned((ns, g.nr, g.nt))
            tq, q = _pinned((ns, g.nr, g.nt))
            keep += [tp, tq]
        else:
            a = start.copy(order="F")
            p = np.zeros((ns, g.nr, g.nt), order="F")
            q = np.zeros((ns, g.nr, g.nt), order="F")
        f2.append(a)
        pe.append(p)
        pa.append(q)
    try:
        for c in range(3):
            gpu.set_kp(-1, 3.0 + c)
            gpu.ram_run_ref(wl.dts, f2, pe, pa)
        for m in range(members):
            for s in range(ns):
                assert np.array_equal(f2[m][s], ref_f2[m][s]), (m, s)
                assert np.array_equal(gpu.download_f2(m, s), ref_f2[m][s]), (m, s)
                if s in species[m]:
                    assert np.array_equal(pe[m][s], ref_mom[m][s][0]), (m, s)
                    assert np.array_equal(pa[m][s], ref_mom[m][s][1]), (m, s)
    finally:
        gpu.close()


def test_ram_run_ref_equals_ram_run_host(wl):
    """The reference-layout call and the per-species host call (page-locked
    buffers of both) leave the same bits in the caller's arrays."""
    g = wl.grid
    ns = len(g.species)
    a = _gpu(wl)
    b = _gpu(wl)
    a.set_graph(True)
    b.set_graph(True)
    host = [np.asfortranarray(wl.f2[s]).copy(order="F") for s in range(ns)]
    pe_h = [np.zeros((g.nr, g.nt), order="F") for _ in range(ns)]
    pa_h = [np.zeros((g.nr, g.nt), order="F") for _ in range(ns)]
    f2r = _interleave([np.asarray(x) for x in wl.f2]).copy(order="F")
    pe_r = np.zeros((ns, g.nr, g.nt), order="F")
    pa_r = np.zeros((ns, g.nr, g.nt), order="F")
    try:
        for c in range(4):
            a.set_kp(-1, 2.0 + c)
            b.set_kp(-1, 2.0 + c)
            a.ram_run_host(wl.dts, host, pe_h, pa_h)
            b.ram_run_ref(wl.dts, [f2r], [pe_r], [pa_r])
        for s in range(ns):
            assert np.array_equal(f2r[s], host[s]), s
            assert np.array_equal(pe_r[s], pe_h[s]) and np.array_equal(pa_r[s], pa_h[s]), s
    finally:
        a.close()
        b.close()
