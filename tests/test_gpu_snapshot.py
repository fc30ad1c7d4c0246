"""GPU: ramgpu_save_state / ramgpu_load_state round trip.  A run saved
after two calls, loaded into a fresh context and continued gives the bits
of the uninterrupted run (F2, moments, CFL), for an ensemble with uneven
species sets, a retired member and an explicit potential; a damaged file
or one of other dimensions is refused and leaves the state unchanged."""
import numpy as np
import pytest

from ramgpu import abi, workload as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def wl():
    return W.make_workload("tiny_pert")


def _model(wl, members=3):
    g = wl.grid
    gpu = abi.RamGpu(g, wl.fields, n_members=members)
    for m in range(members):
        for s in range(len(g.species)):
            gpu.upload_f2(m, s, np.asarray(wl.f2[s]) * (1.0 + 0.5 * m))
            gpu.set_boundary(m, s, wl.fgeos[s] * (1.0 + 0.1 * m))
    gpu.set_member_species(1, [3, 0])
    return gpu


def _state(gpu, wl, members=3):
    ns = len(wl.grid.species)
    return ([gpu.download_f2(m, s) for m in range(members) for s in range(ns)]
            + [np.concatenate(gpu.moments(m, s)) for m in range(members) for s in range(ns)])


def test_round_trip_continues_bitwise(wl, tmp_path):
    g = wl.grid
    vt = np.asfortranarray(np.random.Generator(np.random.PCG64(3)).normal(0.0, 2e3, size=(g.nr + 1, g.nt)))
    a = _model(wl)
    a.set_potential(2, vt)
    for c in range(2):
        a.set_kp(0, 2.0 + c)
        a.set_kp(1, 4.0 - c)
        a.ram_run(wl.dts)
    a.set_member_active(1, False)
    p = tmp_path / "state.snap"
    a.save_state(p, time=600.0)
    info = abi.snapshot_info(p)
    assert info["n_members"] == 3 and info["time"] == 600.0
    for c in range(3):
        a.ram_run(wl.dts)
    want = _state(a, wl)
    b = _model(wl)  # other initial state and settings, overwritten by the load
    assert b.load_state(p) == 600.0
    for c in range(3):
        b.ram_run(wl.dts)
    got = _state(b, wl)
    for x, y in zip(got, want):
        assert np.array_equal(x, y)
    a.close()
    b.close()


def test_damaged_or_foreign_file_leaves_state(wl, tmp_path):
    a = _model(wl)
    a.ram_run(wl.dts)
    p = tmp_path / "s.snap"
    a.save_state(p)
    raw = bytearray(p.read_bytes())
    raw[len(raw) // 2] ^= 0x01
    bad = tmp_path / "bad.snap"
    bad.write_bytes(bytes(raw))
    before = _state(a, wl)
    with pytest.raises(abi.RamGpuError) as e:
        a.load_state(bad)
    assert e.value.code == -6
    for x, y in zip(_state(a, wl), before):
        assert np.array_equal(x, y)
    two = _model(wl, members=2)
    with pytest.raises(abi.RamGpuError) as e:
        two.load_state(p)
    assert e.value.code == -1
    a.close()
    two.close()
