"""Host logic of the ctypes mirror around ramgpu_ram_run_host, on the CPU
with a stand-in for the library: the address tables it passes, their reuse
for a repeated buffer set, and the argument checks."""
import ctypes as C
import types

import numpy as np
import pytest

from ramgpu import abi


class _FakeLib:
    """Records the address tables of each ramgpu_ram_run_host call."""

    def __init__(self):
        self.calls = []

    def ramgpu_ram_run_host(self, h, dts, t_f2, t_pe, t_pa):
        def addrs(t):
            return None if t is None else [t[k] for k in range(len(t))]

        self.calls.append((dts, t_f2, addrs(t_f2), addrs(t_pe), addrs(t_pa)))
        return abi.RAMGPU_OK

    def ramgpu_last_error(self, h, buf, n):
        return 0

    def ramgpu_destroy(self, h):
        return 0


def _model(members=1, ns=2):
    m = abi.RamGpu.__new__(abi.RamGpu)
    m.lib = _FakeLib()
    m.h = None
    m.grid = types.SimpleNamespace(nr=4, nt=5, ne=6, npa=7)
    m.n_members = members
    m.ns = ns
    m._host_tables = None
    return m


def _bufs(ns=2):
    f2 = [np.zeros((4, 5, 6, 7), order="F") for _ in range(ns)]
    pe = [np.zeros((4, 5), order="F") for _ in range(ns)]
    pa = [np.zeros((4, 5), order="F") for _ in range(ns)]
    return f2, pe, pa


def test_tables_hold_the_buffer_addresses():
    m = _model()
    f2, pe, pa = _bufs()
    m.ram_run_host(5.0, f2, pe, pa)
    dts, _, a_f2, a_pe, a_pa = m.lib.calls[-1]
    assert dts == 5.0
    assert a_f2 == [a.ctypes.data for a in f2]
    assert a_pe == [a.ctypes.data for a in pe] and a_pa == [a.ctypes.data for a in pa]
    # None entries stay NULL; omitted moment lists are NULL tables
    m.ram_run_host(5.0, [f2[0], None])
    _, _, a_f2, a_pe, a_pa = m.lib.calls[-1]
    assert a_f2 == [f2[0].ctypes.data, None] and a_pe is None and a_pa is None


def test_repeated_buffer_set_reuses_its_tables():
    m = _model()
    f2, pe, pa = _bufs()
    m.ram_run_host(5.0, f2, pe, pa)
    m.ram_run_host(5.0, list(f2), pe, pa)  # same arrays in a new list
    assert m.lib.calls[0][1] is m.lib.calls[1][1]
    # another array in one slot: a new table with its address
    g = np.zeros((4, 5, 6, 7), order="F")
    m.ram_run_host(5.0, [f2[0], g], pe, pa)
    assert m.lib.calls[2][1] is not m.lib.calls[1][1]
    assert m.lib.calls[2][2] == [f2[0].ctypes.data, g.ctypes.data]
    # a buffer made read-only since: checked again, and refused
    g.flags.writeable = False
    with pytest.raises(abi.RamGpuError):
        m.ram_run_host(5.0, [f2[0], g], pe, pa)
    m.close()
    assert m._host_tables is None


@pytest.mark.parametrize("bad", ["count", "dtype", "size", "layout", "type"])
def test_argument_checks(bad):
    m = _model()
    f2, pe, pa = _bufs()
    if bad == "count":
        f2 = f2[:1]
    elif bad == "dtype":
        f2[1] = f2[1].astype(np.float32)
    elif bad == "size":
        f2[1] = np.zeros(10)
    elif bad == "layout":
        f2[1] = np.zeros((4, 5, 6, 14), order="F")[:, :, :, ::2]
    else:
        f2[1] = [0.0] * (4 * 5 * 6 * 7)
    with pytest.raises(abi.RamGpuError):
        m.ram_run_host(5.0, f2, pe, pa)
    assert not m.lib.calls


def test_argtypes_take_address_tables():
    """The library's entry takes the tables (double *const *) as plain
    pointers, so the c_void_p arrays pass as they are (loads without a GPU)."""
    from ramgpu import build

    if not build.LIB_PATH.exists():
        build.build_library()
    lib = abi.load_library()
    at = lib.ramgpu_ram_run_host.argtypes
    assert at[2] is C.c_void_p and at[3] is C.c_void_p and at[4] is C.c_void_p
    assert C.c_void_p.from_param((C.c_void_p * 2)(1, 2)) is not None
