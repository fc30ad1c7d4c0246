"""The no-allocation SETRC entry point against the library's existing path.

ramgpu_sumrc_noalloc is for callers that cannot allocate device memory: a
host model that gives every device byte to its own pool and forbids
libraries to call cudaMalloc, or code that must not call allocation APIs
while work is in flight.  Its only scratch is a fixed array inside the
library.  Through the C ABI it must give the same SETRC as
ramgpu_reset_losses + ramgpu_losses (which use the context's allocated
scratch), within the 1e-12 relative tolerance of the other parity tests,
on two calls in a row (with a ram_run between them).
"""
import ctypes

import numpy as np
import pytest

from ramgpu import abi, workload as W

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _noalloc(lib, dptr, g, ne=None):
    out = ctypes.c_double(float("nan"))
    we, wmu, ekev = (np.ascontiguousarray(a, dtype=np.float64) for a in (g.we, g.wmu, g.ekev))
    rc = lib.ramgpu_sumrc_noalloc(ctypes.c_void_p(dptr), g.nr, g.nt, g.ne if ne is None else ne, g.npa,
                                  we.ctypes.data_as(abi._P), wmu.ctypes.data_as(abi._P),
                                  ekev.ctypes.data_as(abi._P), None, ctypes.byref(out))
    buf = ctypes.create_string_buffer(256)
    lib.ramgpu_last_error(None, buf, 256)
    return rc, out.value, buf.value.decode()


def test_noalloc_sumrc_matches_existing_entry_point():
    wl = W.make_workload("tiny")
    g = wl.grid
    gpu = abi.RamGpu(g, wl.fields)
    for s in range(len(g.species)):
        gpu.upload_f2(0, s, wl.f2[s])
        gpu.set_boundary(0, s, wl.fgeos[s])
    gpu.set_kp(0, 3.0)
    for call in range(2):
        gpu.reset_losses()  # SETRC of the current state through the existing path
        for s in range(len(g.species)):
            ref = gpu.losses(0, s)[0]
            rc, got, err = _noalloc(gpu.lib, gpu.f2_device_ptr(0, s), g)
            assert rc == 0, err
            assert ref > 0 and abs(got - ref) <= TOL * ref, (call, s, got, ref)
        gpu.ram_run(wl.dts)
    gpu.close()


def test_noalloc_rejects_sizes_beyond_its_scratch():
    wl = W.make_workload("tiny")
    gpu = abi.RamGpu(wl.grid, wl.fields)
    rc, _, err = _noalloc(gpu.lib, gpu.f2_device_ptr(0, 0), wl.grid, ne=2048)
    assert rc == abi.RAMGPU_OK - 1 and "1024" in err
    gpu.close()
