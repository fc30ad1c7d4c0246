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


def test_noalloc_refuses_a_capturing_stream():
    """The call waits for its stream, so on a stream under capture it must
    return RAMGPU_ERR_STATE and leave the capture intact (it ends cleanly)."""
    torch = pytest.importorskip("torch")
    wl = W.make_workload("tiny")
    gpu = abi.RamGpu(wl.grid, wl.fields)
    gpu.upload_f2(0, 0, wl.f2[0])
    rc0, ref, err0 = _noalloc(gpu.lib, gpu.f2_device_ptr(0, 0), wl.grid)  # the set-up call, before capture
    assert rc0 == 0, err0
    x = torch.zeros(4, device="cuda")
    st = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    out = ctypes.c_double(0.0)
    we, wmu, ekev = (np.ascontiguousarray(a, dtype=np.float64) for a in (wl.grid.we, wl.grid.wmu, wl.grid.ekev))
    with torch.cuda.graph(g, stream=st):
        x += 1.0
        rc = gpu.lib.ramgpu_sumrc_noalloc(ctypes.c_void_p(gpu.f2_device_ptr(0, 0)), wl.grid.nr, wl.grid.nt,
                                          wl.grid.ne, wl.grid.npa, we.ctypes.data_as(abi._P),
                                          wmu.ctypes.data_as(abi._P), ekev.ctypes.data_as(abi._P),
                                          ctypes.c_void_p(st.cuda_stream), ctypes.byref(out))
    assert rc == -3
    buf = ctypes.create_string_buffer(256)
    gpu.lib.ramgpu_last_error(None, buf, 256)
    assert b"captured" in buf.value
    g.replay()
    torch.cuda.synchronize()
    assert float(x[0]) == 1.0
    rc1, again, err1 = _noalloc(gpu.lib, gpu.f2_device_ptr(0, 0), wl.grid)
    assert rc1 == 0 and again == ref, err1
    gpu.close()
