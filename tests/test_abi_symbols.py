"""The C-ABI library loads and exports every symbol include/ramgpu.h declares.

No compute call is made (this runs without a GPU)."""
import ctypes
import re

import pytest

from conftest import ROOT
from ramgpu import abi, build


def declared_symbols():
    text = (ROOT / "include" / "ramgpu.h").read_text()
    return sorted(set(re.findall(r"\b(ramgpu_[A-Za-z0-9_]+)\s*\(", text)))


def test_header_and_binding_agree():
    assert declared_symbols() == sorted(abi.EXPORTS)


@pytest.mark.parametrize("bounds", [False, True])
def test_library_exports_every_symbol(bounds):
    """Both the release library and the bounds-checked one."""
    path = build.LIB_BOUNDS_PATH if bounds else build.LIB_PATH
    if not path.exists():
        build.build_library(bounds=bounds)
    lib = ctypes.CDLL(str(path))
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_create_without_gpu_fails_cleanly():
    """ramgpu_create must return an error code (not abort) when no GPU is usable."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    lib = abi.load_library()
    cfg = abi.Config(20, 25, 35, 72, 1, 1, 1.5, 0.8, 0.1, 0)
    h = ctypes.c_void_p()
    rc = lib.ramgpu_create(ctypes.byref(cfg), ctypes.byref(h))
    assert rc != 0
    buf = ctypes.create_string_buffer(256)
    lib.ramgpu_last_error(None, buf, 256)
    assert buf.value


def test_bad_config_rejected_before_device_use():
    lib = abi.load_library()
    cfg = abi.Config(2, 25, 35, 72, 1, 1, 1.5, 0.8, 0.1, 0)  # NR too small
    h = ctypes.c_void_p()
    assert lib.ramgpu_create(ctypes.byref(cfg), ctypes.byref(h)) == -1
