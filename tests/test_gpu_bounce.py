"""GPU bounce integrals of computehI against the oracle: dipole lines on the
standard grid, and distorted lines (non-monotonic B, magnetopause-outside
lines) on the non-dipole test grid."""
import dataclasses

import numpy as np
import pytest

import pyoracle
from ramgpu import abi, workload as W

pytestmark = pytest.mark.gpu
TOL = 1e-12


def rel(a, b):
    den = np.max(np.abs(b))
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / (den if den > 0 else 1.0))


def _compare(wl, fields, lines):
    o = pyoracle.Oracle(wl.grid, fields)
    gpu = abi.RamGpu(wl.grid, fields)
    try:
        got = gpu.bounce_integrals(lines)
    finally:
        gpu.close()
    ref = o.bounce_integrals(lines)
    for name, a, b in zip(("H", "I", "HDens", "Bmirror"), got, ref):
        assert np.isfinite(a).all(), name
        assert rel(a, b) <= TOL, (name, rel(a, b))
    return got


def test_dipole_lines():
    wl = W.make_workload("single_h")
    fields = dataclasses.replace(wl.fields, outside=np.zeros_like(wl.fields.outside))
    h, fi, hd, bm = _compare(wl, fields, W.dipole_lines(wl.grid, 101))
    assert (h[:, :, 1:] > 0).all() and (fi[:, :, 1:] > 0).all()


def test_distorted_lines_and_outside():
    wl = W.make_workload("tiny_pert")
    lines = W.dipole_lines(wl.grid, 61)
    rng = np.random.Generator(np.random.PCG64(3))
    nthe = lines.chi.size
    ph = rng.uniform(0, 2 * np.pi, size=lines.b.shape[1:])
    wig = 1.0 + 0.15 * np.sin(7.0 * lines.chi[:, None, None] + ph[None])
    lines = dataclasses.replace(lines, b=lines.b * wig,
                                dens=lines.dens * rng.lognormal(0.0, 0.2, size=lines.dens.shape))
    assert np.asarray(wl.fields.outside).any()
    h, fi, hd, bm = _compare(wl, wl.fields, lines)
    out = np.asarray(wl.fields.outside) == 1
    assert np.all(h[out] == 0.0)
