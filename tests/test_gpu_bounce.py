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


FIELD_NAMES = ("fnhs", "fnis", "hdns", "bounhs", "bounis", "bnes", "dbdt", "didt", "dibndt", "eir", "eip")


@pytest.mark.parametrize("name,dthi", [("single_h", 0.0), ("tiny_pert", 300.0)])
def test_compute_hI_fills_the_context_fields(name, dthi):
    """ramgpu_compute_hI on the device equals the oracle's fill, and a
    ram_run on the new tables equals the oracle's ram_run on them."""
    wl = W.make_workload(name)
    fields = wl.fields if name == "tiny_pert" else dataclasses.replace(
        wl.fields, outside=np.zeros_like(wl.fields.outside))
    lines = W.dipole_lines(wl.grid, 101)
    if name == "tiny_pert":
        rng = np.random.Generator(np.random.PCG64(4))
        ph = rng.uniform(0, 2 * np.pi, size=lines.b.shape[1:])
        lines = dataclasses.replace(lines, b=lines.b * (1.0 + 0.1 * np.sin(5.0 * lines.chi[:, None, None] + ph[None])))
    o = pyoracle.Oracle(wl.grid, fields)
    f0 = {k: np.asarray(getattr(fields, k)) for k in FIELD_NAMES}
    ref = o.compute_hI(lines, bnormal=3.2e4, dthi=dthi, fields=f0)
    gpu = abi.RamGpu(wl.grid, fields)
    try:
        gpu.compute_hI(lines, wl.grid.pa, wl.grid.pabn, bnormal=3.2e4, dthi=dthi)
        got = gpu.get_fields()
        for k in FIELD_NAMES:
            assert np.isfinite(got[k]).all(), k
            assert rel(got[k], ref[k]) <= TOL, (k, rel(got[k], ref[k]))
        # one step on the new tables, against the oracle on the same tables
        newf = dataclasses.replace(fields, **{k: np.ascontiguousarray(got[k]) for k in FIELD_NAMES})
        o2 = pyoracle.Oracle(wl.grid, newf)
        ref_f2 = [np.asfortranarray(a).copy(order="F") for a in wl.f2]
        for s in range(len(wl.grid.species)):
            gpu.upload_f2(0, s, ref_f2[s])
            gpu.set_boundary(0, s, wl.fgeos[s])
        gpu.set_kp(-1, 3.0)
        gpu.ram_run(wl.dts)
        o2.ram_run(ref_f2, wl.fgeos, wl.dts, kp=3.0)
        for s in range(len(wl.grid.species)):
            assert rel(gpu.download_f2(0, s), ref_f2[s]) <= TOL, s
    finally:
        gpu.close()
