"""GPU: per-step parity from states the GPU itself evolved over long runs.

The short parity tests start every step from the initial state.  Here the
GPU advances alone along a whole workload; at sampled steps its state is
downloaded, the oracle (or the reference's own ram_run, translated) takes
one ram_run call from that state, and the
GPU's own next call must agree to the per-step bar (1e-12 relative
max-norm) for F2, the moments, FLUX and DtsNext.  Late in a run F2 has
steepened, the limiter takes every branch and clip events occur, so this
is where a rounding-level difference could grow into a branch difference.

  * single H+ on 20x25x35x72 at Kp 3, dt 5 s, 720 DTs steps (360 calls);
  * e-, H+, He+, O+ on 20x25x35x72, Kp rising 1 -> 6 over 4320 DTs steps
    (2160 calls, VT recomputed every call);
  * closed faces, no losses or mask: the content sum F2*WE*WMU conserved to
    1e-13 over 720 DTs steps on the standard grid;
  * the refined 40x49x70x144 grid after 100 DTs steps.
"""
import dataclasses
import os

import numpy as np
import pytest

from ramgpu import abi, workload as W
import pyoracle

pytestmark = pytest.mark.gpu
TOL = 1e-12


def rel(a, b):
    den = np.max(np.abs(b))
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / (den if den > 0 else 1.0))


def _threads(ns):
    cores = os.cpu_count() or 1
    outer = max(1, min(ns, cores))
    return outer, max(1, cores // outer)


def _gpu(wl, grid=None, flags=0):
    g = grid or wl.grid
    gpu = abi.RamGpu(g, wl.fields, flags=flags)
    for s in range(len(g.species)):
        gpu.upload_f2(0, s, wl.f2[s])
        gpu.set_boundary(0, s, wl.fgeos[s])
    return gpu


def _check_call(gpu, o, wl, kp, nthreads):
    """One call from the GPU's current state on both sides (o: the C oracle,
    or the reference's own ram_run when o is a refrun.RefRam); returns the
    worst relative error of F2 and the clip events of the GPU's call."""
    g = wl.grid
    ns = len(g.species)
    ref = [gpu.download_f2(0, s) for s in range(ns)]
    gpu.set_kp(0, kp)
    gpu.ram_run(wl.dts)
    clips = gpu.last_status()["clips"]
    if isinstance(o, pyoracle.Oracle):
        out = o.ram_run(ref, wl.fgeos, wl.dts, kp=kp, want_flux=True, nthreads=nthreads)
    else:
        out = o.ram_run(ref, wl.fgeos, wl.dts, kp)
    worst = 0.0
    for s in range(ns):
        e = rel(gpu.download_f2(0, s), ref[s])
        worst = max(worst, e)
        assert e <= TOL, (s, e)
        pe, pa = gpu.moments(0, s)
        assert rel(pe, out["ppert"][s]) <= TOL, s
        assert rel(pa, out["ppart"][s]) <= TOL, s
        assert rel(gpu.flux(0, s), out["flux"][s]) <= TOL, s
    dn = gpu.cfl(0, 0)[4]
    assert abs(dn - out["dts_next"]) <= 1e-12 * out["dts_next"], (dn, out["dts_next"])
    return worst, clips


def _long_run(name, calls, samples, checker="oracle"):
    wl = W.make_workload(name)
    g = wl.grid
    outer, inner = _threads(len(g.species))
    if checker == "reference":
        import refrun
        if refrun.build() is None:
            pytest.skip("translated reference not present (oracle/_ref/ramref.c)")
        o = refrun.RefRam(g, wl.fields, threads=outer)
    else:
        o = pyoracle.Oracle(g, wl.fields)
    gpu = _gpu(wl)
    gpu.set_graph(True)
    gpu.set_check(True)  # status word each call: counts the clip events
    pyoracle.set_inner_threads(inner)
    report = {}
    try:
        c = 0
        for target in sorted(samples):
            while c < target:
                gpu.set_kp(0, wl.kp(2 * c))
                gpu.ram_run(wl.dts)
                c += 1
            report[c] = _check_call(gpu, o, wl, wl.kp(2 * c), outer)
            c += 1
        assert c <= calls
    finally:
        pyoracle.set_inner_threads(1)
        gpu.close()
    return report


def test_single_species_720_steps():
    """H+ at Kp 3 along the whole 720-step run: calls 0, 45, 180, 359
    (DTs steps 0, 90, 360, 718)."""
    rep = _long_run("single_h", 360, [0, 45, 180, 359])
    assert max(w for w, _ in rep.values()) <= TOL
    print("single_h per-step rel err / clips by call:", rep)


def test_four_species_kp_ramp_4320_steps():
    """Four species along the Kp 1 -> 6 ramp to DTs step 4318: calls 0, 45,
    180, 360, 900, 1440, 1980, 2159."""
    rep = _long_run("four_sp", 2160, [0, 45, 180, 360, 900, 1440, 1980, 2159])
    assert max(w for w, _ in rep.values()) <= TOL
    print("four_sp per-step rel err / clips by call:", rep)


def test_four_species_ramp_against_reference():
    """The same ramp checked against the reference's own ram_run (its
    Fortran translated by oracle/f90c.py) at calls 0, 360, 1440 and 2159."""
    rep = _long_run("four_sp", 2160, [0, 360, 1440, 2159], checker="reference")
    assert max(w for w, _ in rep.values()) <= TOL
    print("four_sp against the reference, per-step rel err / clips by call:", rep)


def content_q(g, f2):
    w = g.we[None, None, 1:, None] * g.wmu[None, None, None, 1:-1]
    return float(np.sum(f2[1:, :-1, 1:, 1:-1] * w))


def test_closed_conservation_720_steps():
    """Closed faces (R, E, MU), periodic MLT, no CEX/ATMOL/mask: the content
    sum_{I>=2, J<NT, K>=2, 2<=L<NPA} F2*WE*WMU of H+ on the standard grid
    holds to 1e-13 over 720 DTs steps, with no clip event (an update that
    came out negative would be set to 1e-15 and break the balance)."""
    wl = W.make_workload("single_h")
    g = dataclasses.replace(wl.grid, species=tuple(dataclasses.replace(s, cex_kind=W.CEX_NONE)
                                                   for s in wl.grid.species))
    gpu = _gpu(wl, grid=g, flags=abi.FLAG_CLOSED | abi.FLAG_NO_ATMOL)
    gpu.set_graph(True)
    gpu.set_check(True)
    q0 = content_q(g, np.asfortranarray(wl.f2[0]))
    clips = 0
    try:
        for c in range(360):
            gpu.set_kp(0, 3.0)
            gpu.ram_run(wl.dts)
            clips += gpu.last_status()["clips"]
        f = gpu.download_f2(0, 0)
    finally:
        gpu.close()
    assert clips == 0
    drift = abs(content_q(g, f) - q0) / q0
    assert drift <= 1e-13, drift
    assert f.min() >= 0


def test_refined_grid_after_100_steps():
    """The refined 40x49x70x144 grid (four species, 632 MB of F2): the GPU
    runs 50 calls (100 DTs steps) of the Kp ramp alone, then its next call
    matches the oracle's call from the same state."""
    rep = _long_run("refined", 51, [50])
    assert rep[50][0] <= TOL
