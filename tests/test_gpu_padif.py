"""GPU implicit pitch-angle diffusion (WPADIF / FLCscatter) against the
oracle: one application, ram_run with the diffusion on some species (per
step, graph replay and direct launches), and the LSWAE bookkeeping."""
import numpy as np
import pytest

import pyoracle
from ramgpu import abi, workload as W

pytestmark = pytest.mark.gpu
TOL = 1e-12


def rel(a, b):
    den = np.max(np.abs(b))
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / (den if den > 0 else 1.0))


@pytest.fixture(scope="module")
def pert():
    wl = W.make_workload("tiny_pert")
    d = {s: W.pa_diffusion(wl.grid, wl.fields, seed=30 + s) for s in (0, 2)}
    return wl, d


def _gpu(wl, d, flags=0, kp=3.0):
    g = wl.grid
    gpu = abi.RamGpu(g, wl.fields, flags=flags)
    for s in range(len(g.species)):
        gpu.upload_f2(0, s, wl.f2[s])
        gpu.set_boundary(0, s, wl.fgeos[s])
    for s, a in d.items():
        gpu.set_pa_diffusion(s, a)
    gpu.set_kp(-1, kp)
    return gpu


def test_single_application(pert):
    wl, d = pert
    o = pyoracle.Oracle(wl.grid, wl.fields)
    gpu = _gpu(wl, d)
    try:
        gpu.apply_op(wl.dts, abi.OP_PADIF)
        for s in range(len(wl.grid.species)):
            ref = np.asfortranarray(wl.f2[s]).copy(order="F")
            if s in d:
                o.padif(ref, d[s], wl.dts)
            got = gpu.download_f2(0, s)
            assert rel(got, ref) <= TOL, s
            if s not in d:
                assert np.array_equal(got, ref)
    finally:
        gpu.close()


@pytest.mark.parametrize("graph", [False, True])
def test_ram_run_with_diffusion(pert, graph):
    wl, d = pert
    g = wl.grid
    o = pyoracle.Oracle(g, wl.fields)
    gpu = _gpu(wl, d)
    gpu.set_graph(graph)
    ref = [np.asfortranarray(a).copy(order="F") for a in wl.f2]
    try:
        for step in range(3):
            for s in range(len(g.species)):  # per-step parity from the oracle's state
                gpu.upload_f2(0, s, ref[s])
            gpu.ram_run(wl.dts)
            out = o.ram_run(ref, wl.fgeos, wl.dts, kp=3.0, want_flux=True, daa=d)
            for s in range(len(g.species)):
                assert rel(gpu.download_f2(0, s), ref[s]) <= TOL, (step, s)
                pe, pa = gpu.moments(0, s)
                assert rel(pe, out["ppert"][s]) <= TOL and rel(pa, out["ppart"][s]) <= TOL
        # removing the coefficient restores the plain step (and the graph is recaptured)
        for s in d:
            gpu.set_pa_diffusion(s, None)
        for s in range(len(g.species)):
            gpu.upload_f2(0, s, ref[s])
        gpu.ram_run(wl.dts)
        o.ram_run(ref, wl.fgeos, wl.dts, kp=3.0)
        for s in range(len(g.species)):
            assert rel(gpu.download_f2(0, s), ref[s]) <= TOL
    finally:
        gpu.close()


def test_losses_with_diffusion(pert):
    wl, d = pert
    g = wl.grid
    o = pyoracle.Oracle(g, wl.fields)
    gpu = _gpu(wl, d, flags=abi.FLAG_LOSSES)
    try:
        gpu.reset_losses()
        ref = [np.asfortranarray(a).copy(order="F") for a in wl.f2]
        losses = {s: (o.sumrc(ref[s]), 0.0, 0.0, 0.0) for s in range(len(g.species))}
        wae = {s: 0.0 for s in range(len(g.species))}
        for _ in range(2):
            gpu.ram_run(wl.dts)
            out = o.ram_run(ref, wl.fgeos, wl.dts, kp=3.0, losses=losses, daa=d)
            losses = out["losses"]
            for s in wae:
                wae[s] += out["lswae"][s]
        for s in range(len(g.species)):
            got, exp = gpu.losses(0, s), losses[s]
            assert abs(got[0] - exp[0]) <= 1e-12 * exp[0]
            for k in (1, 2, 3):
                assert abs(got[k] - exp[k]) <= 1e-12 * exp[0], (s, k)
            assert abs(gpu.loss_wae(0, s) - wae[s]) <= 1e-12 * exp[0], (s, gpu.loss_wae(0, s), wae[s])
            if s not in d:
                assert gpu.loss_wae(0, s) == 0.0
            assert rel(gpu.download_f2(0, s), ref[s]) <= TOL
    finally:
        gpu.close()


def test_adjoint_refuses_diffusion(pert):
    wl, d = pert
    gpu = _gpu(wl, d)
    try:
        with pytest.raises(abi.RamGpuError):
            gpu.adj_forward(2, wl.dts, [3.0, 3.0], 1, [])
    finally:
        gpu.close()
