"""CPU scalar adjoint of the oracle (the independent check of the GPU adjoint).

With the limiter branches, the clipped cells and the DRIFTR ghost sources
frozen, each sweep is an affine map of (F2, FGEOS), so a central difference
whose two runs record the same branches as the base run equals the transpose
product <lam, A dx> up to rounding.  The window test then checks the whole
ram_run sequence (sweeps, CHAREXCHANGE/ATMOL factors, periodic copy,
magnetopause mask, the ANISCH F2(:,:,:,1) side effect, the FLUX observation
operator) against finite differences of J.
"""
import math

import numpy as np
import pytest

import pyoracle
from ramgpu import workload as W


@pytest.fixture(scope="module")
def pert():
    wl = W.make_workload("tiny_pert")
    return wl, pyoracle.Oracle(wl.grid, wl.fields)


@pytest.mark.parametrize("which", ["R", "P", "E", "MU"])
def test_sweep_transpose_dot_product(pert, which):
    wl, o = pert
    rng = np.random.Generator(np.random.PCG64(17))
    vt = o.vt_vols(4.0)
    for s in range(len(wl.grid.species)):
        x0 = np.asfortranarray(wl.f2[s])
        fg = np.asfortranarray(wl.fgeos[s])
        dx = rng.uniform(-1, 1, x0.shape) * x0
        dg = rng.uniform(-1, 1, fg.shape) * fg
        lam = np.asfortranarray(rng.standard_normal(x0.shape))

        def run(e):
            f = np.asfortranarray(x0 + e * dx)
            return f, o.sweep_rec(which, s, f, vt, wl.dts, np.asfortranarray(fg + e * dg))

        _, t0 = run(0.0)
        lt = lam.copy(order="F")
        gg = np.zeros(fg.shape, order="F")
        o.sweep_adj(t0, lt, wl.dts, gg)
        ad = float(np.sum(lt * dx) + np.sum(gg * dg))
        if which == "R":
            assert (t0[4] >= 0).any() and np.abs(gg).max() > 0
        else:
            assert not gg.any()
        clean = []
        for eps in (1e-7, 1e-8, 1e-9):
            fp, tp = run(eps)
            fm, tm = run(-eps)
            if np.array_equal(tp[3], t0[3]) and np.array_equal(tm[3], t0[3]):
                fd = float(np.sum(lam * (fp - fm))) / (2 * eps)
                scale = float(np.sum(np.abs(lam * (fp - fm)))) / (2 * eps)
                clean.append(abs(fd - ad) / scale)
        assert clean, (which, s, "every perturbation crossed a limiter kink")
        assert min(clean) <= 1e-8, (which, s, clean)


def _obs(grid, rng, ncalls, n, outer):
    out = []
    for t in range(n):
        lo, hi = (grid.lz[grid.nr - 2], grid.lz[grid.nr - 1] - 1e-6) if t >= n - outer else (2.6, 5.9)
        out.append({"s": int(rng.integers(len(grid.species))), "call": int(rng.integers(ncalls)),
                    "k": int(rng.integers(8, 28)), "l": 1, "lshell": float(rng.uniform(lo, hi)),
                    "mlt": float(rng.uniform(0, 24)), "log_obs": float(rng.normal(0.0, 1.0))})
    return out


def test_window_gradient_finite_differences(pert):
    wl, o = pert
    g = wl.grid
    ns = len(g.species)
    rng = np.random.Generator(np.random.PCG64(23))
    kps = rng.uniform(2.0, 5.0, 3)
    obs = _obs(g, rng, 3, 24, 8)
    f2 = [np.asfortranarray(a) for a in wl.f2]
    fg = [np.asfortranarray(a) for a in wl.fgeos]
    J, gf, gb = o.window_gradient(f2, fg, wl.dts, kps, obs)
    assert J > 0 and all(np.isfinite(gf[s]).all() for s in range(ns))
    assert np.array_equal(f2[0], np.asfortranarray(wl.f2[0]))  # inputs untouched
    for name, eps_list, make, grad, base in (
            ("F2", (1e-6, 1e-7), lambda: [rng.uniform(-1, 1, f2[s].shape) for s in range(ns)], gf, f2),
            ("FGEOS", (1e-4, 1e-5), lambda: [rng.uniform(-1, 1, fg[s].shape) for s in range(ns)], gb, fg)):
        for _ in range(2):
            r = make()
            ad = sum(float(np.sum(grad[s] * base[s] * r[s])) for s in range(ns))
            errs = []
            for eps in eps_list:
                def J_of(sign):
                    x = [np.asfortranarray(base[s] * (1 + sign * eps * r[s])) for s in range(ns)]
                    return o.window_gradient(x, fg, wl.dts, kps, obs)[0] if name == "F2" else \
                        o.window_gradient(f2, x, wl.dts, kps, obs)[0]
                errs.append(abs((J_of(1) - J_of(-1)) / (2 * eps) - ad) / abs(ad))
            assert min(errs) <= 1e-6, (name, errs)


def test_window_forward_matches_ram_run(pert):
    wl, o = pert
    rng = np.random.Generator(np.random.PCG64(29))
    kps = rng.uniform(2.0, 5.0, 2)
    f2 = [np.asfortranarray(a) for a in wl.f2]
    fg = [np.asfortranarray(a) for a in wl.fgeos]
    obs = [{"s": s, "call": 1, "k": 12, "l": 1, "lshell": 4.1, "mlt": 7.3, "log_obs": 0.0}
           for s in range(len(wl.grid.species))]
    J, _, _ = o.window_gradient(f2, fg, wl.dts, kps, obs)
    chk = [a.copy(order="F") for a in f2]
    for kp in kps:
        res = o.ram_run(chk, fg, wl.dts, kp=kp, want_flux=True)
    Jr = 0.0
    for ob in obs:
        v = sum(w * res["flux"][ob["s"]][i, j, ob["k"], ob["l"]] for i, j, w in pyoracle.obs_cells(wl.grid, ob))
        Jr += math.log(v) ** 2
    assert abs(J - Jr) <= 1e-13 * Jr
