"""GPU frozen-limiter adjoint: finite differences, checkpointing, batching.

J = sum (log flux_model - log flux_obs)^2 over virtual-spacecraft samples
of FLUX (src/ModRamRun.f90:214) at pitch-angle bin L=2, bilinear in
(L-shell, MLT).  The observations come from a seed-perturbed "truth" run.
Finite differences use relative perturbations x0*(1 +- eps*r) small enough
that the recorded branch pattern (digest) is unchanged, so the scheme is
linear between the two runs and the directional derivative must agree with
the adjoint to 1e-6 relative.
"""
import math

import numpy as np
import pytest

from ramgpu import abi, workload as W

pytestmark = pytest.mark.gpu


def interp_flux(g, flux, o):
    """Python mirror of the device observation operator."""
    lz = g.lz
    i0 = 1
    while i0 + 1 < g.nr - 1 and lz[i0 + 1] <= o["lshell"]:
        i0 += 1
    wi = min(1.0, max(0.0, (o["lshell"] - lz[i0]) / (lz[i0 + 1] - lz[i0])))
    ph = math.fmod(o["mlt"] * math.pi / 12.0, 2 * math.pi)
    j0 = min(int(ph / g.dphi), g.nt - 2)
    j1 = 0 if j0 + 1 == g.nt - 1 else j0 + 1
    wj = min(1.0, max(0.0, (ph - g.phi[j0]) / g.dphi))
    v = 0.0
    for a in (0, 1):
        for b in (0, 1):
            w = (wi if a else 1 - wi) * (wj if b else 1 - wj)
            v += w * flux[i0 + a, j1 if b else j0, o["k"], o["l"]]
    return v


def make_case(wl, members, ncalls, nobs, seed, species_lists=None, outer=0):
    g = wl.grid
    rng = np.random.Generator(np.random.PCG64(seed))
    ns = len(g.species)
    species_lists = species_lists or [list(range(ns))] * members
    kp = rng.uniform(2.0, 5.0, size=(ncalls, members))
    obs = []
    for t in range(nobs):
        m = int(rng.integers(members))
        s = int(rng.choice(species_lists[m]))
        # the last `outer` samples sit next to the outer boundary, where FGEOS acts
        lo, hi = (g.lz[g.nr - 2], g.lz[g.nr - 1] - 1e-6) if t >= nobs - outer else (2.6, 5.9)
        obs.append({"member": m, "s": s, "call": int(rng.integers(ncalls)), "k": int(rng.integers(8, 28)),
                    "l": 1, "lshell": float(rng.uniform(lo, hi)), "mlt": float(rng.uniform(0, 24)),
                    "log_obs": 0.0})
    # truth: a seed-perturbed initial state, same drivers
    truth = abi.RamGpu(g, wl.fields, n_members=members)
    for m in range(members):
        truth.set_member_species(m, species_lists[m])
        for s in range(ns):
            truth.upload_f2(m, s, np.asarray(wl.f2[s]) * rng.lognormal(0.0, 0.05, size=wl.f2[s].shape))
            truth.set_boundary(m, s, wl.fgeos[s])
    for c in range(ncalls):
        for m in range(members):
            truth.set_kp(m, kp[c, m])
        truth.ram_run(wl.dts)
        for o in obs:
            if o["call"] == c:
                o["log_obs"] = math.log(interp_flux(g, truth.flux(o["member"], o["s"]), o))
    truth.close()
    model = abi.RamGpu(g, wl.fields, n_members=members)
    for m in range(members):
        model.set_member_species(m, species_lists[m])
        for s in range(ns):
            model.upload_f2(m, s, wl.f2[s])
            model.set_boundary(m, s, wl.fgeos[s])
    return model, kp, obs


@pytest.fixture(scope="module")
def tiny():
    return W.make_workload("tiny")


@pytest.fixture(scope="module")
def case(tiny):
    model, kp, obs = make_case(tiny, 1, 4, 30, seed=11, outer=10)
    J = model.adj_forward(NCALLS, tiny.dts, kp, 2, obs)
    digest = model.adj_digest()
    gf, gb = model.adj_backward()
    return tiny, model, kp, obs, J, digest, gf, gb


def _set_f2(model, wl, scale):
    for s in range(len(wl.grid.species)):
        model.upload_f2(0, s, np.asarray(wl.f2[s]) * scale[s])


NCALLS = 4


def _records(model, ns):
    return np.stack([model.adj_record(c, ns) for c in range(NCALLS)])


def _run(model, wl, kp, obs, f2_scale=None, fg_scale=None):
    """J and the branch record of the window for scaled F2 / FGEOS."""
    ns = len(wl.grid.species)
    for s in range(ns):
        model.upload_f2(0, s, np.asarray(wl.f2[s]) * (1.0 if f2_scale is None else f2_scale[s]))
        model.set_boundary(0, s, wl.fgeos[s] * (1.0 if fg_scale is None else fg_scale[s]))
    J = model.adj_forward(NCALLS, wl.dts, kp, NCALLS, obs)[0]
    return J, _records(model, ns)


def _fd_check(case, directions, make_r, use_f2, seed, eps_list):
    """Central differences along x0*(1 +- eps*r) for each eps in eps_list,
    with the branch record of both runs compared byte by byte against the
    unperturbed run.  Faces whose limiter sits on a kink (R at 1/beta, 1 or
    beta, where adjacent linear pieces give equal values) flip for any eps,
    in numbers proportional to eps; being continuous, they do not bias the
    central difference.  The best eps (truncation vs rounding noise) must
    agree with the adjoint to 1e-6, with kink crossings below 1e-3 of the
    faces."""
    wl, model, kp, obs, J0, dig0, gf, gb = case
    ns = len(wl.grid.species)
    rng = np.random.Generator(np.random.PCG64(seed))
    _, rec0 = _run(model, wl, kp, obs)
    nfaces = rec0.size
    worst, flips_max = 0.0, 0
    try:
        for direction in range(directions):
            r = make_r(rng)
            if use_f2:
                ad = sum(float(np.sum(gf[0, s] * np.asarray(wl.f2[s]) * r[s])) for s in range(ns))
            else:
                ad = sum(float(np.sum(gb[0, s] * wl.fgeos[s] * r[s])) for s in range(ns))
            trials = []
            for eps in eps_list:
                sp = [1.0 + eps * x for x in r]
                sm = [1.0 - eps * x for x in r]
                jp, recp = _run(model, wl, kp, obs, **({"f2_scale": sp} if use_f2 else {"fg_scale": sp}))
                jm, recm = _run(model, wl, kp, obs, **({"f2_scale": sm} if use_f2 else {"fg_scale": sm}))
                flips = int(np.count_nonzero(recp != rec0) + np.count_nonzero(recm != rec0))
                fd = (jp - jm) / (2 * eps)
                trials.append((abs(fd - ad) / abs(ad), flips, eps))
            print(direction, [(f"{e:.0e}", f, f"{er:.2e}") for er, f, e in trials])
            err, flips, eps = min(trials)
            worst = max(worst, err)
            flips_max = max(flips_max, flips)
            assert err <= 1e-6, (direction, eps, err, flips)
            assert flips <= 1e-3 * nfaces, (direction, flips, nfaces)
    finally:
        _run(model, wl, kp, obs)
    print(f"FD {'F2' if use_f2 else 'FGEOS'}: {directions} directions, worst relative error {worst:.2e}, "
          f"most flipped faces {flips_max} of {nfaces}")


def test_gradient_finite_differences_f2(case):
    wl, model, kp, obs, J0, dig0, gf, _ = case
    ns = len(wl.grid.species)
    assert J0[0] > 0 and np.isfinite(gf).all()
    # two identical runs record identical branches
    model.adj_forward(NCALLS, wl.dts, kp, 2, obs)
    assert model.adj_digest() == dig0
    _fd_check(case, 16, lambda rng: [rng.uniform(-1.0, 1.0, size=wl.f2[s].shape) for s in range(ns)],
              True, 5, (1e-6, 1e-7))


def test_gradient_finite_differences_fgeos(case):
    wl, model, kp, obs, J0, dig0, _, gb = case
    ns = len(wl.grid.species)
    assert np.abs(gb).max() > 0
    _fd_check(case, 4, lambda rng: [rng.uniform(-1.0, 1.0, size=wl.fgeos[s].shape) for s in range(ns)],
              False, 6, (1e-4, 1e-5, 1e-6))


@pytest.mark.parametrize("overlap", [False, True])
@pytest.mark.parametrize("k,keep", [(1, 1), (1, 2), (1, 4), (2, 1), (4, 1)])
def test_checkpoint_spacing_and_record_budget(case, k, keep, overlap):
    """Checkpoints every k calls with a record ring of `keep` segments (the
    older segments are recomputed from their checkpoints, on a second stream
    while the next segment is transposed when overlap is on; the ring then
    keeps at least two): the same J and gradients as the default (every
    record kept); records of kept segments are readable, the others are
    not."""
    wl, model, kp, obs, J0, _, gf, gb = case
    g = wl.grid
    ns = len(g.species)
    per_call = 4 * ns * g.nr * g.nt * g.ne * g.npa  # 4 bits per face and sweep, 8 sweeps
    model.set_adj_record_budget(keep * k * per_call)
    model.set_adj_overlap(overlap)
    try:
        _set_f2(model, wl, [1.0] * ns)
        J1 = model.adj_forward(NCALLS, wl.dts, kp, k, obs)
        nseg, nkeep = model.adj_segments()
        least = 2 if overlap and nseg > 1 else 1
        assert nseg == -(-NCALLS // k) and nkeep == min(max(keep, least), nseg)
        for c in range(NCALLS):
            if c // k >= nseg - nkeep:
                assert model.adj_record(c, ns).size > 0
            else:
                with pytest.raises(abi.RamGpuError):
                    model.adj_record(c, ns)
        gf1, gb1 = model.adj_backward()
        assert abs(J1[0] - J0[0]) <= 1e-13 * J0[0]
        assert np.max(np.abs(gf1 - gf)) <= 1e-12 * np.max(np.abs(gf))
        assert np.max(np.abs(gb1 - gb)) <= 1e-12 * np.max(np.abs(gb))
        # after the backward pass F2 is the window's initial state
        assert np.array_equal(model.download_f2(0, 1), np.asfortranarray(wl.f2[1]))
        if nseg > nkeep:  # recomputed segments replaced the kept records
            with pytest.raises(abi.RamGpuError):
                model.adj_record(NCALLS - 1, ns)
            # a second backward pass recomputes everything and agrees (dJ/dFGEOS
            # sums stale-ghost contributions with atomics: rounding order only)
            gf2, gb2 = model.adj_backward()
            assert np.max(np.abs(gf2 - gf1)) <= 1e-13 * np.max(np.abs(gf1))
            assert np.max(np.abs(gb2 - gb1)) <= 1e-13 * np.max(np.abs(gb1))
    finally:
        model.set_adj_record_budget(-1)
        model.set_adj_overlap(True)


@pytest.mark.parametrize("groups", [1, 2, 3])
def test_item_groups_same_window(case, groups):
    """The recording forward, the replay and the transposed sweeps over 1,
    2 or 3 concurrent item groups: the same J, records, digest and dJ/dF2
    bits as the default groups (dJ/dFGEOS to rounding order: it sums with
    atomics)."""
    wl, model, kp, obs, J0, digest0, gf, gb = case
    ns = len(wl.grid.species)
    g0 = model.step_groups()
    model.set_step_groups(groups)
    try:
        _set_f2(model, wl, [1.0] * ns)
        J1 = model.adj_forward(NCALLS, wl.dts, kp, 2, obs)
        assert J1[0] == J0[0]
        assert model.adj_digest() == digest0
        gf1, gb1 = model.adj_backward()
        assert np.array_equal(gf1, gf)
        assert np.max(np.abs(gb1 - gb)) <= 1e-13 * np.max(np.abs(gb))
        _set_f2(model, wl, [1.0] * ns)
        J2 = model.adj_forward(NCALLS, wl.dts, kp, NCALLS, obs)
        end = [model.download_f2(0, s) for s in range(ns)]
        rec = _records(model, ns)
        _set_f2(model, wl, [1.0] * ns)
        Jr = model.adj_replay()
        assert abs(Jr[0] - J2[0]) <= 1e-14 * J2[0]
        for s in range(ns):
            assert np.array_equal(model.download_f2(0, s), end[s])
        model.set_step_groups(g0)
        _set_f2(model, wl, [1.0] * ns)
        assert np.array_equal(model.adj_forward(NCALLS, wl.dts, kp, NCALLS, obs), J2)
        assert np.array_equal(_records(model, ns), rec)
        _set_f2(model, wl, [1.0] * ns)
    finally:
        model.set_step_groups(g0)


def test_drifte_transpose_store_same_bits(case):
    """The first DRIFTE transpose of each call keeps its face coefficients
    for the second (the DRIFTE coefficient store): the same dJ/dF2 bits as
    recomputing them (dJ/dFGEOS to rounding order: it sums with atomics)."""
    wl, model, kp, obs, J0, _, gf, gb = case
    ns = len(wl.grid.species)
    try:
        model.set_coef_store(0)
        _set_f2(model, wl, [1.0] * ns)
        J1 = model.adj_forward(NCALLS, wl.dts, kp, 2, obs)
        gf1, gb1 = model.adj_backward()
        assert J1[0] == J0[0]
        assert np.array_equal(gf1, gf)
        assert np.max(np.abs(gb1 - gb)) <= 1e-13 * np.max(np.abs(gb))
    finally:
        model.set_coef_store(4)
        _set_f2(model, wl, [1.0] * ns)


def test_batched_gradients_equal_solo(tiny):
    lists = [[0, 1, 2, 3], [1, 3], [2]]
    model, kp, obs = make_case(tiny, 3, 3, 24, seed=21, species_lists=lists)
    J = model.adj_forward(3, tiny.dts, kp, 2, obs)
    gf, gb = model.adj_backward()
    for m in range(3):
        solo, _, _ = make_case(tiny, 1, 3, 0, seed=99, species_lists=[lists[m]])
        obs_m = [dict(o, member=0) for o in obs if o["member"] == m]
        Jm = solo.adj_forward(3, tiny.dts, kp[:, m], 2, obs_m)
        gfm, gbm = solo.adj_backward()
        assert abs(Jm[0] - J[m]) <= 1e-13 * max(J[m], 1e-300)
        assert np.max(np.abs(gfm[0] - gf[m])) <= 1e-12 * max(np.max(np.abs(gf[m])), 1e-300)
        assert np.max(np.abs(gbm[0] - gb[m])) <= 1e-12 * max(np.max(np.abs(gb[m])), 1e-300)
        solo.close()


@pytest.mark.parametrize("name", ["tiny_pert", "tiny_pert8"])
def test_gradient_matches_cpu_adjoint(name):
    """GPU adjoint vs the oracle's scalar C adjoint on a non-dipole grid with
    magnetopause-outside cells and stale DRIFTR ghosts: same J, same branch
    records, same gradients (NR = 6, and NR = 8 where the transposed DRIFTR
    reads lambda through the read-only path)."""
    import pyoracle
    wl = W.make_workload(name)
    g = wl.grid
    ns = len(g.species)
    rng = np.random.Generator(np.random.PCG64(41))
    ncalls = 4
    kp = rng.uniform(2.0, 5.0, size=(ncalls, 1))
    obs = []
    for t in range(32):
        lo, hi = (g.lz[g.nr - 2], g.lz[g.nr - 1] - 1e-6) if t >= 20 else (2.6, 5.9)
        obs.append({"member": 0, "s": int(rng.integers(ns)), "call": int(rng.integers(ncalls)),
                    "k": int(rng.integers(8, 28)), "l": int(rng.integers(1, 4)), "lshell": float(rng.uniform(lo, hi)),
                    "mlt": float(rng.uniform(0, 24)), "log_obs": float(rng.normal(0.0, 1.0))})
    model = abi.RamGpu(g, wl.fields, n_members=1)
    try:
        for s in range(ns):
            model.upload_f2(0, s, wl.f2[s])
            model.set_boundary(0, s, wl.fgeos[s])
        Jg = model.adj_forward(ncalls, wl.dts, kp, 2, obs)[0]
        recg = [model.adj_record(c, ns) for c in (2, 3)]
        gf, gb = model.adj_backward()
    finally:
        model.close()
    o = pyoracle.Oracle(g, wl.fields)
    recs, states = [], []
    Jc, cf, cb = o.window_gradient([np.asfortranarray(a) for a in wl.f2], [np.asfortranarray(a) for a in wl.fgeos],
                                   wl.dts, kp[:, 0], obs, records=recs, states=states)
    assert abs(Jg - Jc) <= 1e-12 * Jc, (Jg, Jc)
    mism = sum(int(np.count_nonzero(recg[i][:, :, :] != recs[c])) for i, c in enumerate((2, 3)))
    errs = []
    for s in range(ns):
        ef = np.max(np.abs(gf[0, s] - cf[s])) / np.max(np.abs(cf[s]))
        eb = np.max(np.abs(gb[0, s] - cb[s])) / max(np.max(np.abs(cb[s])), 1e-300)
        print(f"species {s}: dJ/dF2 {ef:.2e}  dJ/dFGEOS {eb:.2e}  record mismatches {mism}")
        errs.append((s, ef, eb))
    assert all(ef <= 1e-9 and eb <= 1e-9 for _, ef, eb in errs), errs
    # Branch codes may differ only where F2 is tiny next to its species'
    # maximum (the mask and clip floors, far tails of the distribution): there
    # the 1e-12-relative differences of the two forward evaluations exceed
    # the cell values themselves and move the limiter ratio or the 1e-27
    # threshold, while the adjoint weight of such faces does not reach the
    # gradient at the tolerance above.
    for i, c in enumerate((2, 3)):
        q, s_, cell = np.nonzero(recg[i] != recs[c])
        if cell.size == 0:
            continue
        st = states[c]
        rel = []
        for qq, ss, cc in zip(q, s_, cell):
            # neighbourhood along every axis within two cells
            idx = [cc + o for o in (-2, -1, 0, 1, 2)]
            for stride in (g.nr, g.nr * g.nt, g.nr * g.nt * g.ne):
                idx += [cc + o * stride for o in (-2, -1, 1, 2)]
            idx = [x for x in idx if 0 <= x < st.shape[1]]
            rel.append(np.min(np.abs(st[ss, idx])) / np.max(np.abs(st[ss])))
        print(f"call {c}: {cell.size} differing codes, local/max F2 at most {max(rel):.1e}")
        assert max(rel) < 1e-6, (c, sorted(rel)[-5:])


def test_autograd_function_matches_c_abi(tiny):
    """The torch.autograd.Function wrapper: same J as ramgpu_adj_forward, and
    backward() delivers the C-ABI gradients scaled by the upstream weights."""
    import torch

    from ramgpu import autograd as A

    model, kp, obs = make_case(tiny, 2, 3, 20, seed=31)
    try:
        J = model.adj_forward(3, tiny.dts, kp, 2, obs)
        gf, gb = model.adj_backward()
        f2, fg = A.device_state(model, tiny.f2, tiny.fgeos, "cuda")
        Jt = A.window_misfit(model, f2, fg, 3, tiny.dts, kp, 2, obs)
        assert np.allclose(Jt.detach().cpu().numpy(), J, rtol=1e-13, atol=0)
        w = torch.tensor([1.0, -2.5], dtype=torch.float64, device="cuda")
        (Jt * w).sum().backward()
        gt, gbt = f2.grad.cpu().numpy(), fg.grad.cpu().numpy()
        for m, wm in enumerate((1.0, -2.5)):
            for s in range(len(tiny.grid.species)):
                ref = wm * gf[m, s]
                assert np.max(np.abs(gt[m, s].transpose(3, 2, 1, 0) - ref)) <= 1e-13 * np.max(np.abs(ref))
                refb = wm * gb[m, s]
                assert np.max(np.abs(gbt[m, s].transpose(2, 1, 0) - refb)) <= 1e-13 * max(np.max(np.abs(refb)), 1e-300)
    finally:
        model.close()


def test_frozen_replay_and_finite_differences(tiny):
    """ramgpu_adj_replay reruns the window with the recorded branches frozen:
    from the same F2 it reproduces the recorded run bit for bit, and since
    the frozen scheme is affine in F2 and FGEOS its J is smooth, so central
    differences agree with the adjoint to 1e-7 whatever
    kinks the unfrozen scheme would cross."""
    model, kp, obs = make_case(tiny, 1, 4, 30, seed=12, outer=10)
    ns = len(tiny.grid.species)
    try:
        J0 = model.adj_forward(4, tiny.dts, kp, 4, obs)[0]
        end = [model.download_f2(0, s) for s in range(ns)]
        gf, gb = model.adj_backward()
        _set_f2(model, tiny, [1.0] * ns)
        Jr = model.adj_replay()[0]
        assert abs(Jr - J0) <= 1e-14 * J0
        for s in range(ns):
            assert np.array_equal(model.download_f2(0, s), end[s])
        rng = np.random.Generator(np.random.PCG64(8))
        for use_f2 in (True, False):
            for _ in range(3):
                shp = [(tiny.f2[s] if use_f2 else tiny.fgeos[s]).shape for s in range(ns)]
                r = [rng.uniform(-1.0, 1.0, size=shp[s]) for s in range(ns)]
                base = tiny.f2 if use_f2 else tiny.fgeos
                grad = gf[0] if use_f2 else gb[0]
                ad = sum(float(np.sum(grad[s] * np.asarray(base[s]) * r[s])) for s in range(ns))

                def central(eps):
                    jj = []
                    for sign in (1.0, -1.0):
                        for s in range(ns):
                            x = np.asarray(base[s]) * (1.0 + sign * eps * r[s])
                            if use_f2:
                                model.upload_f2(0, s, x)
                            else:
                                model.upload_f2(0, s, tiny.f2[s])
                                model.set_boundary(0, s, x)
                        jj.append(model.adj_replay()[0])
                    return (jj[0] - jj[1]) / (2 * eps)

                # J is smooth but not quadratic (log of affine fluxes): Richardson
                # extrapolation of two central differences removes the O(eps^2) term
                fd = (4.0 * central(1e-5) - central(2e-5)) / 3.0
                err = abs(fd - ad) / abs(ad)
                print("frozen FD", "F2" if use_f2 else "FGEOS", f"{err:.2e}")
                assert err <= 1e-7, err
        for s in range(ns):
            model.set_boundary(0, s, tiny.fgeos[s])
    finally:
        model.close()
