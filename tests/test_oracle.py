"""Pinning the CPU oracle without the Fortran reference.

The reference ships no per-routine golden vectors for this path and no
Fortran compiler is available, so the C oracle is pinned by
  * known values of the ARRAYS grid (src/ModRamInit.f90:392-583),
  * exact properties: identity at zero drift, phi periodicity, closed-face
    conservation, the ANISCH L=1 side effect,
  * an independent pure-Python restatement of the sweep line updates of
    src/ModRamDrift.f90 (written from the Fortran text, including DRIFTR's
    F(NR+1:NR+2) persistence across lines), fed the face coefficients of
    the independent NumPy restatement (oracle/ram_numpy.py), never the C
    oracle's: it must agree with the C oracle bit for bit and exercise
    every limiter branch,
  * an independent NumPy evaluation of the CEPARA cross sections.
"""
import dataclasses
import math

import numpy as np
import pytest

from ramgpu import workload as W
import pyoracle
import ram_numpy as RN


@pytest.fixture(scope="module")
def tiny():
    return W.make_workload("tiny")


@pytest.fixture(scope="module")
def tiny_pert():
    return W.make_workload("tiny_pert")


@pytest.fixture(scope="module")
def std_grid():
    return W.arrays(20, 25, 35, 72, species=(W.HYDROGEN,))


# ------------------------------------------------------------------ ARRAYS
def test_arrays_known_values(std_grid):
    g = std_grid
    assert g.we[0] == 3e-2 and g.ekev[0] == 0.1 + 0.5 * 3e-2 and g.ebnd[0] == 0.1 + 3e-2
    assert g.we[1] == 3e-2 * 1.27
    assert g.de[34] == 0.5 * g.we[34] * (1. + 1.27)
    assert g.mu[0] == 0.0 and g.mu[71] == 1.0 and g.wmu[0] == 1.0 / 32
    assert g.pa[47] == 18.7 and g.pa[49] == 16.0 and g.pa[71] == 0.0
    assert list(g.pa[68:72]) == [2.5, 1.5, 1.0, 0.0]
    assert g.dl1 == 0.25 and g.lz[0] == 1.75 and g.lz[20] == 6.75
    assert g.conf1 == ((6.5 + 0.25) / 6.5) ** 2
    assert g.dphi == 2 * math.pi / 24
    assert np.all(np.diff(g.mu) > 0) and np.all(g.wmu > 0)
    assert np.all(np.diff(g.upa) >= 0) and g.upa.min() >= 2
    assert np.array_equal(g.ffactor[:, :, :, 0], g.ffactor[:, :, :, 1])
    # ERNH/EPP (src/ModRamInit.f90:573-577)
    gr = g.grel[0, 5]
    assert g.ernh[0, 5] == g.we[5] * gr / math.sqrt((gr - 1.) * (gr + 1.))


def test_refined_grid_shape():
    g = W.refined_arrays(40, 49, 70, 144, species=(W.HYDROGEN,))
    assert g.mu.size == 144 and g.ekev.size == 70
    assert np.all(np.diff(g.mu) > 0) and np.all(g.wmu > 0) and np.all(g.dmu > 0)
    assert abs(g.ebnd[-1] - 400.0) / 400.0 < 0.2
    assert abs(g.we[0] + g.we[1] - 3e-2) < 1e-15


# ------------------------------------------------------- exact properties
def test_zero_drift_is_identity(tiny):
    """VT = 0, EIP = 0 and J-independent dipole tables make CDriftR vanish up
    to the rounding of the CGR1 sum ((a+b)-a)-b, so DRIFTR leaves F2
    unchanged to 1e-14 of its maximum."""
    wl = tiny
    o = pyoracle.Oracle(wl.grid, wl.fields)
    f2 = np.asfortranarray(wl.f2[1]).copy(order="F")
    before = f2.copy(order="F")
    vt = np.zeros((wl.grid.nr + 1, wl.grid.nt), order="F")
    cd = np.zeros_like(f2, order="F")
    o.sweep("R", 1, f2, vt, wl.dts, fgeos=wl.fgeos[1], cdrift=cd)
    assert np.max(np.abs(cd)) < 1e-14
    assert np.max(np.abs(f2 - before)) <= 1e-14 * np.max(before)


def test_driftp_periodic(tiny):
    wl = tiny
    o = pyoracle.Oracle(wl.grid, wl.fields)
    f2 = np.asfortranarray(wl.f2[1]).copy(order="F")
    o.sweep("P", 1, f2, o.vt_vols(4.0), wl.dts)
    assert np.array_equal(f2[1:, 0], f2[1:, -1])


def test_anisch_side_effect(tiny):
    wl = tiny
    o = pyoracle.Oracle(wl.grid, wl.fields)
    f2 = np.asfortranarray(wl.f2[2]).copy(order="F")
    f2[:, :, :, 0] = -7.0
    pe, pa = o.anisch(2, f2)
    assert np.array_equal(f2[1:, :, 1:, 0], f2[1:, :, 1:, 1])
    assert np.all(f2[0, :, :, 0] == -7.0) and np.all(f2[:, :, 0, 0] == -7.0)
    assert np.all(pe[1:] > 0) and np.all(pa[1:] > 0)


def _closed_species(grid):
    sp = tuple(dataclasses.replace(s, cex_kind=W.CEX_NONE) for s in grid.species)
    return dataclasses.replace(grid, species=sp)


def content_q(g, f2):
    w = g.we[None, None, 1:, None] * g.wmu[None, None, None, 1:-1]
    return float(np.sum(f2[1:, :-1, 1:, 1:-1] * w))


def test_closed_conservation_oracle(tiny):
    wl = tiny
    g = _closed_species(wl.grid)
    o = pyoracle.Oracle(g, wl.fields)
    f2 = [np.asfortranarray(a).copy(order="F") for a in wl.f2]
    q0 = [content_q(g, a) for a in f2]
    for step in range(3):
        o.ram_run(f2, wl.fgeos, 1.0, kp=4.0, closed=True, do_atmol=False)
    for s in range(len(f2)):
        assert abs(content_q(g, f2[s]) - q0[s]) <= 1e-13 * q0[s], s


def test_cex_against_numpy(tiny):
    wl = tiny
    g = wl.grid
    o = pyoracle.Oracle(g, wl.fields)
    coefs = {1: (-18.767, -0.11017, -3.8173e-2, -0.1232, -5.0488e-2),
             2: (-20.789, 0.92316, -0.68017, 0.66153, -0.20998),
             3: (-18.987, -0.10613, -5.4841E-3, -1.6262E-2, -7.0554E-3)}
    for s, sp in enumerate(g.species):
        charge, atlos = o.cepara(s, wl.dts)
        if sp.cex_kind == 0:
            assert np.all(charge == 1.0)
            continue
        x = np.maximum(np.log10(g.ekev), -2.0)
        c = coefs[sp.cex_kind]
        y = c[0] + c[1] * x + c[2] * x ** 2 + c[3] * x ** 3 + c[4] * x ** 4
        sig_v = 10.0 ** y * g.v[s]
        hd = wl.fields.hdns[:g.nr]                              # (I, J, L)
        ref = np.exp(-(sig_v[None, None, :, None] * hd[:, :, None, :] * wl.dts))
        np.testing.assert_allclose(charge[1:, :, 1:, 1:], ref[1:, :, 1:, 1:], rtol=1e-13, atol=0)
        assert np.all(charge[0] == 1.0) and np.all(charge[:, :, 0] == 1.0) and np.all(charge[..., 0] == 1.0)
        taub = 2 * g.rlz[:g.nr, None] / g.v[s][None, :]
        np.testing.assert_allclose(atlos[1:, 1:], np.exp(-wl.dts / taub)[1:, 1:], rtol=1e-14)


# ------------------------------------ independent restatement of the sweeps
BETA = 1.5


def _face(F, I, s, X, C, beta, counts, I1=None, N=None):
    """FBND(I) for the reference's limiter block, literal.  I1 is the right
    cell (I+1, or the periodic J1) and N the upwind index."""
    I1 = I + 1 if I1 is None else I1
    FUP = 0.5 * (F[I] + F[I1] - s * X)
    if abs(X) <= 1.e-27:
        counts["small"] += 1
        return FUP
    if N is None:
        N = I + 1 - s
    R = (F[N] - F[N - 1]) / X
    if R <= 0:
        counts["fup"] += 1
        return FUP
    a, b = min(beta * R, 1.), min(R, beta)
    LIM = max(a, b)
    counts["betaR" if LIM == beta * R and beta * R < 1 else
           "one" if LIM == 1. and R <= 1 else
           "R" if LIM == R and R < beta else "beta"] += 1
    CORR = -0.5 * (C - s) * X
    return FUP + LIM * CORR


def python_driftr(g, f2, cd, fgeos, fnhs, outside, counts):
    """DRIFTR line updates with F(NR+1:NR+2) persisting across lines
    (src/ModRamDrift.f90:130-194); 1-based lists, C from the oracle's CDriftR."""
    NR, NT, NE, NPA = f2.shape
    out = f2.copy(order="F")
    F = [0.0] * (NR + 3)
    for K in range(NE):
        for L in range(NPA):
            for J in range(NT):
                for I in range(NR):
                    F[I + 1] = float(f2[I, J, K, L])
                C = [0.0] + [float(cd[I, J, K, L]) for I in range(NR)]
                sgn = [0] + [(-1 if C[I] < 0 else 1) for I in range(1, NR + 1)]
                FB = [0.0] * (NR + 1)
                if sgn[NR] == 1:
                    FB[1] = 0.
                    FB[NR] = F[NR]
                    UR = NR - 1
                else:
                    FB[1] = F[2]
                    UR = NR
                    if outside[NR - 1, J] == 1:
                        F[NR + 1] = 0.
                        F[NR + 2] = 0.
                    else:
                        F[NR + 1] = fgeos[J, K, L] * g.conf1 * fnhs[NR - 1, J, L]
                        F[NR + 2] = fgeos[J, K, L] * g.conf2 * fnhs[NR - 1, J, L]
                for I in range(2, UR + 1):
                    FB[I] = _face(F, I, sgn[I], F[I + 1] - F[I], C[I], BETA, counts)
                for I in range(2, NR + 1):
                    v = f2[I - 1, J, K, L] - C[I] * FB[I] + C[I - 1] * FB[I - 1]
                    out[I - 1, J, K, L] = 1E-15 if v < 0 else v
    return out


def python_driftmu(g, f2, cd, fnhs, counts):
    """DRIFTMU line updates (src/ModRamDrift.f90:406-467) from CDriftMu."""
    NR, NT, NE, NPA = f2.shape
    out = f2.copy(order="F")
    for K in range(NE):
        for J in range(NT):
            for I in range(1, NR):
                F = [0.0] + [float(f2[I, J, K, L]) for L in range(NPA)]
                F[1] = F[2]
                C = [0.0] + [float(cd[I, J, K, L]) for L in range(NPA)]
                FB = [0.0] * (NPA + 1)
                for L in range(2, NPA - 1):
                    s = -1 if C[L] < 0.0 else 1
                    FB[L] = _face(F, L, s, F[L + 1] - F[L], C[L] / g.dmu[L - 1], BETA, counts)
                C[1] = 0.
                FB[1] = 0.
                FB[NPA - 1] = F[NPA]
                for L in range(2, NPA):
                    v = (f2[I, J, K, L - 1] - C[L] / g.wmu[L - 1] * FB[L]
                         + C[L - 1] / g.wmu[L - 1] * FB[L - 1])
                    out[I, J, K, L - 1] = 1E-15 if v < 0 else v
                out[I, J, K, NPA - 1] = (out[I, J, K, NPA - 2] * fnhs[I, J, NPA - 1] * g.mu[NPA - 1]
                                         / fnhs[I, J, NPA - 2] / g.mu[NPA - 2])
    return out


def python_driftp(g, f2, cd, counts):
    """DRIFTP line updates with the periodic wrap (src/ModRamDrift.f90:225-273)."""
    NR, NT, NE, NPA = f2.shape
    out = f2.copy(order="F")
    for L in range(NPA):
        for K in range(NE):
            for I in range(1, NR):
                F = [0.0] + [float(f2[I, J, K, L]) for J in range(NT)]
                C = [0.0] + [float(cd[I, J, K, L]) for J in range(NT)]
                FB = [0.0] * (NT + 1)
                for J in range(2, NT + 1):
                    J1 = 2 if J == NT else J + 1
                    s = -1 if C[J] < 0 else 1
                    N = J + 1 - s
                    if N > NT:
                        N = N - NT + 1
                    FB[J] = _face(F, J, s, F[J1] - F[J], C[J], BETA, counts, I1=J1, N=N)
                C[1] = C[NT]
                FB[1] = FB[NT]
                for J in range(2, NT + 1):
                    v = f2[I, J - 1, K, L] - C[J] * FB[J] + C[J - 1] * FB[J - 1]
                    out[I, J - 1, K, L] = 1E-15 if v < 0 else v
                out[I, 0, K, L] = out[I, NT - 1, K, L]
    return out


def python_drifte(g, s_idx, f2, cd, counts):
    """DRIFTE line updates with the extrapolated F(0), F(1) and zero F(NE+1:NE+2)
    (src/ModRamDrift.f90:305-370)."""
    NR, NT, NE, NPA = f2.shape
    out = f2.copy(order="F")
    grel = g.grel[s_idx]
    EZERO = g.ekev[0] - g.we[0]
    GRZERO = 1. + EZERO * 1000. * W.Q / g.rmas[s_idx] / W.CS / W.CS
    for J in range(NT):
        for I in range(1, NR):
            for L in range(NPA):
                F = [0.0] * (NE + 3)
                for K in range(NE):
                    F[K + 1] = float(f2[I, J, K, L])
                F[1] = F[2] * grel[0] / grel[1] * math.sqrt((grel[1] ** 2 - 1) / (grel[0] ** 2 - 1))
                F[0] = F[1] * GRZERO / grel[0] * math.sqrt((grel[0] ** 2 - 1) / (GRZERO ** 2 - 1))
                C = [0.0] + [float(cd[I, J, K, L]) for K in range(NE)]
                FB = [0.0] * (NE + 1)
                for K in range(1, NE + 1):
                    s = -1 if C[K] < 0 else 1
                    FB[K] = _face(F, K, s, F[K + 1] - F[K], C[K] / g.de[K - 1], BETA, counts)
                for K in range(2, NE + 1):
                    v = (f2[I, J, K - 1, L] - C[K] / g.we[K - 1] * FB[K]
                         + C[K - 1] / g.we[K - 1] * FB[K - 1])
                    out[I, J, K - 1, L] = 1E-15 if v < 0 else v
    return out


@pytest.mark.parametrize("which", ["P", "E"])
@pytest.mark.parametrize("name", ["tiny", "tiny_pert"])
def test_driftp_drifte_match_independent_restatement(which, name, tiny, tiny_pert):
    wl = {"tiny": tiny, "tiny_pert": tiny_pert}[name]
    g = wl.grid
    o = pyoracle.Oracle(g, wl.fields)
    s = 3
    f2 = np.asfortranarray(wl.f2[s]).copy(order="F")
    cd = np.zeros_like(f2, order="F")
    f_in = f2.copy(order="F")
    vt = RN.vt_vols(g, 5.0)
    o.sweep(which, s, f2, np.asfortranarray(vt), wl.dts, cdrift=cd)
    # the coefficients of the independent restatement, not the oracle's
    cd = (RN.cdrift_p if which == "P" else RN.cdrift_e)(g, RN.Fld(wl.fields), s, wl.dts, vt)[0]
    counts = {k: 0 for k in ("small", "fup", "betaR", "one", "R", "beta")}
    if which == "P":
        ref = python_driftp(g, f_in, cd, counts)
    else:
        ref = python_drifte(g, s, f_in, cd, counts)
    assert np.array_equal(f2[1:], ref[1:])
    assert counts["fup"] > 0 and counts["R"] + counts["one"] + counts["betaR"] + counts["beta"] > 0


@pytest.mark.parametrize("name,kp", [("tiny", 7.0), ("tiny_pert", 4.0)])
def test_driftr_matches_independent_restatement(name, kp, tiny, tiny_pert):
    wl = {"tiny": tiny, "tiny_pert": tiny_pert}[name]
    g = wl.grid
    o = pyoracle.Oracle(g, wl.fields)
    s = 1
    # a potential strong enough that both inflow and outflow lines exist
    vt = RN.vt_vols(g, kp)
    f2 = np.asfortranarray(wl.f2[s]).copy(order="F")
    f_in = f2.copy(order="F")
    o.sweep("R", s, f2, np.asfortranarray(vt), wl.dts, fgeos=wl.fgeos[s])
    cd = RN.cdrift_r(g, RN.Fld(wl.fields), s, wl.dts, vt)[0]
    counts = {k: 0 for k in ("small", "fup", "betaR", "one", "R", "beta")}
    ref = python_driftr(g, f_in, cd, wl.fgeos[s], wl.fields.fnhs, wl.fields.outside, counts)
    assert np.array_equal(f2, ref)
    for k in ("fup", "betaR", "one", "R", "beta"):
        assert counts[k] > 0, counts
    # both boundary cases occur
    assert (cd[-1] < 0).any() and (cd[-1] >= 0).any()


def test_stale_ghost_scenario_exercised(tiny_pert):
    """Lines that are outflow at NR but upwinded from the right at NR-1 read
    F(NR+1) left by the previous inflow line.  With the non-dipole tables
    such lines exist, so the bitwise match of the restatement above covers
    them (with the pure dipole the sign of CDriftR depends on J only)."""
    wl = tiny_pert
    g = wl.grid
    o = pyoracle.Oracle(g, wl.fields)
    vt = o.vt_vols(4.0)
    f2 = np.asfortranarray(wl.f2[1]).copy(order="F")
    cd = np.zeros_like(f2, order="F")
    o.sweep("R", 1, f2, vt, wl.dts, fgeos=wl.fgeos[1], cdrift=cd)
    stale = (cd[-1] >= 0) & (cd[-2] < 0)
    inflow = cd[-1] < 0
    assert stale.any() and inflow.any()


@pytest.mark.parametrize("name", ["tiny", "tiny_pert"])
def test_driftmu_matches_independent_restatement(name, tiny, tiny_pert):
    wl = {"tiny": tiny, "tiny_pert": tiny_pert}[name]
    g = wl.grid
    o = pyoracle.Oracle(g, wl.fields)
    s = 2
    f2 = np.asfortranarray(wl.f2[s]).copy(order="F")
    f_in = f2.copy(order="F")
    vt = RN.vt_vols(g, 4.0)
    o.sweep("MU", s, f2, np.asfortranarray(vt), wl.dts)
    cd = RN.cdrift_mu(g, RN.Fld(wl.fields), s, wl.dts, vt)[0]
    counts = {k: 0 for k in ("small", "fup", "betaR", "one", "R", "beta")}
    ref = python_driftmu(g, f_in, cd, wl.fields.fnhs, counts)
    assert np.array_equal(f2[1:], ref[1:])
    assert counts["fup"] > 0 and counts["R"] + counts["one"] + counts["betaR"] + counts["beta"] > 0


def test_threaded_oracle_is_bitwise_serial():
    """Threading the oracle's independent lines (and nesting them under the
    species threads) leaves every result bit-identical, including DRIFTR's
    stale ghosts on the perturbed grid and the DtDrift minima."""
    wl = W.make_workload("tiny_pert")
    o = pyoracle.Oracle(wl.grid, wl.fields)
    runs = []
    for inner, outer in ((1, 1), (4, 4), (3, 2)):
        pyoracle.set_inner_threads(inner)
        f = [np.asfortranarray(a).copy(order="F") for a in wl.f2]
        outs = [o.ram_run(f, wl.fgeos, wl.dts, kp=3.0 + c, nthreads=outer, want_flux=True) for c in range(2)]
        runs.append((f, outs))
    pyoracle.set_inner_threads(1)
    f0, o0 = runs[0]
    for f, outs in runs[1:]:
        for s in range(len(f)):
            assert np.array_equal(f[s], f0[s])
            assert np.array_equal(outs[1]["ppert"][s], o0[1]["ppert"][s])
            assert np.array_equal(outs[1]["flux"][s], o0[1]["flux"][s])
        assert outs[1]["dts_next"] == o0[1]["dts_next"]


def test_padif_identity_and_conservation():
    """Implicit pitch-angle diffusion (WPADIF / FLCscatter): with D = 0 the
    interior bins are unchanged up to the F2/FACMU*FACMU round trip; with D > 0 the scheme is a flux-form
    tridiagonal solve with zero flux through both ends, so the content
    sum_{L=2..NPA-1} F2*WMU of every line is conserved."""
    wl = W.make_workload("tiny_pert")
    g = wl.grid
    o = pyoracle.Oracle(g, wl.fields)
    f0 = np.asfortranarray(wl.f2[1]).copy(order="F")
    f = f0.copy(order="F")
    o.padif(f, np.zeros_like(f0), wl.dts)
    inner = (slice(1, None), slice(None), slice(1, None), slice(1, g.npa - 1))
    assert np.max(np.abs(f[inner] - f0[inner]) / f0[inner]) <= 4.5e-16  # F2/FACMU*FACMU
    d = W.pa_diffusion(g, wl.fields)
    f = f0.copy(order="F")
    o.padif(f, d, wl.dts)
    w = np.asarray(g.wmu)[1:g.npa - 1]
    c0 = np.sum(f0[1:, :, 1:, 1:g.npa - 1] * w, axis=-1)
    c1 = np.sum(f[1:, :, 1:, 1:g.npa - 1] * w, axis=-1)
    assert np.max(np.abs(c1 - c0) / c0) < 1e-13
    # it does diffuse, and keeps F2 positive
    assert np.max(np.abs(f - f0)) > 1e-3 * np.max(np.abs(f0)) and f.min() >= 0
    # untouched: I = 1 and K = 1
    assert np.array_equal(f[0], f0[0]) and np.array_equal(f[:, :, 0], f0[:, :, 0])


def _dipole_setup(nthe):
    import dataclasses
    wl = W.make_workload("single_h")
    fl = dataclasses.replace(wl.fields, outside=np.zeros_like(wl.fields.outside))
    return wl.grid, pyoracle.Oracle(wl.grid, fl), W.dipole_lines(wl.grid, nthe)


def test_bounce_integrals_dipole_known_answer():
    """computehI's h and I integrals on dipole field lines reproduce Ejiri's
    h(y), I(y) (FUNT, FUNI, src/ModRamFunctions.f90:90-143) to their fit
    accuracy wherever the mirror point lies above the surface."""
    g, o, lines = _dipole_setup(1601)
    h, fi, hd, bm = o.bounce_integrals(lines)
    mu = np.asarray(g.mu)
    beq = lines.b[lines.ieq - 1]     # (NR, NT)
    bend = lines.b[-1]
    checked = 0
    for L in range(3, g.npa - 1):
        # mirror point well above the surface (outside the loss cone); near
        # 90 degrees the bracket spans too few nodes and the reference copies
        # the neighbouring pitch angle, so L >= 4 (1-based) only
        ok = beq / (1.0 - mu[L] ** 2) < 0.8 * bend
        if not ok.any():
            continue
        t, u = W.funt(mu[L]), W.funi(mu[L])
        assert abs(h[:, :, L][ok] / t - 1).max() < 2e-3, L
        assert abs(fi[:, :, L][ok] / u - 1).max() < 2e-3, L
        checked += int(ok.sum())
    assert checked > 0.7 * g.nr * g.nt * (g.npa - 4)
    assert np.all(fi[:, :, 0] == 0.0)  # I at 90 degrees
    # bounce-averaged density lies between the equatorial and the foot values
    assert np.all(hd[:, :, 1:] > 0)


def test_bounce_integrals_exact_for_the_interpolant():
    """The closed-form segment integrals equal adaptive quadrature of the
    reference's integrands (linear interpolant of B and of the density,
    cut off where B >= Bm) far below the reference's 1e-3 tolerance."""
    from scipy import integrate

    g, o, lines = _dipole_setup(101)
    h, fi, hd, bm = o.bounce_integrals(lines)
    chi = lines.chi
    i, j = 7, 4
    B = lines.b[:, i, j]
    n = lines.dens[:, i, j]
    xl, yl, zl = lines.x[:, i, j], lines.y[:, i, j], lines.z[:, i, j]
    length = float(np.sum(np.sqrt(np.diff(xl) ** 2 + np.diff(yl) ** 2 + np.diff(zl) ** 2)))
    e = lines.ieq - 1
    r0 = math.hypot(xl[e], yl[e])
    for L in (5, 17, 33, 48):
        m = bm[i, j, L]
        inside = np.nonzero(B < m)[0]
        # crossings of the interpolant through Bm, as quadrature break points
        pts = []
        for k in range(len(B) - 1):
            if (B[k] - m) * (B[k + 1] - m) < 0:
                pts.append(chi[k] + (chi[k + 1] - chi[k]) * (m - B[k]) / (B[k + 1] - B[k]))
        lo, hi = pts[0], pts[-1]
        bi = lambda c: np.interp(c, chi, B)
        ni = lambda c: np.interp(c, chi, n)
        fh = lambda c: 1.0 / math.sqrt(max(m - bi(c), 1e-300)) if m > bi(c) else 0.0
        fI = lambda c: math.sqrt(m - bi(c)) if m > bi(c) else 0.0
        fd = lambda c: ni(c) * fh(c)
        kw = dict(points=list(chi[inside[0]:inside[-1] + 1]), limit=500, epsabs=0, epsrel=1e-12)
        yh = integrate.quad(fh, lo, hi, **kw)[0]
        yi = integrate.quad(fI, lo, hi, **kw)[0]
        yd = integrate.quad(fd, lo, hi, **kw)[0]
        assert abs((length / (math.pi * 2 * r0)) * yh * math.sqrt(m) / h[i, j, L] - 1) < 1e-9, L
        assert abs((length / (math.pi * r0)) * yi / math.sqrt(m) / fi[i, j, L] - 1) < 1e-9, L
        assert abs((yd / yh) / hd[i, j, L] - 1) < 1e-8, L


def test_compute_hI_fills_dipole_tables():
    """computehI's fill on dipole field lines rebuilds the dipole tables that
    ARRAYS-era RAM computes from Ejiri's fits: FNHS, FNIS and the bin-
    boundary BOUNHS, BOUNIS agree in the trapped range; BNES is the dipole
    equatorial field; row 1 copies row 2; no time derivatives at dthi = 0,
    finite differences of the tables at dthi > 0."""
    g, o, lines = _dipole_setup(401)
    wl = W.make_workload("single_h")
    f0 = {k: np.asarray(getattr(wl.fields, k)) for k in
          ("fnhs", "fnis", "hdns", "bounhs", "bounis", "bnes", "dbdt", "didt", "dibndt", "eir", "eip")}
    out = o.compute_hI(lines, bnormal=3.2e4, dthi=0.0, fields=f0)
    for k in ("fnhs", "fnis", "bounhs", "bounis"):
        # near 90 degrees a narrow mirror bracket makes the reference copy
        # the neighbouring pitch angle (a 1 % effect on the outermost line)
        r = np.abs(out[k][1:, :, 3:45] / f0[k][1:, :, 3:45] - 1)
        assert np.median(r) < 2e-3 and r.max() < 1.5e-2, (k, np.median(r), r.max())
    np.testing.assert_allclose(out["bnes"][1:], f0["bnes"][1:], rtol=1e-12)
    for k in ("fnhs", "fnis", "bounhs", "bounis", "hdns"):
        assert np.array_equal(out[k][0], out[k][1])
    assert not out["didt"].any() and not out["dbdt"].any()
    out2 = o.compute_hI(lines, bnormal=3.2e4, dthi=300.0, fields=f0)
    np.testing.assert_allclose(out2["didt"][1:], (out2["fnis"][1:] - f0["fnis"][1:]) / 300.0, rtol=1e-12,
                               atol=1e-300)
    assert not out2["didt"][0].any()


def _golden():
    import json
    from conftest import ROOT
    return json.loads((ROOT / "tests" / "golden" / "ram_run_tiny.json").read_text())


def test_oracle_matches_golden_fixture():
    """The committed fixture (tests/golden/make_golden.py, made by the
    reference's own ram_run translated by oracle/f90c.py) pins the oracle's
    ram_run on the non-dipole test grid; libm differences between machines
    stay far inside 1e-12."""
    gd = _golden()
    wl = W.make_workload(gd["workload"])
    o = pyoracle.Oracle(wl.grid, wl.fields)
    f2 = [np.asfortranarray(a).copy(order="F") for a in wl.f2]
    out = o.ram_run(f2, wl.fgeos, gd["dts"], kp=gd["kp"], want_flux=True)
    assert abs(out["dts_next"] - gd["dts_next"]) <= 1e-12 * gd["dts_next"]
    for s, sd in enumerate(gd["species"]):
        assert abs(np.sum(f2[s]) - sd["sum"]) <= 1e-12 * abs(sd["sum"])
        scale = max(abs(v) for _, v in sd["cells"])
        for c, v in sd["cells"]:
            assert abs(f2[s][tuple(c)] - v) <= 1e-12 * scale
        for key in ("ppert", "ppart"):
            sc = max(abs(v) for _, v in sd[key])
            for c, v in sd[key]:
                assert abs(out[key][s][tuple(c)] - v) <= 1e-12 * sc


def test_oracle_follows_reference_ramp_fixture():
    """Three successive calls along a Kp ramp on the perturbed 8x9x35x72
    grid against the reference's own results (tests/golden/ram_run_ramp.json):
    sums, sampled cells, moments, FLUX, DtsNext and the SUMRC losses."""
    import json
    from conftest import ROOT
    gd = json.loads((ROOT / "tests" / "golden" / "ram_run_ramp.json").read_text())
    wl = W.make_workload(gd["workload"])
    o = pyoracle.Oracle(wl.grid, wl.fields)
    f2 = [np.asfortranarray(a).copy(order="F") for a in wl.f2]
    losses = {s: (0.0, 0.0, 0.0, 0.0) for s in range(len(wl.grid.species))}
    for call in gd["calls"]:
        out = o.ram_run(f2, wl.fgeos, gd["dts"], kp=call["kp"], want_flux=True, losses=losses)
        losses = out["losses"]
        assert abs(out["dts_next"] - call["dts_next"]) <= 1e-12 * call["dts_next"]
        for s, sd in enumerate(call["species"]):
            assert abs(np.sum(f2[s]) - sd["sum"]) <= 1e-12 * abs(sd["sum"])
            scale = max(abs(v) for _, v in sd["cells"])
            for c, v in sd["cells"]:
                assert abs(f2[s][tuple(c)] - v) <= 1e-12 * scale
            for key in ("ppert", "ppart", "flux"):
                sc = max(abs(v) for _, v in sd[key])
                for c, v in sd[key]:
                    assert abs(out[key][s][tuple(c)] - v) <= 1e-12 * sc
            for a, b in zip(losses[s], call["losses"][s]):
                assert abs(a - b) <= 1e-12 * max(abs(b), 1e-300)
