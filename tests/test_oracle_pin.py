"""The C oracle against a second, independent restatement of the reference.

oracle/ram_numpy.py restates, in vectorised NumPy and straight from the
Fortran text, every formula of the path: the VOLS potential
(src/ModRamRun.f90:45-54), DRIFTPARA (src/ModRamDrift.f90:36-88), the face
coefficients and CFL limits of DRIFTR/DRIFTP/DRIFTE/DRIFTMU (CR/CGR :117-146,
CDriftP :232-239, CDriftE :314-342, CDriftMu :406-433), their line updates,
CEPARA and ATMOL (src/ModRamLoss.f90:34-87,162-167,485-507), the ram_run
sequence and tail (src/ModRamRun.f90:64-222) and ANISCH's moment block
(:343-415).  It takes no array from the C oracle.  Where the reference's
arithmetic uses no library function the two must agree bit for bit; SIN,
LOG10, EXP and real powers may differ by an ulp between libm and NumPy, so
those results are compared at 1e-15 relative max-norm.
"""
import dataclasses

import numpy as np
import pytest

from ramgpu import workload as W
import pyoracle
import ram_numpy as RN


def rel(a, b):
    den = np.max(np.abs(b))
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / (den if den > 0 else 1.0))


_WL = {}


def wl_of(name):
    if name not in _WL:
        _WL[name] = W.make_workload(name)
    return _WL[name]


GRIDS = ["tiny", "tiny_pert", "single_h"]


@pytest.mark.parametrize("name", GRIDS)
@pytest.mark.parametrize("kp", [1.0, 3.0, 6.0])
def test_vols_potential(name, kp):
    wl = wl_of(name)
    o = pyoracle.Oracle(wl.grid, wl.fields)
    assert rel(RN.vt_vols(wl.grid, kp), o.vt_vols(kp)) <= 1e-15


@pytest.mark.parametrize("name", GRIDS)
@pytest.mark.parametrize("dts", [5.0, 1.0])
def test_driftpara_bitwise(name, dts):
    wl = wl_of(name)
    g = wl.grid
    o = pyoracle.Oracle(g, wl.fields)
    for s in range(len(g.species)):
        c, n = o.driftpara(s, dts), RN.driftpara(g, s, dts)
        for k in ("vr", "p1", "p2", "mudot", "edot"):
            assert np.array_equal(c[k], n[k]), (s, k)


@pytest.mark.parametrize("which", ["R", "P", "E", "MU"])
@pytest.mark.parametrize("name", GRIDS)
@pytest.mark.parametrize("kp", [1.0, 3.0, 6.0])
def test_sweep_coefficients_and_update_bitwise(which, name, kp):
    """Face coefficients CDrift*, the CFL limit DtDrift* and the swept F2 of
    every species equal the C oracle bit for bit (the same VT goes to both)."""
    wl = wl_of(name)
    g = wl.grid
    o = pyoracle.Oracle(g, wl.fields)
    f = RN.Fld(wl.fields)
    vt = RN.vt_vols(g, kp)
    species = range(len(g.species)) if name != "single_h" or which != "R" else [0]
    for s in species:
        f2 = np.asfortranarray(wl.f2[s]).copy(order="F")
        cd = np.zeros_like(f2, order="F")
        dt_c = o.sweep(which, s, f2, np.asfortranarray(vt), wl.dts, fgeos=wl.fgeos[s], cdrift=cd)
        x = np.asarray(wl.f2[s], dtype=np.float64)
        if which == "R":
            y, c, dt = RN.drift_r(g, f, s, x, wl.fgeos[s], wl.dts, vt)
        else:
            y, c, dt = {"P": RN.drift_p, "E": RN.drift_e, "MU": RN.drift_mu}[which](g, f, s, x, wl.dts, vt)
        assert np.array_equal(c, cd), (s, rel(c, cd))
        assert dt == dt_c, (s, dt, dt_c)
        assert np.array_equal(y, f2), (s, rel(y, f2))


@pytest.mark.parametrize("name", GRIDS)
def test_cepara_atlos(name):
    """CHARGE and ATLOS through LOG10, 10.**Y and EXP: within an ulp or two."""
    wl = wl_of(name)
    g = wl.grid
    o = pyoracle.Oracle(g, wl.fields)
    f = RN.Fld(wl.fields)
    for s in range(len(g.species)):
        ch, at = o.cepara(s, wl.dts)
        chn, atn = RN.cepara(g, f, s, wl.dts)
        assert rel(chn[1:, :, 1:, 1:], ch[1:, :, 1:, 1:]) <= 1e-15, s
        assert rel(atn[1:, 1:], at[1:, 1:]) <= 1e-15, s
        if g.species[s].cex_kind == W.CEX_NONE:
            assert np.all(ch == 1.0) and np.all(chn == 1.0)


@pytest.mark.parametrize("name", GRIDS)
def test_anisch_and_flux_bitwise(name):
    """PPERT, PPART, the L=1 side effect and FLUX, bit for bit."""
    wl = wl_of(name)
    g = wl.grid
    o = pyoracle.Oracle(g, wl.fields)
    f = RN.Fld(wl.fields)
    for s in range(len(g.species)):
        x = np.asfortranarray(wl.f2[s]).copy(order="F")
        pe, pa = o.anisch(s, x)
        y, pen, pan = RN.anisch(g, f, s, np.asarray(wl.f2[s], dtype=np.float64))
        assert np.array_equal(pe, pen) and np.array_equal(pa, pan) and np.array_equal(x, y), s
        assert np.array_equal(o.flux(s, x), RN.flux(g, f, s, y)), s


def _no_cex(g):
    return dataclasses.replace(g, species=tuple(dataclasses.replace(s, cex_kind=W.CEX_NONE) for s in g.species))


@pytest.mark.parametrize("name", GRIDS)
@pytest.mark.parametrize("kp", [1.0, 3.0, 6.0])
def test_ram_run_without_library_functions_bitwise(name, kp):
    """The whole ram_run call (sweeps both ways, periodic copy, mask,
    DtsNext, ANISCH, FLUX) with the CEX and ATMOL factors off, so that no
    library function enters: F2, moments, FLUX and DtsNext bit for bit."""
    wl = wl_of(name)
    g = _no_cex(wl.grid)
    o = pyoracle.Oracle(g, wl.fields)
    vt = RN.vt_vols(g, kp)
    ref = [np.asfortranarray(a).copy(order="F") for a in wl.f2]
    out = o.ram_run(ref, wl.fgeos, wl.dts, vt=np.asfortranarray(vt), want_flux=True, do_atmol=False)
    nn = RN.ram_run(g, wl.fields, [np.asarray(a, dtype=np.float64) for a in wl.f2], wl.fgeos, wl.dts, vt=vt,
                    do_atmol=False)
    assert nn["dts_next"] == out["dts_next"]
    for s in range(len(g.species)):
        assert np.array_equal(nn["f2"][s], ref[s]), (s, rel(nn["f2"][s], ref[s]))
        assert np.array_equal(nn["ppert"][s], out["ppert"][s]) and np.array_equal(nn["ppart"][s], out["ppart"][s])
        assert np.array_equal(nn["flux"][s], out["flux"][s])


@pytest.mark.parametrize("name", GRIDS)
@pytest.mark.parametrize("kp", [1.0, 3.0, 6.0])
def test_ram_run_full(name, kp):
    """The reference's ram_run with charge exchange and atmospheric loss:
    F2, moments and FLUX within 1e-15 relative max-norm (the loss factors
    pass through EXP and real powers), DtsNext bit for bit."""
    wl = wl_of(name)
    g = wl.grid
    o = pyoracle.Oracle(g, wl.fields)
    ref = [np.asfortranarray(a).copy(order="F") for a in wl.f2]
    vt = RN.vt_vols(g, kp)
    out = o.ram_run(ref, wl.fgeos, wl.dts, vt=np.asfortranarray(vt), want_flux=True)
    nn = RN.ram_run(g, wl.fields, [np.asarray(a, dtype=np.float64) for a in wl.f2], wl.fgeos, wl.dts, vt=vt)
    assert nn["dts_next"] == out["dts_next"]
    for s in range(len(g.species)):
        assert rel(nn["f2"][s], ref[s]) <= 1e-15, s
        assert rel(nn["ppert"][s], out["ppert"][s]) <= 1e-15 and rel(nn["ppart"][s], out["ppart"][s]) <= 1e-15
        assert rel(nn["flux"][s], out["flux"][s]) <= 1e-15
