"""Output products on the CPU: the virtual-spacecraft sampler and the SCB
pressure hand-off of the oracle (known answers), and the host-side
trajectory interpolation."""
import math

import numpy as np
import pytest

import pyoracle
from ramgpu import sats as S
from ramgpu import workload as W


@pytest.fixture(scope="module")
def tiny():
    return W.make_workload("tiny")


def _flux_field(g, fn):
    f = np.zeros((g.nr, g.nt, g.ne, g.npa), order="F")
    for i in range(1, g.nr):
        for j in range(g.nt - 1):
            f[i, j, 1:, 1:] = fn(i, j)
    return f


def test_constant_flux_samples_exactly(tiny):
    g = tiny.grid
    flux = {s: _flux_field(g, lambda i, j: 7.25) for s in range(len(g.species))}
    sf, om = pyoracle.sat_samples(g, flux, [(0, 3.3, 1.0), (0, 4.9, 23.7), (0, 99.0, -3.0)])
    assert np.all(sf[:, :, 0, :] == pyoracle.BAD_DATA) and np.all(sf[:, :, :, 0] == pyoracle.BAD_DATA)
    np.testing.assert_allclose(sf[:, :, 1:, 1:], 7.25, rtol=2e-16, atol=0)
    expect = sum(7.25 * 4.0 * math.pi * g.wmu[l] for l in range(1, g.npa))
    np.testing.assert_allclose(om[:, :, 1:], expect, rtol=1e-14)
    assert np.all(om[:, :, 0] == pyoracle.BAD_DATA)


def test_bilinear_reproduces_linear_field(tiny):
    g = tiny.grid
    lz = np.asarray(g.lz)
    flux = {s: _flux_field(g, lambda i, j: 2.0 + 3.0 * lz[i] + 0.5 * g.phi[j]) for s in range(len(g.species))}
    for lsh, mlt in ((2.9, 2.0), (3.71, 11.5), (5.0, 17.25)):
        sf, _ = pyoracle.sat_samples(g, flux, [(0, lsh, mlt)])
        ph = mlt * math.pi / 12.0
        np.testing.assert_allclose(sf[0, 0, 5, 5], 2.0 + 3.0 * lsh + 0.5 * ph, rtol=1e-13)


def test_nonpositive_corner_is_bad_data(tiny):
    g = tiny.grid
    flux = {s: _flux_field(g, lambda i, j: 1.0) for s in range(len(g.species))}
    cells = pyoracle.obs_cells(g, {"lshell": 3.4, "mlt": 6.0})
    i, j, _ = cells[3]
    flux[1][i, j, 4, 7] = 0.0
    sf, om = pyoracle.sat_samples(g, flux, [(0, 3.4, 6.0)], species_of={0: [1, 2]})
    assert sf[0, 1, 4, 7] == pyoracle.BAD_DATA and sf[0, 1, 4, 8] > 0
    assert np.all(sf[0, 0] == pyoracle.BAD_DATA) and np.all(om[0, 3] == pyoracle.BAD_DATA)
    assert om[0, 1, 4] < om[0, 2, 4]  # the bad bin is left out of the omnidirectional sum


def test_sum_pressure_known_answer():
    pe = {0: np.array([[3.0, 6.0]]), 1: np.array([[9.0, 0.0]])}
    pa = {0: np.array([[3.0, 0.0]]), 1: np.array([[6.0, 3.0]])}
    pall, ppar = pyoracle.sum_pressure(pe, pa, [0, 1])
    np.testing.assert_allclose(pall, [[2.0 + 1.0 + 6.0 + 2.0, 4.0 + 0.0 + 0.0 + 1.0]], rtol=1e-15)
    np.testing.assert_array_equal(ppar, [[9.0, 3.0]])


def test_circular_orbit_track():
    tr = S.circular_orbit(lshell=6.6, mlt0=12.0, t0=0.0)
    assert abs(tr.period - 86164.0) / 86164.0 < 0.02  # geosynchronous at L = 6.6
    l1, m1 = tr.position(tr.period / 4)
    assert l1 == 6.6 and abs(m1 - 18.0) < 1e-9


def test_track_interpolation_and_gaps():
    tr = S.Track(times=[0.0, 60.0, 120.0, 900.0], lshell=[4.0, 4.0, 5.0, 6.0], mlt=[6.0, 6.0, 23.5, 1.0])
    l, m = tr.position(30.0)
    assert abs(l - 4.0) < 1e-12 and abs(m - 6.0) < 1e-12
    # Cartesian interpolation between (4 RE, 06 MLT) and (5 RE, 23.5 MLT)
    x0, y0 = 0.0, 4.0
    x1, y1 = 5.0 * math.cos(23.5 * math.pi / 12), 5.0 * math.sin(23.5 * math.pi / 12)
    l, m = tr.position(90.0)
    xe, ye = 0.5 * (x0 + x1), 0.5 * (y0 + y1)
    assert abs(l - math.hypot(xe, ye)) < 1e-12
    assert abs(m - (math.atan2(ye, xe) * 12 / math.pi) % 24) < 1e-12
    assert tr.position(500.0) is None   # bracketing points 780 s apart: no sample
    assert tr.position(-1.0) is None and tr.position(900.0) is None
    assert tr.position(0.0) == (4.0, 6.0)
