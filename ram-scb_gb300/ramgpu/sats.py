"""Virtual-spacecraft trajectories on the equatorial plane.

Host-side part of the satellite flyer: where each spacecraft is at the
current simulation time.  The time handling follows fly_sats
(src/ModRamSats.f90:500-530): no sample before the first or at/after the
last trajectory time, no sample when the bracketing trajectory points are
more than 600 s apart, otherwise the position is interpolated linearly in
time between the bracketing points in Cartesian coordinates.  The flux
sampling itself runs on the device (RamGpu.fly_sats / ramgpu_fly_sats).
"""
from __future__ import annotations

import bisect
import math
from dataclasses import dataclass

import numpy as np

GM_EARTH = 3.986004418e14   # m^3 s^-2
RE = 6.371e6                # m, src/ModRamConst.f90:14
MAX_GAP_S = 600.0           # src/ModRamSats.f90:514


def _xy(lshell: float, mlt: float):
    ph = mlt * math.pi / 12.0
    return lshell * math.cos(ph), lshell * math.sin(ph)


def _lm(x: float, y: float):
    return math.hypot(x, y), math.fmod(math.atan2(y, x) * 12.0 / math.pi + 24.0, 24.0)


@dataclass
class Track:
    """Trajectory samples: times [s], L-shell [RE] and MLT [h]."""
    times: list
    lshell: list
    mlt: list

    def position(self, t: float):
        """(lshell, mlt) at time t, or None where fly_sats writes no flux."""
        ts = self.times
        if t < ts[0] or t >= ts[-1]:
            return None
        i = max(1, bisect.bisect_left(ts, t))
        if ts[i] - ts[i - 1] > MAX_GAP_S:
            return None
        w = (t - ts[i - 1]) / (ts[i] - ts[i - 1])
        x0, y0 = _xy(self.lshell[i - 1], self.mlt[i - 1])
        x1, y1 = _xy(self.lshell[i], self.mlt[i])
        return _lm(w * (x1 - x0) + x0, w * (y1 - y0) + y0)


@dataclass
class CircularOrbit:
    """Circular equatorial orbit at fixed L-shell; MLT advances by 24 h per
    Kepler period."""
    lshell: float
    mlt0: float
    t0: float
    period: float

    def position(self, t: float):
        return self.lshell, math.fmod(self.mlt0 + 24.0 * (t - self.t0) / self.period, 24.0) % 24.0


def circular_orbit(lshell: float, mlt0: float, t0: float = 0.0) -> CircularOrbit:
    a = lshell * RE
    return CircularOrbit(lshell, mlt0, t0, 2.0 * math.pi * math.sqrt(a ** 3 / GM_EARTH))


def orbit_observations(grid, ncalls: int, dts: float, nobs: int, seed: int, members: int = 1,
                       species=None, lmin=4.0, lmax=6.0, emin_kev=10.0, emax_kev=200.0, pa_bin=1):
    """Observation samples of spacecraft on circular equatorial orbits at
    L = lmin..lmax: each sample is (member, species, ram_run call, energy bin
    nearest to a draw log-uniform in emin..emax keV, pitch-angle bin pa_bin
    (0-based; 1 is PA(2), the bin nearest 90 deg where FLUX is defined),
    position after that call).  log_obs is left 0 for the caller to fill."""
    rng = np.random.Generator(np.random.PCG64(seed))
    nsc = max(1, nobs // 10)
    orbits = [circular_orbit(float(rng.uniform(lmin, lmax)), float(rng.uniform(0.0, 24.0)))
              for _ in range(nsc)]
    ekev = np.asarray(grid.ekev)
    species = species or [list(range(len(grid.species)))] * members
    out = []
    for t in range(nobs):
        m = int(rng.integers(members))
        s = int(rng.choice(species[m]))
        c = int(rng.integers(ncalls))
        e = math.exp(rng.uniform(math.log(emin_kev), math.log(emax_kev)))
        k = int(np.argmin(np.abs(np.log(ekev[1:]) - math.log(e)))) + 1
        lsh, mlt = orbits[t % nsc].position((c + 1) * 2.0 * dts)
        out.append({"member": m, "s": s, "call": c, "k": k, "l": int(pa_bin), "lshell": lsh,
                    "mlt": mlt, "log_obs": 0.0})
    return out
