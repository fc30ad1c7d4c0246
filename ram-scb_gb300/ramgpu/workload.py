"""Synthetic inputs for the RAM kinetic step (grid, dipole fields, state).

No dataset is involved: every input is generated from the grid formulas of
the reference and a seeded NumPy PCG64 generator.

* ``arrays`` restates ARRAYS (src/ModRamInit.f90:364-587) for the standard
  grid (the reference's hard-wired energy series WE(1)=3E-2, RW=1.27 for
  EnergyMin=0.1 keV and its NPA/=90 pitch-angle construction with the
  loss-cone points CONE(IC)), keeping its loop order and literals.
* ``refined_arrays`` is a generalised generator for grids ARRAYS cannot
  build (NE=70 over 0.1-400 keV, NPA=144): the energy series is the same
  geometric series with ratio sqrt(1.27), the mu grid bisects the standard
  one.  The kernels and the oracle take grid arrays as inputs and never
  regenerate them.
* ``dipole_fields`` follows the DIPL pattern of src/ModRamIO.f90:458-466:
  FNHS=FUNT(MU), FNIS=FUNI(MU), BOUNHS/BOUNIS at cosd(PAbn), BNES=0.32/L^3
  [G -> T], zero time derivatives and electric fields, everything inside the
  magnetopause; HDNS is a Rairden-profile geocorona (src/ModRamScb.f90:366-369)
  with a pitch-angle factor and a seeded 10 % lognormal perturbation.
* ``initial_f2`` and ``boundary_fgeos`` build F2 = flux*FFACTOR*FNHS (the
  inverse of src/ModRamRun.f90:214) from a kappa distribution, and FGEOS as
  GEOSB does (src/ModRamBoundary.f90:288-295).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

# src/ModRamConst.f90:13-23 (doubles under -fdefault-real-8)
RE = 6.371e6
HMIN = 2e5
MP = 1.673e-27
Q = 1.602e-19
CS = 2.998e8
PI = 3.1415926535897932384626433832795

CEX_NONE, CEX_HYDROGEN, CEX_HELIUM1, CEX_OXYGEN1 = 0, 1, 2, 3


@dataclass(frozen=True)
class Species:
    name: str
    code: str
    mass: float      # multiple of the proton mass
    charge: int
    cex_kind: int


# src/ModRamSpecies.f90:37-138 (the four species the configurations use)
ELECTRON = Species("Electron", "_e", 5.4462e-4, -1, CEX_NONE)
HYDROGEN = Species("Hydrogen", "_H", 1.0, 1, CEX_HYDROGEN)
HELIUM1 = Species("HeliumP1", "He", 4.0, 1, CEX_HELIUM1)
OXYGEN1 = Species("OxygenP1", "_O", 16.0, 1, CEX_OXYGEN1)
SPECIES = {"e": ELECTRON, "H": HYDROGEN, "He": HELIUM1, "O": OXYGEN1}


def _asind(x):
    return 180.0 / PI * math.asin(x)


def _acosd(x):
    return 180.0 / PI * math.acos(x)


def _cosd(x):
    return math.cos(PI / 180.0 * x)


def _sind(x):
    return math.sin(PI / 180.0 * x)


@dataclass
class Grid:
    nr: int
    nt: int
    ne: int
    npa: int
    species: tuple
    dl1: float
    mdr: float
    dphi: float
    conf1: float
    conf2: float
    lz: np.ndarray
    rlz: np.ndarray
    phi: np.ndarray
    mlt: np.ndarray
    ekev: np.ndarray
    ebnd: np.ndarray
    we: np.ndarray
    de: np.ndarray
    mu: np.ndarray
    dmu: np.ndarray
    wmu: np.ndarray
    pa: np.ndarray
    pabn: np.ndarray
    upa: np.ndarray
    cone: np.ndarray
    rmas: np.ndarray          # (NS)
    grel: np.ndarray          # (NS, NE)
    grbnd: np.ndarray
    v: np.ndarray
    vbnd: np.ndarray
    ernh: np.ndarray
    epp: np.ndarray
    ffactor: np.ndarray       # (NS, NR, NE, NPA), C order == reference index order
    extra: dict = field(default_factory=dict)

    @property
    def ncell(self) -> int:
        return self.nr * self.nt * self.ne * self.npa


def _energy_and_species(ne, we1, rw, elb, species):
    ns = len(species)
    we = np.zeros(ne); ebnd = np.zeros(ne); de = np.zeros(ne); ekev = np.zeros(ne)
    rmas = np.array([MP * sp.mass for sp in species])
    grel = np.zeros((ns, ne)); v = np.zeros((ns, ne)); grbnd = np.zeros((ns, ne)); vbnd = np.zeros((ns, ne))
    we[0] = we1
    ekev[0] = elb + 0.5 * we[0]
    ebnd[0] = elb + we[0]
    for s in range(ns):
        grel[s, 0] = 1. + ekev[0] * 1000. * Q / rmas[s] / CS / CS
        v[s, 0] = CS * math.sqrt(grel[s, 0] * grel[s, 0] - 1.) / grel[s, 0]
        grbnd[s, 0] = 1. + ebnd[0] * 1000. * Q / rmas[s] / CS / CS
        vbnd[s, 0] = CS * math.sqrt(grbnd[s, 0] * grbnd[s, 0] - 1.) / grbnd[s, 0]
    for k in range(ne - 1):  # K = k+1
        we[k + 1] = we[k] * rw
        ebnd[k + 1] = ebnd[k] + we[k + 1]
        de[k] = 0.5 * (we[k] + we[k + 1])
        ekev[k + 1] = ekev[k] + de[k]
        for s in range(ns):
            grel[s, k + 1] = 1. + ekev[k + 1] * 1000. * Q / rmas[s] / CS / CS
            v[s, k + 1] = CS * math.sqrt(grel[s, k + 1] * grel[s, k + 1] - 1.) / grel[s, k + 1]
            grbnd[s, k + 1] = 1. + ebnd[k + 1] * 1000. * Q / rmas[s] / CS / CS
            vbnd[s, k + 1] = CS * math.sqrt(grbnd[s, k + 1] * grbnd[s, k + 1] - 1.) / grbnd[s, k + 1]
    de[ne - 1] = 0.5 * we[ne - 1] * (1. + rw)
    return we, ebnd, de, ekev, rmas, grel, v, grbnd, vbnd


def _finish(nr, nt, ne, npa, species, dl1, lz, rlz, mu, dmu, wmu, pa, pabn, cone,
            we, ebnd, de, ekev, rmas, grel, v, grbnd, vbnd, extra):
    ns = len(species)
    mdr = dl1 * RE
    dphi = 2. * PI / (nt - 1)
    phi = np.array([j * dphi for j in range(nt)])
    mlt = phi * 12. / PI
    # UPA(I): smallest L with PA(L) <= CONE(I) (src/ModRamInit.f90:539-544)
    upa = np.zeros(nr)
    for i in range(nr):
        upa[i] = npa
        for l in range(npa - 1, -1, -1):
            if pa[l] <= cone[i]:
                upa[i] = l + 1
    ffactor = np.zeros((ns, nr, ne, npa))
    for s in range(ns):
        for i in range(nr):
            for k in range(ne):
                g = grel[s, k]
                for l in range(1, npa):
                    ffactor[s, i, k, l] = lz[i] * lz[i] * g / math.sqrt(g * g - 1.) * mu[l]
                ffactor[s, i, k, 0] = ffactor[s, i, k, 1]
    ernh = np.zeros((ns, ne)); epp = np.zeros((ns, ne))
    for s in range(ns):
        for k in range(ne):
            g = grel[s, k]
            ernh[s, k] = we[k] * g / math.sqrt((g - 1.) * (g + 1.))
            epp[s, k] = ernh[s, k] * ekev[k]
    t1 = (lz[nr - 1] + dl1) / lz[nr - 1]
    t2 = (lz[nr - 1] + 2. * dl1) / lz[nr - 1]
    return Grid(nr=nr, nt=nt, ne=ne, npa=npa, species=tuple(species), dl1=dl1, mdr=mdr, dphi=dphi,
                conf1=t1 * t1, conf2=t2 * t2, lz=lz, rlz=rlz, phi=phi, mlt=mlt, ekev=ekev, ebnd=ebnd,
                we=we, de=de, mu=mu, dmu=dmu, wmu=wmu, pa=pa, pabn=pabn, upa=upa, cone=cone, rmas=rmas,
                grel=grel, grbnd=grbnd, v=v, vbnd=vbnd, ernh=ernh, epp=epp, ffactor=ffactor, extra=extra)


def _radial(nr, dl1, rmin):
    lz = np.array([rmin + i * dl1 for i in range(nr + 1)])
    rlz = RE * lz
    cone = np.zeros(nr + 4)
    for i in range(nr):
        clc = (RE + HMIN) / rlz[i]
        cone[i] = _asind(math.sqrt(clc * clc * clc / math.sqrt(4. - 3. * clc)))
    cone[nr:nr + 4] = [2.5, 1.5, 1., 0.]
    return lz, rlz, cone


def arrays(nr=20, nt=25, ne=35, npa=72, species=(HYDROGEN,), energy_min=0.1,
           radius_min=1.75, radius_max=6.5, mu_grid_nr=None) -> Grid:
    """ARRAYS for the standard grid (src/ModRamInit.f90:392-583).

    mu_grid_nr: radial size whose loss-cone points CONE(IC) build the mu grid
    (default nr).  ARRAYS steps IC by (NR-1)/19, so it only builds a valid
    mu grid for NR >= 20; small test grids borrow the NR=20 mu grid."""
    if npa == 90:
        raise ValueError("only the NPA/=90 pitch-angle branch is restated")
    if npa < 50 or nr < 2:
        raise ValueError("ARRAYS' hard-wired mu grid needs NPA >= 50")
    dl1 = (radius_max - radius_min) / (nr - 1)
    lz, rlz, cone = _radial(nr, dl1, radius_min)
    mnr = nr if mu_grid_nr is None else mu_grid_nr
    if mnr < 20:
        raise ValueError("ARRAYS builds a valid mu grid only for NR >= 20")
    cone_mu = cone if mnr == nr else _radial(mnr, (radius_max - radius_min) / (mnr - 1), radius_min)[2]
    if abs(energy_min - 0.01) <= 1e-9:
        we1, rw = 2.8e-3, 1.36
    elif abs(energy_min - 0.1) <= 1e-9:
        we1, rw = 3e-2, 1.27
    elif abs(energy_min - 1.0) <= 1e-9:
        we1, rw = 0.31, 1.16
    else:
        raise ValueError("EnergyMin must be 0.01, 0.1 or 1.0 keV")
    en = _energy_and_species(ne, we1, rw, energy_min, species)
    # pitch-angle grid, NPA /= 90 branch (src/ModRamInit.f90:494-534)
    pa = np.zeros(npa); mu = np.zeros(npa); wmu = np.zeros(npa); dmu = np.zeros(npa); pabn = np.zeros(npa)
    pa[0] = 90.; mu[0] = 0.; pa[npa - 1] = 0.; mu[npa - 1] = 1.
    rwu = 0.98
    wmu[0] = (mu[npa - 1] - mu[0]) / 32
    for L in range(1, 47):
        wmu[L] = wmu[L - 1] * rwu
        dmu[L - 1] = 0.5 * (wmu[L - 1] + wmu[L])
        mu[L] = mu[L - 1] + dmu[L - 1]
        pa[L] = _acosd(mu[L])
    pa[47] = 18.7
    mu[47] = _cosd(pa[47])
    dmu[46] = mu[47] - mu[46]
    ic = 2
    for L in range(48, npa):  # Fortran L = 48..NPA-1
        pa[L] = cone_mu[ic - 1]
        if L == 49:
            pa[49] = 16.
        else:
            if ic < mnr:
                ic = ic + (mnr - 1) // 19
            else:
                ic = ic + 1
        mu[L] = _cosd(pa[L])
        dmu[L - 1] = mu[L] - mu[L - 1]
        wmu[L - 1] = 2. * (dmu[L - 2] - 0.5 * wmu[L - 2])
        if L > 55:
            wmu[L - 1] = 0.5 * (dmu[L - 1] + dmu[L - 2])
    dmu[npa - 1] = dmu[npa - 2]
    wmu[npa - 1] = dmu[npa - 2]
    for L in range(npa - 1):
        pabn[L] = _acosd(mu[L] + 0.5 * wmu[L])
    pabn[npa - 1] = 0.
    return _finish(nr, nt, ne, npa, species, dl1, lz, rlz, mu, dmu, wmu, pa, pabn, cone, *en,
                   extra={"generator": "ARRAYS", "energy_min": energy_min})


def refined_arrays(nr=40, nt=49, ne=70, npa=144, species=(HYDROGEN,), dl1=0.125,
                   radius_min=1.75, energy_min=0.1) -> Grid:
    """Generalised grid for sizes ARRAYS cannot build (NE=70, NPA=144)."""
    if npa != 144 or ne % 35 != 0:
        raise ValueError("refined_arrays builds the NE=35*r, NPA=144 grid only")
    lz, rlz, cone = _radial(nr, dl1, radius_min)
    r = ne // 35
    rw = 1.27 ** (1.0 / r)
    we1 = 3e-2 * (rw - 1.0) / (rw ** r - 1.0)   # the first r sub-bins tile WE(1)=3E-2
    en = _energy_and_species(ne, we1, rw, energy_min, species)
    base = arrays(20, 25, 35, 72, species=species[:1])
    bm = base.mu
    mu = [bm[0]]
    for L in range(71):
        mu.append(0.5 * (bm[L] + bm[L + 1]))
        mu.append(bm[L + 1])
    mu.insert(len(mu) - 1, 0.5 * (mu[-2] + mu[-1]))
    mu = np.array(mu)
    assert mu.size == npa
    dmu = np.zeros(npa); wmu = np.zeros(npa); pa = np.zeros(npa); pabn = np.zeros(npa)
    for L in range(npa - 1):
        dmu[L] = mu[L + 1] - mu[L]
    dmu[npa - 1] = dmu[npa - 2]
    wmu[0] = dmu[0]
    for L in range(1, npa - 1):
        wmu[L] = 0.5 * (dmu[L - 1] + dmu[L])
    wmu[npa - 1] = dmu[npa - 2]
    for L in range(npa):
        pa[L] = _acosd(min(1.0, mu[L]))
    for L in range(npa - 1):
        pabn[L] = _acosd(min(1.0, mu[L] + 0.5 * wmu[L]))
    pabn[npa - 1] = 0.
    return _finish(nr, nt, ne, npa, species, dl1, lz, rlz, mu, dmu, wmu, pa, pabn, cone, *en,
                   extra={"generator": "refined", "energy_min": energy_min})


# ------------------------------------------------------------------ dipole
def funt(x):
    """FUNT, Ejiri 1978 h(y) (src/ModRamFunctions.f90:90-114)."""
    y = math.sqrt(1 - x * x)
    alpha = 1. + math.log(2. + math.sqrt(3.)) / 2. / math.sqrt(3.)
    beta = alpha / 2. - PI * math.sqrt(2.) / 12.
    a1, a2, a3, a4 = 0.055, -0.037, -0.074, 0.056
    return (alpha - beta * (y + math.sqrt(y)) + a1 * y ** (1. / 3.) + a2 * y ** (2. / 3.) + a3 * y
            + a4 * y ** (4. / 3.))


def funi(x):
    """FUNI, Ejiri 1978 I(y) (src/ModRamFunctions.f90:117-143)."""
    ylog = 0.0
    y = math.sqrt(1 - x * x)
    if y > 0:
        ylog = math.log(y)
    alpha = 1. + math.log(2. + math.sqrt(3.)) / 2. / math.sqrt(3.)
    beta = alpha / 2. - PI * math.sqrt(2.) / 12.
    a1, a2, a3, a4 = 0.055, -0.037, -0.074, 0.056
    return (2. * alpha * (1. - y) + 2. * beta * y * ylog + 4. * beta * (y - math.sqrt(y))
            + 3. * a1 * (y ** (1. / 3.) - y) + 6. * a2 * (y ** (2. / 3.) - y) + 6. * a4 * (y - y ** (4. / 3.))
            - 2. * a3 * y * ylog)


@dataclass
class Fields:
    """Field tables in C order with the reference's index order
    (I, J, L) / (I, J); transposed to Fortran order at the ABI."""
    fnhs: np.ndarray
    fnis: np.ndarray
    bounhs: np.ndarray
    bounis: np.ndarray
    hdns: np.ndarray
    didt: np.ndarray
    dibndt: np.ndarray
    bnes: np.ndarray
    dbdt: np.ndarray
    eir: np.ndarray
    eip: np.ndarray
    outside: np.ndarray  # int (NR, NT)


def rairden(r):
    """Rairden geocorona density [m^-3] at radial distance r [RE]."""
    return 10 ** (13.326 - 3.6908 * r + 1.1362 * r ** 2 - 0.16984 * r ** 3 + 0.009553 * r ** 4)


def dipole_fields(g: Grid, seed: int = 1234, hdns_sigma: float = 0.1) -> Fields:
    nf, nt, npa = g.nr + 1, g.nt, g.npa
    fh = np.array([funt(m) for m in g.mu])
    fi = np.array([funi(m) for m in g.mu])
    bh = np.array([funt(_cosd(p)) for p in g.pabn])
    bi = np.array([funi(_cosd(p)) for p in g.pabn])
    shape3 = (nf, nt, npa)
    fnhs = np.broadcast_to(fh, shape3).copy()
    fnis = np.broadcast_to(fi, shape3).copy()
    bounhs = np.broadcast_to(bh, shape3).copy()
    bounis = np.broadcast_to(bi, shape3).copy()
    bnes = np.array([[0.32 / g.lz[i] ** 3 / 1.e4 for _ in range(nt)] for i in range(nf)])
    rng = np.random.Generator(np.random.PCG64(seed))
    pert = rng.lognormal(0.0, hdns_sigma, size=shape3)
    hd = np.array([rairden(g.lz[i]) for i in range(nf)])
    hdns = hd[:, None, None] * (1.0 + 4.0 * g.mu[None, None, :] ** 2) * pert
    hdns[:, nt - 1, :] = hdns[:, 0, :]
    hdns[0] = hdns[1]
    z3 = np.zeros(shape3)
    z2 = np.zeros((nf, nt))
    return Fields(fnhs=fnhs, fnis=fnis, bounhs=bounhs, bounis=bounis, hdns=hdns, didt=z3.copy(),
                  dibndt=z3.copy(), bnes=bnes, dbdt=z2.copy(), eir=z2.copy(), eip=z2.copy(),
                  outside=np.zeros((g.nr, nt), dtype=np.int32))


def perturbed_fields(g: Grid, seed: int = 99, compress: float = 0.15, efield: float = 2e-4,
                     rates: float = 1.0, outside_cells: int = 3) -> Fields:
    """Non-dipole tables that switch on every term the dipole zeroes: a
    day-night compressed B and h/I (so the gradient-curvature drift and its
    J derivatives are nonzero), seeded induced fields EIR/EIP [V/m], time
    derivatives dBdt, dIdt, dIbndt, and a few outer cells outside the
    magnetopause.  Used to exercise the DRIFTR stale-ghost lines and the
    magnetopause paths."""
    f = dipole_fields(g, seed=seed)
    nf, nt, npa = g.nr + 1, g.nt, g.npa
    rng = np.random.Generator(np.random.PCG64(seed + 1))
    lz = g.lz[:, None]
    cphi = np.cos(g.phi)[None, :]
    bfac = 1.0 + compress * cphi * (lz / 6.5) ** 3
    f.bnes = f.bnes * bfac
    hfac = (1.0 + 0.5 * compress * cphi[:, :, None] * (lz[:, :, None] / 6.5) ** 2
            * (1.0 - g.mu[None, None, :] ** 2))
    for k in ("fnhs", "fnis", "bounhs", "bounis"):
        setattr(f, k, getattr(f, k) * hfac)
    smooth = lambda a: 0.5 * (a + np.roll(a, 1, axis=1))  # noqa: E731
    f.eir = efield * smooth(rng.standard_normal((nf, nt)))
    f.eip = efield * smooth(rng.standard_normal((nf, nt)))
    f.dbdt = rates * 1e-12 * smooth(rng.standard_normal((nf, nt)))
    f.didt = rates * 1e-6 * rng.standard_normal((nf, nt, npa))
    f.dibndt = rates * 1e-6 * rng.standard_normal((nf, nt, npa))
    for k in ("bnes", "eir", "eip", "dbdt"):
        a = getattr(f, k)
        a[:, nt - 1] = a[:, 0]
    for k in ("fnhs", "fnis", "bounhs", "bounis", "didt", "dibndt"):
        a = getattr(f, k)
        a[:, nt - 1, :] = a[:, 0, :]
    out = np.zeros((g.nr, nt), dtype=np.int32)
    jmid = (nt - 1) // 2  # noon side
    for c in range(outside_cells):
        out[g.nr - 1, (jmid + c) % (nt - 1)] = 1
    f.outside = out
    return f


# ------------------------------------------------------------------ state
def kappa_flux(e_kev, kt=5.0, kappa=3.0, amp=1.0e5):
    """Kappa differential flux [1/cm2/s/sr/keV] (shape only; amp sets scale)."""
    return amp * (e_kev / kt) * (1.0 + e_kev / (kappa * kt)) ** (-(kappa + 1.0))


def initial_f2(g: Grid, f: Fields, s: int, seed: int, kt=5.0, kappa=3.0, amp=1.0e5,
               l0=4.5, sigma_l=0.8, noise=0.01, density_scale=1.0) -> np.ndarray:
    """F2(I,J,K,L) of species s: kappa x sin^2(alpha) x Gaussian(L) x
    (1+0.2 cos phi) x lognormal(noise), times FFACTOR*FNHS.  C order (I,J,K,L)."""
    nr, nt, ne, npa = g.nr, g.nt, g.ne, g.npa
    rng = np.random.Generator(np.random.PCG64(seed))
    j_e = kappa_flux(g.ekev, kt, kappa, amp) * density_scale
    sin2 = 1.0 - g.mu ** 2
    radial = np.exp(-(g.lz[:nr] - l0) ** 2 / (2.0 * sigma_l ** 2))
    azim = 1.0 + 0.2 * np.cos(g.phi)
    flux = (radial[:, None, None, None] * azim[None, :, None, None] * j_e[None, None, :, None]
            * sin2[None, None, None, :])
    flux = flux * rng.lognormal(0.0, noise, size=flux.shape)
    f2 = flux * g.ffactor[s][:, None, :, :] * f.fnhs[:nr, :, None, :]
    f2[:, nt - 1] = f2[:, 0]
    return np.ascontiguousarray(f2)


def edge_state(f2s, seed: int = 5):
    """Copies of the species' F2 arrays edited to reach every corner of the
    sweeps: blocks of exact zeros (faces with X = 0, the |X| <= 1e-27
    upwind branch, R = 0), cells of 1e-30 (differences below 1e-27 next to
    zeros), isolated spikes 1e3 above their neighbours (limiter ratios
    R < 0 and R > beta, and at high Kp updates that come out negative and
    are clipped to 1e-15), and a whole line of one value (X = 0 along it)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for f in f2s:
        a = np.array(f, dtype=np.float64, copy=True)
        nr, nt, ne, npa = a.shape
        for _ in range(6):  # zero blocks
            i0, j0 = int(rng.integers(nr - 2)), int(rng.integers(nt - 3))
            k0, l0 = int(rng.integers(1, ne - 4)), int(rng.integers(1, npa - 6))
            a[i0:i0 + 2, j0:j0 + 3, k0:k0 + 4, l0:l0 + 6] = 0.0
        for _ in range(64):  # tiny cells
            a[tuple(int(rng.integers(d)) for d in a.shape)] = 1e-30
        for _ in range(64):  # spikes
            c = tuple(int(rng.integers(d)) for d in a.shape)
            a[c] = a[c] * 1e3 + 1e-10
        i, j, k = int(rng.integers(1, nr)), int(rng.integers(nt)), int(rng.integers(1, ne))
        a[i, j, k, :] = a[i, j, k, 1]  # one flat pitch-angle line
        a[:, nt - 1] = a[:, 0]
        out.append(np.asfortranarray(a))
    return out


def boundary_fgeos(g: Grid, s: int, kt=5.0, kappa=3.0, amp=1.0e5, density_scale=1.0) -> np.ndarray:
    """FGEOS(J,K,L) = flux(K)*FFACTOR(S,NR,K,L) for L=2..int(UPA(NR)-1), as GEOSB.
    C order (J,K,L)."""
    nt, ne, npa = g.nt, g.ne, g.npa
    j_e = kappa_flux(g.ekev, kt, kappa, amp) * density_scale
    u = int(g.upa[g.nr - 1] - 1)
    out = np.zeros((nt, ne, npa))
    for L in range(2, u + 1):
        out[:, :, L - 1] = j_e[None, :] * g.ffactor[s, g.nr - 1, :, L - 1][None, :]
    return out


def pa_diffusion(g: Grid, f: Fields, seed: int = 7, d0: float = 2.0e-5) -> np.ndarray:
    """Synthetic pitch-angle diffusion coefficient D(I,J,K,L) in RAM's form
    D_mumu*mu*h (the coefficient WPADIF and FLCscatter divide by DMU): a
    (1-mu^2) profile, decreasing with energy, log-normal in space.  d0 sets
    the implicit step's off-diagonal weight AN ~ d0*DTs*(1-mu^2)/(DMU*WMU)
    near O(0.1-1) on the standard grid.  C order (I,J,K,L)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    nr, nt, ne, npa = g.nr, g.nt, g.ne, g.npa
    mu = np.asarray(g.mu)
    prof = (1.0 - mu ** 2) * mu
    ek = (np.asarray(g.ekev) / 10.0) ** -0.5
    d = (d0 * ek[None, None, :, None] * prof[None, None, None, :] * f.fnhs[:nr, :, None, :]
         * rng.lognormal(0.0, 0.3, size=(nr, nt, ne, npa)))
    d[:, nt - 1] = d[:, 0]
    return np.ascontiguousarray(d)


def rairden_density(dist):
    """Rairden-like hydrogen geocorona density [m^-3] against geocentric
    distance [RE], the RAIRDEN mode of computehI (src/ModRamScb.f90:364-369)."""
    d = np.asarray(dist)
    return 10 ** (13.326 - 3.6908 * d + 1.1362 * d ** 2 - 0.16984 * d ** 3 + 0.009553 * d ** 4)


@dataclass
class FieldLines:
    """Field lines through the RAM grid points, the input of the bounce
    integrals: chi (nthe) and x, y, z, B, density (nthe, NR, NT), lines
    I = 1..NR at L-shell LZ(I+1) (they fill FNHS(I+1,...)); ieq is the
    1-based equator node."""
    chi: np.ndarray
    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    b: np.ndarray
    dens: np.ndarray
    ieq: int


def dipole_lines(g: Grid, nthe: int = 201) -> FieldLines:
    """Dipole field lines (B in units of the surface equatorial field) from
    foot to foot, nodes equally spaced in arc length; chi = pi*s/length."""
    if nthe % 2 == 0:
        raise ValueError("nthe must be odd (a node on the equator)")
    nr, nt = g.nr, g.nt
    x = np.zeros((nthe, nr, nt)); y = np.zeros_like(x); z = np.zeros_like(x); b = np.zeros_like(x)
    chi = np.zeros(nthe)
    for i in range(nr):
        lsh = g.lz[i + 1]
        lam0 = math.acos(math.sqrt(1.0 / lsh))
        lam = np.linspace(-lam0, lam0, 20001)
        ds = lsh * np.cos(lam) * np.sqrt(1 + 3 * np.sin(lam) ** 2)
        s = np.concatenate([[0.0], np.cumsum(0.5 * (ds[1:] + ds[:-1]) * np.diff(lam))])
        sk = np.linspace(0.0, s[-1], nthe)
        lk = np.interp(sk, s, lam)
        lk[(nthe - 1) // 2] = 0.0
        r = lsh * np.cos(lk) ** 2
        bb = np.sqrt(1 + 3 * np.sin(lk) ** 2) / r ** 3
        chi = math.pi * sk / s[-1]
        for j in range(nt):
            ph = g.phi[j]
            x[:, i, j] = r * np.cos(lk) * math.cos(ph)
            y[:, i, j] = r * np.cos(lk) * math.sin(ph)
            z[:, i, j] = r * np.sin(lk)
            b[:, i, j] = bb
    dens = rairden_density(np.sqrt(x ** 2 + y ** 2 + z ** 2))
    return FieldLines(chi, x, y, z, b, dens, (nthe + 1) // 2)


def vols_vt(g: Grid, kp: float) -> np.ndarray:
    """VT(I,J), I=1..NR+1 (src/ModRamRun.f90:45-54).  C order (I,J)."""
    t = 1. - 0.159 * kp + 0.0093 * (kp * kp)
    avs = 7.05e-6 / (t * t * t) / RE
    vt = np.zeros((g.nr + 1, g.nt))
    for i in range(g.nr + 1):
        lr = g.lz[i] * RE
        for j in range(g.nt):
            vt[i, j] = avs * (lr * lr) * math.sin(g.phi[j] - 0.0)
    return vt


# --------------------------------------------------------------- workloads
# Species parameters of the four-species configuration: (kT [keV], density share)
FOUR_SPECIES = (("e", 1.0, 1.0), ("H", 5.0, 0.6), ("He", 5.0, 0.05), ("O", 5.0, 0.3))


@dataclass
class Workload:
    name: str
    grid: Grid
    fields: Fields
    f2: list            # per species, C order (I,J,K,L)
    fgeos: list         # per species, C order (J,K,L)
    kp: object          # callable(step_index) -> Kp
    dts: float
    steps: int          # DTs half-steps (a ram_run call is two)
    meta: dict = field(default_factory=dict)


def make_workload(name: str, seed: int = 2024) -> Workload:
    """The synthetic workloads:
      single_h   : H+ only, 20x25x35x72, Kp=3, dt=5 s, 720 steps
      four_sp    : e-,H+,He+,O+, 20x25x35x72, Kp 1->6 over 4320 steps, dt=5 s
      refined    : four species, 40x49x70x144, Kp 1->6, dt=2.5 s, 1440 steps
      tiny       : four species on a reduced 6x9x35x72 grid (tests)
      tiny_pert  : tiny with perturbed_fields (non-dipole, E_ind, dB/dt,
                   magnetopause cells) for coverage of the zero-in-dipole terms
      tiny_pert8 : tiny_pert on an 8x9x35x72 grid (NR a multiple of 4: the
                   DRIFTR lines own whole 32-byte sectors)
    """
    if name == "single_h":
        sp = [HYDROGEN]
        g = arrays(20, 25, 35, 72, species=tuple(sp))
        params = [(5.0, 1.0)]
        kp = lambda step: 3.0  # noqa: E731
        dts, steps = 5.0, 720
    elif name in ("four_sp", "tiny", "tiny_pert", "tiny_pert8"):
        sp = [SPECIES[c] for c, _, _ in FOUR_SPECIES]
        if name in ("tiny", "tiny_pert"):
            g = arrays(6, 9, 35, 72, species=tuple(sp), mu_grid_nr=20)
        elif name == "tiny_pert8":
            g = arrays(8, 9, 35, 72, species=tuple(sp), mu_grid_nr=20)
        else:
            g = arrays(20, 25, 35, 72, species=tuple(sp))
        params = [(kt, sh) for _, kt, sh in FOUR_SPECIES]
        steps = 4320 if name == "four_sp" else 16
        kp = (lambda step, n=steps: 1.0 + 5.0 * min(step, n) / n)
        dts = 5.0
    elif name == "refined":
        sp = [SPECIES[c] for c, _, _ in FOUR_SPECIES]
        g = refined_arrays(40, 49, 70, 144, species=tuple(sp))
        params = [(kt, sh) for _, kt, sh in FOUR_SPECIES]
        steps = 1440
        kp = (lambda step, n=steps: 1.0 + 5.0 * min(step, n) / n)
        dts = 2.5
    else:
        raise ValueError(f"unknown workload {name!r}")
    fl = perturbed_fields(g, seed=seed) if name in ("tiny_pert", "tiny_pert8") else dipole_fields(g, seed=seed)
    f2 = [initial_f2(g, fl, s, seed=seed + 17 * (s + 1), kt=params[s][0], density_scale=params[s][1])
          for s in range(len(sp))]
    fg = [boundary_fgeos(g, s, kt=params[s][0], density_scale=params[s][1]) for s in range(len(sp))]
    return Workload(name=name, grid=g, fields=fl, f2=f2, fgeos=fg, kp=kp, dts=dts, steps=steps,
                    meta={"seed": seed, "species": [s.name for s in sp]})


# ---------------------------------------------------------------- ensembles
@dataclass
class Ensemble:
    """Members of the batched-ensemble workload on the standard grid:
    species subsets of size uniform 1-4, Kp drivers piecewise linear with
    knots every 30 min drawn uniform 1-7, initial-density scale lognormal
    (sigma 0.5), run lengths uniform 360-1440 DTs steps."""
    base: Workload
    species: list        # per member: sorted species indices
    kp_knots: np.ndarray  # (members, nknots)
    scale: np.ndarray     # (members,)
    length: np.ndarray    # (members,) DTs steps
    knot_steps: int       # DTs steps between knots (30 min / DTs)

    @property
    def members(self) -> int:
        return len(self.species)

    def kp(self, step: int) -> np.ndarray:
        """Kp of every member at DTs step `step` (piecewise linear)."""
        x = step / self.knot_steps
        i = min(int(x), self.kp_knots.shape[1] - 2)
        w = x - i
        return (1.0 - w) * self.kp_knots[:, i] + w * self.kp_knots[:, i + 1]


def make_ensemble(members: int = 256, seed: int = 4242) -> Ensemble:
    base = make_workload("four_sp", seed=seed)
    rng = np.random.Generator(np.random.PCG64(seed))
    species = []
    for _ in range(members):
        n = int(rng.integers(1, 5))
        species.append(sorted(rng.choice(4, size=n, replace=False).tolist()))
    knot_steps = int(round(1800.0 / base.dts))
    nknots = 1440 // knot_steps + 2
    kp_knots = rng.uniform(1.0, 7.0, size=(members, nknots))
    scale = rng.lognormal(0.0, 0.5, size=members)
    length = rng.integers(360, 1441, size=members)
    return Ensemble(base=base, species=species, kp_knots=kp_knots, scale=scale, length=length,
                    knot_steps=knot_steps)
