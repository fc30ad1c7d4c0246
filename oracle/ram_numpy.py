"""Second, independent CPU restatement of the RAM step, in vectorised NumPy.

TEST INFRASTRUCTURE ONLY: imported by tests/ to pin the C oracle
(oracle/ram_oracle.c), never by the product.  It is written from the
Fortran text of the reference without reading the C oracle and takes no
array computed by it: inputs are the grid, the field tables, F2 and FGEOS.

Every expression keeps the reference's operation order (Fortran evaluates
a chain of +,- or *,/ left to right), so where no library function is
involved the results equal the C oracle bit for bit:

  VOLS potential       src/ModRamRun.f90:45-54
  DRIFTPARA            src/ModRamDrift.f90:36-88
  DRIFTR (CR, CGR)     src/ModRamDrift.f90:95-198
  DRIFTP (CDriftP)     src/ModRamDrift.f90:204-279
  DRIFTE (CDriftE)     src/ModRamDrift.f90:285-376
  DRIFTMU (CDriftMu)   src/ModRamDrift.f90:382-473
  CEPARA               src/ModRamLoss.f90:19-170
  CHAREXCHANGE, ATMOL  src/ModRamLoss.f90:457-507
  ram_run sequence     src/ModRamRun.f90:64-222
  ANISCH moments       src/ModRamRun.f90:343-415

Integer powers: gfortran expands X**2 as X*X, X**3 as (X*X)*X and X**4 as
(X*X)*(X*X) (the binary powering of __builtin_powi), and integer constants
in real expressions (2*FNHS, /2, 1/FNHS) convert exactly.  The library
functions (SIN in VOLS, LOG10/10.**Y/EXP in CEPARA, ** with a real exponent
in ATMOL) may differ from the C library's in the last place, so results that
pass through them agree to a few units in the last place, not bit for bit.

Arrays use the reference's index order with 0-based indices: F2 is
(NR, NT, NE, NPA) for one species, field tables (NR+1, NT, NPA) and
(NR+1, NT), FGEOS (NT, NE, NPA).
"""
from __future__ import annotations

import numpy as np

RE = 6.371E6          # src/ModRamConst.f90:14
Q = 1.602E-19         # src/ModRamConst.f90:19
CS = 2.998E8          # src/ModRamConst.f90:20
PI = 3.1415926535897932384626433832795
OME = 7.3E-5          # src/ModRamDrift.f90:224,300,397

# CEPARA's fitted cross sections, src/ModRamLoss.f90:46,61,76 (by cex kind)
CEX_POLY = {1: (-18.767, -0.11017, -3.8173e-2, -0.1232, -5.0488e-2),
            2: (-20.789, 0.92316, -0.68017, 0.66153, -0.20998),
            3: (-18.987, -0.10613, -5.4841E-3, -1.6262E-2, -7.0554E-3)}


def _jm(nt):
    """J0 of the reference (J-1, with J=1 -> NT-1), 0-based."""
    j = np.arange(nt)
    return np.where(j == 0, nt - 2, j - 1)


def _jp(nt):
    """J1/J2 of the reference (J+1, with J=NT -> 2), 0-based."""
    j = np.arange(nt)
    return np.where(j == nt - 1, 1, j + 1)


class Fld:
    """Field tables as float64 arrays in the reference's index order."""

    def __init__(self, fields):
        for k in ("fnhs", "fnis", "bounhs", "bounis", "hdns", "didt", "dibndt", "bnes", "dbdt", "eir", "eip"):
            setattr(self, k, np.asarray(getattr(fields, k), dtype=np.float64))
        self.outside = np.asarray(fields.outside)


# ------------------------------------------------------------------ VOLS
def vt_vols(g, kp):
    """VT(I,J) = AVS*(LZ(I)*RE)**2*SIN(PHI(J)-PHIOFS), PHIOFS = 0,
    AVS = 7.05E-6/(1.-0.159*KP+0.0093*KP**2)**3/RE (src/ModRamRun.f90:45-54)."""
    t = (1. - 0.159 * kp) + 0.0093 * (kp * kp)
    avs = (7.05E-6 / ((t * t) * t)) / RE
    lr = np.asarray(g.lz, dtype=np.float64) * RE
    return (avs * (lr * lr))[:, None] * np.sin(np.asarray(g.phi) - 0.0)[None, :]


# ------------------------------------------------------------- DRIFTPARA
def driftpara(g, s, dts):
    """VR, P1, P2, MUDOT, EDOT of DRIFTPARA (src/ModRamDrift.f90:66-86)."""
    rlz = np.asarray(g.rlz[:g.nr], dtype=np.float64)
    mdr, dphi, qs = g.mdr, g.dphi, float(g.species[s].charge)
    grel, grbnd = np.asarray(g.grel[s]), np.asarray(g.grbnd[s])
    ekev, ebnd, mu, wmu = (np.asarray(a, dtype=np.float64) for a in (g.ekev, g.ebnd, g.mu, g.wmu))
    vr = ((((dts / mdr) / (rlz + 0.5 * mdr)) / 2) / dphi)
    p1 = ((((dts / dphi) / 2) / mdr) / rlz)
    num = ((dts * ekev) * 1000) * (grel + 1)
    p2 = ((((num / grel)[None, :] / (rlz * rlz)[:, None]) / dphi) / qs)
    muboun = mu[:-1] + 0.5 * wmu[:-1]
    mudot = np.zeros((g.nr, g.npa))
    mudot[:, :-1] = (((((1. - muboun * muboun) * dts) / 2) / muboun)[None, :] / rlz[:, None])
    edot = ((((((ebnd * dts)[None, :] / rlz[:, None]) * (grbnd + 1)[None, :]) / grbnd[None, :]) / 2.))
    return {"vr": vr, "p1": p1, "p2": p2, "mudot": mudot, "edot": edot}


def _dt_min(c, outside_ij, num, floor, init):
    """min over cells inside the magnetopause of num/max(|C|,floor)."""
    ct = np.maximum(np.abs(c), floor)
    q = num / ct
    inside = np.broadcast_to((outside_ij == 0).reshape(outside_ij.shape + (1,) * (q.ndim - 2)), q.shape)
    return float(min(init, q[inside].min())) if inside.any() else float(init)


# ---------------------------------------------------------------- DRIFTR
def cdrift_r(g, f, s, dts, vt, fraccfl=0.8):
    """CDriftR(I,J,K,L) = CR + CGR for I = 1..NR (src/ModRamDrift.f90:117-146)
    and DtDriftR (:147-150)."""
    nr, nt = g.nr, g.nt
    mdr, dphi, qs = g.mdr, g.dphi, float(g.species[s].charge)
    dp = driftpara(g, s, dts)
    j0, j1 = _jm(nt), _jp(nt)
    bn, vt = f.bnes, np.asarray(vt, dtype=np.float64)
    i = np.arange(nr)
    den = bn[i, :] + bn[i + 1, :]                                         # BNES(I,J)+BNES(I+1,J)
    vsum = ((vt[i][:, j0] + vt[i + 1][:, j0]) - vt[i][:, j1]) - vt[i + 1][:, j1]
    cr = (dp["vr"][:, None] * vsum) / den + ((((f.eip[i, :] + f.eip[i + 1, :]) / den) * dts) / mdr)
    grel = np.asarray(g.grel[s])
    p4 = ((((((dts * np.asarray(g.ekev)) * 1000.0) * (grel + 1)) / grel) / dphi) / mdr) / qs
    fi, fh = f.fnis, f.fnhs                                               # (NR+1, NT, NPA)
    cgr1 = ((fi[i + 1][:, j1] + fi[i][:, j1]) - fi[i + 1][:, j0]) - fi[i][:, j0]
    cgr2 = ((bn[i + 1][:, j1] + bn[i][:, j1]) - bn[i + 1][:, j0]) - bn[i][:, j0]
    cgr3 = cgr1 + (((((fi[i + 1] + fi[i]) - 2 * fh[i + 1]) - 2 * fh[i]) * cgr2[:, :, None]) / 2.) \
        / (bn[i + 1] + bn[i])[:, :, None]
    t = (cgr3 / (fh[i] + fh[i + 1]))[:, :, None, :] * p4[None, None, :, None]
    cgr = ((t / 2.) / den[:, :, None, None]) / (np.asarray(g.rlz[:nr]) + 0.5 * mdr)[:, None, None, None]
    c = cr[:, :, None, None] + cgr
    dt = _dt_min(c, f.outside, fraccfl * dts, 1E-10, 100000.0)
    return c, dt


def _limited_face(fi, fn, x, c_over_d, sg, d, beta):
    """FBND of the reference's limiter block (src/ModRamDrift.f90:169-183):
    fi = F(I), fn = F(I+1), x = X, d = F(N)-F(N-1), c_over_d = the Courant
    number of CORR, sg = sgn (+-1)."""
    fup = 0.5 * ((fi + fn) - sg * x)
    with np.errstate(divide="ignore", invalid="ignore"):
        r = d / x
    lim = np.maximum(np.minimum(beta * r, 1.), np.minimum(r, beta))
    corr = -((0.5 * (c_over_d - sg)) * x)
    fb = fup + lim * corr
    keep = (np.abs(x) <= 1.E-27) | ~(r > 0)
    return np.where(keep, fup, fb)


def drift_r(g, f, s, f2, fgeos, dts, vt, beta=1.5, fraccfl=0.8, closed=False):
    """DRIFTR (src/ModRamDrift.f90:95-198), lines (J,K,L) along I; F(NR+1:NR+2)
    persist across lines in the K -> L -> J loop order.  Returns the new F2,
    CDriftR and DtDriftR."""
    nr, nt, ne, npa = g.nr, g.nt, g.ne, g.npa
    c, dt = cdrift_r(g, f, s, dts, vt, fraccfl)
    sgn = np.where(c < 0, -1.0, 1.0)
    inflow = sgn[nr - 1] < 0                                           # (NT, NE, NPA)
    fg = np.asarray(fgeos, dtype=np.float64)
    fh_nr = f.fnhs[nr - 1][:, None, :]                                  # FNHS(NR,J,L)
    outs = (f.outside[nr - 1] == 1)[:, None, None]
    v1 = np.where(outs, 0.0, (fg * g.conf1) * fh_nr)
    v2 = np.where(outs, 0.0, (fg * g.conf2) * fh_nr)
    # the ghost a line sees: set by the most recent inflow line in K,L,J order
    order = lambda a: np.transpose(a, (1, 2, 0)).reshape(-1)            # noqa: E731
    n = np.arange(nt * ne * npa)
    last = np.maximum.accumulate(np.where(order(inflow), n, -1))
    g1 = np.where(last >= 0, order(v1)[np.maximum(last, 0)], 0.0)
    g2 = np.where(last >= 0, order(v2)[np.maximum(last, 0)], 0.0)
    unorder = lambda a: np.transpose(a.reshape(ne, npa, nt), (2, 0, 1))  # noqa: E731
    fe = np.concatenate([f2, unorder(g1)[None], unorder(g2)[None]], axis=0)  # F(1..NR+2)
    fb = np.zeros_like(f2)
    fb[0] = np.where(inflow, fe[1], 0.0)                                 # FBND(1)
    for I in range(2, nr + 1):                                          # 1-based face
        sg = sgn[I - 1]
        x = fe[I] - fe[I - 1]
        if I < nr:
            d = np.where(sg > 0, fe[I - 1] - fe[I - 2], fe[I + 1] - fe[I])
        else:
            d = fe[I + 1] - fe[I]                                       # inflow lines only
        face = _limited_face(fe[I - 1], fe[I], x, c[I - 1], sg, d, beta)
        fb[I - 1] = face if I < nr else np.where(inflow, face, fe[nr - 1])
    if closed:
        fb[0] = 0.0
        fb[nr - 1] = 0.0
    out = f2.copy()
    for I in range(2, nr + 1):
        v = (f2[I - 1] - c[I - 1] * fb[I - 1]) + c[I - 2] * fb[I - 2]
        out[I - 1] = np.where(v < 0, 1E-15, v)
    return out, c, dt


# ---------------------------------------------------------------- DRIFTP
def cdrift_p(g, f, s, dts, vt, fraccfl=0.8):
    """CDriftP(I,J,K,L), I = 2..NR, J = 2..NT, with CDriftP(I,1) = CDriftP(I,NT)
    (src/ModRamDrift.f90:225-262), and DtDriftP."""
    nr, nt = g.nr, g.nt
    mdr, dphi = g.mdr, g.dphi
    dp = driftpara(g, s, dts)
    i = np.arange(1, nr)[:, None]
    j = np.arange(1, nt)[None, :]
    j1 = _jp(nt)[1:][None, :]
    fi, fh, bn, vt = f.fnis, f.fnhs, f.bnes, np.asarray(vt, dtype=np.float64)
    rlz = np.asarray(g.rlz)[1:nr][:, None]
    gpa1 = (fi[i, j] + fi[i, j1]) + (((((fi[i + 1, j1] + fi[i + 1, j]) - fi[i - 1, j]) - fi[i - 1, j1])
                                      * rlz[..., None]) / 2.) / mdr
    gpa2 = ((((rlz / 4.) / mdr)[..., None] * (((fi[i, j] + fi[i, j1]) - 2 * fh[i, j]) - 2 * fh[i, j1]))
            * (((bn[i + 1, j1] + bn[i + 1, j]) - bn[i - 1, j]) - bn[i - 1, j1])[..., None]) \
        / (bn[i, j] + bn[i, j1])[..., None]                                # (NR-1, NT-1, NPA)
    vterm = (((vt[i + 1, j] + vt[i + 1, j1]) - vt[i - 1, j]) - vt[i - 1, j1]) * dp["p1"][1:nr][:, None]
    eterm = (((f.eir[i, j1] + f.eir[i, j]) / rlz) * dts) / dphi
    p2 = dp["p2"][1:nr]                                                 # (NR-1, NE)
    grad = (p2[:, None, :, None] * (gpa1 + gpa2)[:, :, None, :]) / (fh[i, j] + fh[i, j1])[:, :, None, :]
    cp = ((vterm[:, :, None, None] - grad) - eterm[:, :, None, None]) / (bn[i, j] + bn[i, j1])[:, :, None, None] \
        + ((OME * dts) / dphi)
    dt = _dt_min(cp, f.outside[1:nr, 1:nt], fraccfl * dts, 1E-10, 100000.0)
    c = np.zeros((nr, nt, g.ne, g.npa))
    c[1:, 1:] = cp
    c[1:, 0] = c[1:, nt - 1]
    return c, dt


def drift_p(g, f, s, f2, dts, vt, beta=1.5, fraccfl=0.8):
    """DRIFTP (src/ModRamDrift.f90:204-279): periodic lines along J for I >= 2."""
    nt = g.nt
    c, dt = cdrift_p(g, f, s, dts, vt, fraccfl)
    F = f2[1:]                                                          # (NR-1, NT, NE, NPA)
    C = c[1:]
    fb = np.zeros_like(F)
    for J in range(2, nt + 1):                                          # 1-based face
        J1 = 2 if J == nt else J + 1
        sg = np.where(C[:, J - 1] < 0, -1.0, 1.0)
        x = F[:, J1 - 1] - F[:, J - 1]
        Np = J                                                          # N for sgn = +1
        Nm = J + 2                                                      # N for sgn = -1
        if Nm > nt:
            Nm = Nm - nt + 1
        d = np.where(sg > 0, F[:, Np - 1] - F[:, Np - 2], F[:, Nm - 1] - F[:, Nm - 2])
        fb[:, J - 1] = _limited_face(F[:, J - 1], F[:, J1 - 1], x, C[:, J - 1], sg, d, beta)
    fb[:, 0] = fb[:, nt - 1]
    out = f2.copy()
    for J in range(2, nt + 1):
        v = (F[:, J - 1] - C[:, J - 1] * fb[:, J - 1]) + C[:, J - 2] * fb[:, J - 2]
        out[1:, J - 1] = np.where(v < 0, 1E-15, v)
    out[1:, 0] = out[1:, nt - 1]
    return out, c, dt


# ---------------------------------------------------------------- DRIFTE
def cdrift_e(g, f, s, dts, vt, fraccfl=0.8):
    """CDriftE(I,J,K,L) for I = 2..NR (src/ModRamDrift.f90:314-342) and
    DtDriftE."""
    nr, nt = g.nr, g.nt
    mdr, dphi, qs = g.mdr, g.dphi, float(g.species[s].charge)
    dp = driftpara(g, s, dts)
    i = np.arange(1, nr)[:, None]
    j = np.arange(nt)[None, :]
    j0, j2 = _jm(nt)[None, :], _jp(nt)[None, :]
    fi, fh, bn, vt = f.fnis, f.fnhs, f.bnes, np.asarray(vt, dtype=np.float64)
    rlz = np.asarray(g.rlz)[1:nr][:, None]
    drd1 = ((f.eip[i, j] * rlz) - (((vt[i, j2] - vt[i, j0]) / 2.) / dphi)) / bn[i, j]
    dpd1 = (OME * rlz) + (((((vt[i + 1, j] - vt[i - 1, j]) / 2) / mdr) - f.eir[i, j]) / bn[i, j])
    r3, b3 = rlz[..., None], bn[i, j][..., None]
    gpa = (1. - ((fi[i, j] / 2.) / fh[i, j])) / b3
    gpr1 = ((gpa * (bn[i + 1, j] - bn[i - 1, j])[..., None]) / 2.) / mdr
    gpr2 = -((fi[i, j] / fh[i, j]) / r3)
    gpr3 = -((((fi[i + 1, j] - fi[i - 1, j]) / 2.) / mdr) / fh[i, j])
    gpp1 = ((gpa * (bn[i, j2] - bn[i, j0])[..., None]) / 2.) / dphi
    gpp2 = -((((fi[i, j2] - fi[i, j0]) / 2.) / dphi) / fh[i, j])
    drd2 = (((fi[i, j2] - fi[i, j0]) / 2.) / dphi) \
        + (((((fi[i, j] - 2 * fh[i, j]) * (bn[i, j2] - bn[i, j0])[..., None]) / 4) / b3) / dphi)
    dpd2 = (fi[i, j] + ((((fi[i + 1, j] - fi[i - 1, j]) * r3) / 2) / mdr)) \
        + (((((r3 * (fi[i, j] - 2 * fh[i, j])) / 4) / mdr) * (bn[i + 1, j] - bn[i - 1, j])[..., None]) / b3)
    grbnd = np.asarray(g.grbnd[s])
    eb = (((np.asarray(g.ebnd) * 1e3) * (grbnd + 1)) / 2) / grbnd           # (NE)
    edt1 = (((eb[None, None, :, None] / fh[i, j][:, :, None, :]) / r3[..., None]) / b3[..., None]) / qs
    drdt = drd1[:, :, None, None] + ((edt1 * drd2[:, :, None, :]) * r3[..., None])
    dpdt = dpd1[:, :, None, None] - edt1 * dpd2[:, :, None, :]
    dbdt1 = ((f.dbdt[i, j][..., None] * (1. - ((fi[i, j] / 2.) / fh[i, j]))) * r3) / b3
    didt1 = -((f.didt[i, j] * r3) / fh[i, j])
    ce = dp["edot"][1:nr][:, None, :, None] * (
        ((((gpr1 + gpr2) + gpr3)[:, :, None, :] * drdt) + ((gpp1 + gpp2)[:, :, None, :] * dpdt))
        + dbdt1[:, :, None, :] + didt1[:, :, None, :])
    de = np.asarray(g.de)[None, None, :, None]
    dt = _dt_min(ce, f.outside[1:nr], (fraccfl * dts) * de, 1E-10, 10000.0)
    c = np.zeros((nr, nt, g.ne, g.npa))
    c[1:] = ce
    return c, dt


def drift_e(g, f, s, f2, dts, vt, beta=1.5, fraccfl=0.8, closed=False):
    """DRIFTE (src/ModRamDrift.f90:285-376): lines (I,J,L) along K with the
    relativistic extrapolation of F(1), F(0) and F(NE+1) = F(NE+2) = 0."""
    ne = g.ne
    c, dt = cdrift_e(g, f, s, dts, vt, fraccfl)
    grel = np.asarray(g.grel[s])
    ezero = g.ekev[0] - g.we[0]
    grzero = 1. + (((ezero * 1000.) * Q) / g.rmas[s]) / CS / CS
    F = np.zeros((g.nr - 1, g.nt, ne + 3, g.npa))                       # F(0..NE+2)
    F[:, :, 1:ne + 1] = f2[1:]
    F[:, :, 1] = ((F[:, :, 2] * grel[0]) / grel[1]) * np.sqrt(((grel[1] * grel[1]) - 1) / ((grel[0] * grel[0]) - 1))
    F[:, :, 0] = ((F[:, :, 1] * grzero) / grel[0]) * np.sqrt(((grel[0] * grel[0]) - 1) / ((grzero * grzero) - 1))
    C = c[1:]
    de = np.asarray(g.de)
    fb = np.zeros((g.nr - 1, g.nt, ne, g.npa))
    for K in range(1, ne + 1):
        sg = np.where(C[:, :, K - 1] < 0, -1.0, 1.0)
        x = F[:, :, K + 1] - F[:, :, K]
        d = np.where(sg > 0, F[:, :, K] - F[:, :, K - 1], F[:, :, K + 2] - F[:, :, K + 1])
        fb[:, :, K - 1] = _limited_face(F[:, :, K], F[:, :, K + 1], x, C[:, :, K - 1] / de[K - 1], sg, d, beta)
    if closed:
        fb[:, :, 0] = 0.0
        fb[:, :, ne - 1] = 0.0
    we = np.asarray(g.we)
    out = f2.copy()
    for K in range(2, ne + 1):
        v = (f2[1:, :, K - 1] - (C[:, :, K - 1] / we[K - 1]) * fb[:, :, K - 1]) \
            + (C[:, :, K - 2] / we[K - 1]) * fb[:, :, K - 2]
        out[1:, :, K - 1] = np.where(v < 0, 1E-15, v)
    return out, c, dt


# --------------------------------------------------------------- DRIFTMU
def cdrift_mu(g, f, s, dts, vt, fraccfl=0.8):
    """CDriftMu(I,J,K,L) for I = 2..NR, L = 2..NPA, CDriftMu(.,1) = 0
    (src/ModRamDrift.f90:406-456), and DtDriftMu."""
    nr, nt = g.nr, g.nt
    mdr, dphi, qs = g.mdr, g.dphi, float(g.species[s].charge)
    dp = driftpara(g, s, dts)
    i = np.arange(1, nr)[:, None]
    j = np.arange(nt)[None, :]
    j0, j1 = _jm(nt)[None, :], _jp(nt)[None, :]
    bi, bh, bn, vt = f.bounis, f.bounhs, f.bnes, np.asarray(vt, dtype=np.float64)
    rlz = np.asarray(g.rlz)[1:nr][:, None]
    r3, b3 = rlz[..., None], bn[i, j][..., None]
    drm1 = ((f.eip[i, j] * rlz) - (((vt[i, j1] - vt[i, j0]) / 2) / dphi)) / bn[i, j]
    dpm1 = (OME * rlz) + (((((vt[i + 1, j] - vt[i - 1, j]) / 2) / mdr) - f.eir[i, j]) / bn[i, j])
    L = slice(1, g.npa)
    cmudot = (dp["mudot"][1:nr][:, None, L] * bi[i, j, L]) / bh[i, j, L]
    gmr1 = (((bn[i + 1, j] - bn[i - 1, j]) / 4) / mdr) / bn[i, j]
    gmr2 = 1 / rlz
    gmr3 = (((bi[i + 1, j, L] - bi[i - 1, j, L]) / 2) / mdr) / bi[i, j, L]
    gmp1 = (((bn[i, j1] - bn[i, j0]) / 4) / dphi) / bn[i, j]
    gmp2 = (((bi[i, j1, L] - bi[i, j0, L]) / 2) / dphi) / bi[i, j, L]
    grel = np.asarray(g.grel[s])
    ek = (((np.asarray(g.ekev) * 1e3) * (grel + 1)) / 2) / grel            # (NE)
    edt = (((ek[None, None, :, None] / bh[i, j, L][:, :, None, :]) / r3[..., None]) / b3[..., None]) / qs
    drm2 = (((bi[i, j1, L] - bi[i, j0, L]) / 2) / dphi) \
        + (((((bi[i, j, L] - 2 * bh[i, j, L]) * (bn[i, j1] - bn[i, j0])[..., None]) / 4) / b3) / dphi)
    dpm2 = (bi[i, j, L] + ((((bi[i + 1, j, L] - bi[i - 1, j, L]) * r3) / 2) / mdr)) \
        + ((((((bi[i, j, L] - 2 * bh[i, j, L]) * r3) / 4) / mdr) * (bn[i + 1, j] - bn[i - 1, j])[..., None]) / b3)
    drdm = drm1[:, :, None, None] + ((edt * drm2[:, :, None, :]) * r3[..., None])
    dpdm = dpm1[:, :, None, None] - edt * dpm2[:, :, None, :]
    dbdt2 = ((f.dbdt[i, j] / 2.) / bn[i, j]) * rlz
    dibndt2 = (f.dibndt[i, j, L] * r3) / bi[i, j, L]
    gr = ((gmr1 + gmr2)[..., None] + gmr3)[:, :, None, :]             # GMR1+GMR2+GMR3
    gp = (gmp1[..., None] + gmp2)[:, :, None, :]                      # GMP1+GMP2
    inner = (((gr * drdm) + (gp * dpdm)) + dbdt2[:, :, None, None]) + dibndt2[:, :, None, :]
    cm = -(cmudot[:, :, None, :] * inner)
    dmu = np.asarray(g.dmu)[None, None, None, 1:]
    dt = _dt_min(cm, f.outside[1:nr], (fraccfl * dts) * dmu, 1E-32, 10000.0)
    c = np.zeros((nr, nt, g.ne, g.npa))
    c[1:, :, :, 1:] = cm
    return c, dt


def drift_mu(g, f, s, f2, dts, vt, beta=1.5, fraccfl=0.8, closed=False):
    """DRIFTMU (src/ModRamDrift.f90:382-473): lines (I,J,K) along L, F(1) = F(2),
    faces 2..NPA-2 limited, FBND(1) = 0, FBND(NPA-1) = F(NPA), and the
    extrapolated F2(NPA)."""
    npa = g.npa
    c, dt = cdrift_mu(g, f, s, dts, vt, fraccfl)
    F = f2[1:].copy()
    F[..., 0] = F[..., 1]
    C = c[1:]
    dmu = np.asarray(g.dmu)
    fb = np.zeros_like(F)
    for L in range(2, npa - 1):
        sg = np.where(C[..., L - 1] < 0.0, -1.0, 1.0)
        x = F[..., L] - F[..., L - 1]
        d = np.where(sg > 0, F[..., L - 1] - F[..., L - 2], F[..., L + 1] - F[..., L])
        fb[..., L - 1] = _limited_face(F[..., L - 1], F[..., L], x, C[..., L - 1] / dmu[L - 1], sg, d, beta)
    fb[..., 0] = 0.
    fb[..., npa - 2] = 0.0 if closed else F[..., npa - 1]
    wmu = np.asarray(g.wmu)
    out = f2.copy()
    for L in range(2, npa):
        v = (f2[1:, ..., L - 1] - (C[..., L - 1] / wmu[L - 1]) * fb[..., L - 1]) \
            + (C[..., L - 2] / wmu[L - 1]) * fb[..., L - 2]
        out[1:, ..., L - 1] = np.where(v < 0, 1E-15, v)
    fh = f.fnhs[1:g.nr]
    mu = np.asarray(g.mu)
    out[1:, ..., npa - 1] = ((((out[1:, ..., npa - 2] * fh[:, :, None, npa - 1]) * mu[npa - 1])
                              / fh[:, :, None, npa - 2]) / mu[npa - 2])
    return out, c, dt


# ----------------------------------------------------------------- losses
def cepara(g, f, s, dts):
    """CHARGE(I,J,K,L) and ATLOS(I,K) of CEPARA (src/ModRamLoss.f90:34-87,
    162-167): exp(-10**Y*V*HDNS*DTs) for I, K, L >= 2 (1 elsewhere and for
    species without a fitted cross section); ATLOS = exp(-DTs/TAUB),
    TAUB = 2*RLZ/V, for I, K >= 2 (1 elsewhere)."""
    nr, nt, ne, npa = g.nr, g.nt, g.ne, g.npa
    v = np.asarray(g.v[s])
    charge = np.ones((nr, nt, ne, npa))
    kind = g.species[s].cex_kind
    if kind in CEX_POLY:
        a0, a1, a2, a3, a4 = CEX_POLY[kind]
        x = np.log10(np.asarray(g.ekev, dtype=np.float64))
        x = np.where(x < -2., -2., x)
        x2 = x * x
        y = (((a0 + a1 * x) + a2 * x2) + a3 * (x2 * x)) + a4 * (x2 * x2)
        alpha = ((np.power(10., y) * v)[None, None, :, None] * f.hdns[:nr][:, :, None, :]) * dts
        charge[1:, :, 1:, 1:] = np.exp(-alpha)[1:, :, 1:, 1:]
    taub = (2 * np.asarray(g.rlz[:nr]))[:, None] / v[None, :]
    atlos = np.ones((nr, ne))
    atlos[1:, 1:] = np.exp(-dts / taub)[1:, 1:]
    return charge, atlos


def charexchange(g, f2, charge):
    """F2 = F2*CHARGE for I, K, L >= 2 (src/ModRamLoss.f90:457-478)."""
    out = f2.copy()
    out[1:, :, 1:, 1:] = f2[1:, :, 1:, 1:] * charge[1:, :, 1:, 1:]
    return out


def atmol(g, f, f2, atlos):
    """F2 = F2*ATLOS(I,K)**(1/FNHS(I,J,L)) for K >= 2, I >= 2 and
    L >= int(UPA(I)) (src/ModRamLoss.f90:485-507)."""
    out = f2.copy()
    for I in range(2, g.nr + 1):
        u = int(g.upa[I - 1])
        e = 1 / f.fnhs[I - 1, :, u - 1:]                               # (NT, NPA-u+1)
        fac = np.power(atlos[I - 1, 1:][None, :, None], e[:, None, :])
        out[I - 1, :, 1:, u - 1:] = f2[I - 1, :, 1:, u - 1:] * fac
    return out


# ------------------------------------------------------------------ ANISCH
def anisch(g, f, s, f2):
    """ANISCH's moment block (src/ModRamRun.f90:343-415): the side effect
    F2(I,J,K,1) = F2(I,J,K,2) for I, K >= 2 (returned), and PPERT, PPART
    (NR, NT) summed in the reference's order: L = 1..int(UPA(I)-1) inside K,
    K inside the five energy bands KHI = (6,10,25,30,NE)."""
    nr, nt, ne = g.nr, g.nt, g.ne
    out = f2.copy()
    rfac = (4 * PI) / (CS * 100)
    khi = [6, 10, 25, 30, ne]
    ff = np.asarray(g.ffactor[s])                                      # (NR, NE, NPA)
    wmu, mu, epp = np.asarray(g.wmu), np.asarray(g.mu), np.asarray(g.epp[s])
    ppert = np.zeros((nr, nt))
    ppart = np.zeros((nr, nt))
    for I in range(2, nr + 1):
        i = I - 1
        u = int(g.upa[i] - 1)
        out[i, :, 1:, 0] = out[i, :, 1:, 1]
        pt = np.zeros(nt)
        pa = np.zeros(nt)
        klo = 2
        for hi in khi:
            pper = np.zeros(nt)
            ppar = np.zeros(nt)
            for K in range(klo, hi + 1):
                k = K - 1
                sume = np.zeros(nt)
                suma = np.zeros(nt)
                for L in range(1, u + 1):
                    l = L - 1
                    ernm = (wmu[l] / ff[i, k, l]) / f.fnhs[i, :, l]
                    epma = (ernm * mu[l]) * mu[l]
                    epme = ernm - epma
                    sume = sume + out[i, :, k, l] * epme
                    suma = suma + out[i, :, k, l] * epma
                pper = pper + epp[k] * sume
                ppar = ppar + epp[k] * suma
            ppar = (2 * rfac) * ppar
            pper = rfac * pper
            pt = pt + pper
            pa = pa + ppar
            klo = hi + 1
        ppert[i] = pt
        ppart[i] = pa
    return out, ppert, ppart


def flux(g, f, s, f2):
    """FLUX = F2/FFACTOR/FNHS for I, K, L >= 2, J <= NT-1 (src/ModRamRun.f90:208-222),
    zero elsewhere."""
    out = np.zeros_like(f2)
    ff = np.asarray(g.ffactor[s])[1:, None, 1:, 1:]
    fh = f.fnhs[1:g.nr, :g.nt - 1][:, :, None, 1:]
    out[1:, :g.nt - 1, 1:, 1:] = (f2[1:, :g.nt - 1, 1:, 1:] / ff) / fh
    return out


# ----------------------------------------------------------------- ram_run
def ram_run(g, fields, f2s, fgeos, dts, kp=None, vt=None, beta=1.5, fraccfl=0.8, dtsmin=0.1, do_atmol=True):
    """One ram_run call for every species (src/ModRamRun.f90:45-222, the
    processes the path keeps): VT from VOLS, per species R, P, E, MU, CEX,
    ATMOL | ATMOL, CEX, MU, E, P, R; then the periodic copy J = NT <- 1, the
    magnetopause mask, DtsNext, ANISCH and FLUX.  Returns new F2 arrays and
    the outputs."""
    f = Fld(fields)
    vt = vt_vols(g, kp) if vt is None else np.asarray(vt, dtype=np.float64)
    out = {"f2": [], "ppert": [], "ppart": [], "flux": [], "dt": []}
    for s in range(len(g.species)):
        x = np.asarray(f2s[s], dtype=np.float64)
        charge, atlos = cepara(g, f, s, dts)
        cex = g.species[s].cex_kind in CEX_POLY
        x, _, dtr = drift_r(g, f, s, x, fgeos[s], dts, vt, beta, fraccfl)
        x, _, dtp = drift_p(g, f, s, x, dts, vt, beta, fraccfl)
        x, _, dte = drift_e(g, f, s, x, dts, vt, beta, fraccfl)
        x, _, dtm = drift_mu(g, f, s, x, dts, vt, beta, fraccfl)
        if cex:
            x = charexchange(g, x, charge)
        if do_atmol:
            x = atmol(g, f, x, atlos)
            x = atmol(g, f, x, atlos)
        if cex:
            x = charexchange(g, x, charge)
        x, _, _ = drift_mu(g, f, s, x, dts, vt, beta, fraccfl)
        x, _, _ = drift_e(g, f, s, x, dts, vt, beta, fraccfl)
        x, _, _ = drift_p(g, f, s, x, dts, vt, beta, fraccfl)
        x, _, _ = drift_r(g, f, s, x, fgeos[s], dts, vt, beta, fraccfl)
        out["f2"].append(x)
        out["dt"].append((dtr, dtp, dte, dtm))
    for s in range(len(g.species)):
        x = out["f2"][s]
        x[:, g.nt - 1] = x[:, 0]
        x[f.outside == 1] = 1.e-31
    dn = min(min(d) for d in out["dt"])
    out["dts_next"] = max(dn, dtsmin)
    for s in range(len(g.species)):
        x, pe, pa = anisch(g, f, s, out["f2"][s])
        out["f2"][s] = x
        out["ppert"].append(pe)
        out["ppart"].append(pa)
        out["flux"].append(flux(g, f, s, x))
    out["vt"] = vt
    return out
