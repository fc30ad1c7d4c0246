"""ctypes binding of the CPU oracle (oracle/ram_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU legs, never by the product.  The oracle equals the
reference's own routines bit for bit (they run here translated from the
Fortran by oracle/f90c.py, oracle/refrun.py); see ram_oracle.h.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess
from pathlib import Path

import numpy as np

ORACLE_DIR = Path(__file__).resolve().parent
LIB_PATH = ORACLE_DIR / "liboracle.so"

_P = C.POINTER(C.c_double)
_IP = C.POINTER(C.c_int)


class RoGrid(C.Structure):
    _fields_ = [("nr", C.c_int), ("nt", C.c_int), ("ne", C.c_int), ("npa", C.c_int),
                ("lz", _P), ("rlz", _P), ("phi", _P),
                ("dl1", C.c_double), ("mdr", C.c_double), ("dphi", C.c_double),
                ("conf1", C.c_double), ("conf2", C.c_double),
                ("ekev", _P), ("ebnd", _P), ("we", _P), ("de", _P),
                ("mu", _P), ("dmu", _P), ("wmu", _P), ("upa", _P),
                ("fnhs", _P), ("fnis", _P), ("bounhs", _P), ("bounis", _P), ("hdns", _P),
                ("didt", _P), ("dibndt", _P), ("bnes", _P), ("dbdt", _P), ("eir", _P), ("eip", _P),
                ("outside_mgnp", _IP)]


class RoSpecies(C.Structure):
    _fields_ = [("qs", C.c_int), ("cex_kind", C.c_int), ("rmas", C.c_double),
                ("grel", _P), ("grbnd", _P), ("v", _P), ("ffactor", _P), ("epp", _P), ("ernh", _P)]


class RoParams(C.Structure):
    _fields_ = [("betalim", C.c_double), ("fraccfl", C.c_double), ("dts", C.c_double),
                ("dtsmin", C.c_double), ("closed", C.c_int), ("do_atmol", C.c_int)]


class RoDriftPara(C.Structure):
    _fields_ = [("vr", _P), ("p1", _P), ("p2", _P), ("edot", _P), ("mudot", _P)]


class RoLosses(C.Structure):
    _fields_ = [("setrc", C.c_double), ("lsdr", C.c_double), ("lscha", C.c_double),
                ("lsatm", C.c_double), ("lswae", C.c_double)]


def build(force: bool = False) -> Path:
    src = ORACLE_DIR / "ram_oracle.c"
    if force or not LIB_PATH.exists() or LIB_PATH.stat().st_mtime < src.stat().st_mtime:
        cc = os.environ.get("CC", "gcc")
        subprocess.run([cc, "-O3", "-ffp-contract=off", "-fPIC", "-fopenmp", "-std=c11", "-shared",
                        "-o", str(LIB_PATH), str(src), "-lm"], check=True)
    return LIB_PATH


_lib = None


def load():
    global _lib
    if _lib is None:
        build()
        lib = C.CDLL(str(LIB_PATH))
        gp, sp, pp = C.POINTER(RoGrid), C.POINTER(RoSpecies), C.POINTER(RoParams)
        dpp = C.POINTER(RoDriftPara)
        lib.ro_set_inner_threads.argtypes = [C.c_int]
        lib.ro_vt_vols.argtypes = [gp, C.c_double, _P]
        lib.ro_driftpara.argtypes = [gp, sp, pp, dpp]
        lib.ro_driftr.argtypes = [gp, sp, pp, dpp, _P, _P, _P, _P]
        lib.ro_driftr.restype = C.c_double
        for n in ("ro_driftp", "ro_drifte", "ro_driftmu"):
            f = getattr(lib, n)
            f.argtypes = [gp, sp, pp, dpp, _P, _P, _P]
            f.restype = C.c_double
        lib.ro_cepara.argtypes = [gp, sp, pp, _P, _P]
        lib.ro_charexchange.argtypes = [gp, _P, _P]
        lib.ro_atmol.argtypes = [gp, _P, _P]
        lib.ro_sumrc.argtypes = [gp, _P]
        lib.ro_sumrc.restype = C.c_double
        lib.ro_anisch.argtypes = [gp, sp, _P, _P, _P]
        lib.ro_flux.argtypes = [gp, sp, _P, _P]
        PP = C.POINTER(_P)
        lib.ro_ram_run.argtypes = [gp, C.c_int, sp, pp, C.c_double, _P, _P, PP, PP, PP, PP, PP,
                                   C.POINTER(RoLosses), _P, C.c_int]
        lib.ro_half_step.argtypes = [gp, sp, pp, dpp, _P, _P, _P, _P, _P, C.c_int]
        lib.ro_ram_run2.argtypes = [gp, C.c_int, sp, pp, C.c_double, _P, _P, PP, PP, PP, PP, PP,
                                    C.POINTER(RoLosses), _P, C.c_int, PP]
        lib.ro_padif.argtypes = [gp, pp, _P, _P]
        lib.ro_bounce_integrals.argtypes = [gp, C.c_int, _P, _P, _P, _P, _P, _P, C.c_int, _P, _P, _P, _P]
        lib.ro_install_hI.argtypes = [gp, _P, _P, _P, _P, _P, _P, C.c_double, C.c_double] + [_P] * 11
        U8 = C.POINTER(C.c_ubyte)
        lib.ro_driftr_rec.argtypes = [gp, sp, pp, dpp, _P, _P, _P, _P, U8, _IP]
        lib.ro_driftr_rec.restype = C.c_double
        for n in ("ro_driftp_rec", "ro_drifte_rec", "ro_driftmu_rec"):
            f = getattr(lib, n)
            f.argtypes = [gp, sp, pp, dpp, _P, _P, _P, U8]
            f.restype = C.c_double
        lib.ro_driftr_adj.argtypes = [gp, pp, _P, U8, _IP, _P, _P]
        lib.ro_driftp_adj.argtypes = [gp, pp, _P, U8, _P]
        lib.ro_drifte_adj.argtypes = [gp, sp, pp, _P, U8, _P]
        lib.ro_driftmu_adj.argtypes = [gp, pp, _P, U8, _P]
        _lib = lib
    return _lib


def set_inner_threads(n: int):
    """Threads for the independent-line loops inside each oracle routine."""
    load().ro_set_inner_threads(int(n))


def _f(a, dtype=np.float64):
    return np.asfortranarray(np.asarray(a, dtype=dtype))


def _p(a):
    return a.ctypes.data_as(_P) if a is not None else None


def _u8(a):
    return a.ctypes.data_as(C.POINTER(C.c_ubyte))


def _ip(a):
    return a.ctypes.data_as(_IP)


def obs_cells(grid, o):
    """Bilinear (L-shell, MLT) stencil of one observation: four (i, j, weight)
    over I >= 2 (0-based i >= 1) with J = NT folded onto J = 1."""
    lz, nr, nt, dphi = grid.lz, grid.nr, grid.nt, grid.dphi
    i0 = 1
    while i0 + 1 < nr - 1 and lz[i0 + 1] <= o["lshell"]:
        i0 += 1
    wi = min(1.0, max(0.0, (o["lshell"] - lz[i0]) / (lz[i0 + 1] - lz[i0])))
    ph = math.fmod(o["mlt"] * math.pi / 12.0, 2 * math.pi)
    if ph < 0:
        ph += 2 * math.pi
    j0 = min(int(ph / dphi), nt - 2)
    j1 = 0 if j0 + 1 == nt - 1 else j0 + 1
    wj = min(1.0, max(0.0, (ph - grid.phi[j0]) / dphi))
    return [(i0 + a, j1 if b else j0, (wi if a else 1 - wi) * (wj if b else 1 - wj))
            for a in (0, 1) for b in (0, 1)]


class Oracle:
    """CPU restatement of the reference routines for one grid and field set.

    F2 arrays are Fortran-ordered (NR,NT,NE,NPA) float64 and are updated in
    place."""

    def __init__(self, grid, fields, betalim=1.5, fraccfl=0.8, dtsmin=0.1):
        self.lib = load()
        self.grid = grid
        self.ns = len(grid.species)
        self.betalim, self.fraccfl, self.dtsmin = betalim, fraccfl, dtsmin
        g = grid
        self._keep = {}

        def keep(name, a, dtype=np.float64):
            arr = _f(a, dtype)
            self._keep[name] = arr
            return arr

        rg = RoGrid()
        rg.nr, rg.nt, rg.ne, rg.npa = g.nr, g.nt, g.ne, g.npa
        for k in ("lz", "rlz", "phi", "ekev", "ebnd", "we", "de", "mu", "dmu", "wmu", "upa"):
            setattr(rg, k, _p(keep(k, getattr(g, k))))
        rg.dl1, rg.mdr, rg.dphi, rg.conf1, rg.conf2 = g.dl1, g.mdr, g.dphi, g.conf1, g.conf2
        for k in ("fnhs", "fnis", "bounhs", "bounis", "hdns", "didt", "dibndt", "bnes", "dbdt", "eir", "eip"):
            setattr(rg, k, _p(keep("f_" + k, getattr(fields, k))))
        rg.outside_mgnp = keep("outside", fields.outside, np.int32).ctypes.data_as(_IP)
        self.rg = rg
        self.sp = (RoSpecies * self.ns)()
        for s, spc in enumerate(g.species):
            o = self.sp[s]
            o.qs, o.cex_kind, o.rmas = spc.charge, spc.cex_kind, g.rmas[s]
            o.grel = _p(keep(f"grel{s}", g.grel[s]))
            o.grbnd = _p(keep(f"grbnd{s}", g.grbnd[s]))
            o.v = _p(keep(f"v{s}", g.v[s]))
            o.ffactor = _p(keep(f"ff{s}", g.ffactor[s]))
            o.epp = _p(keep(f"epp{s}", g.epp[s]))
            o.ernh = _p(keep(f"ernh{s}", g.ernh[s]))

    def params(self, dts, closed=False, do_atmol=True):
        return RoParams(self.betalim, self.fraccfl, float(dts), self.dtsmin, int(closed), int(do_atmol))

    def vt_vols(self, kp):
        vt = np.zeros((self.grid.nr + 1, self.grid.nt), order="F")
        self.lib.ro_vt_vols(C.byref(self.rg), float(kp), _p(vt))
        return vt

    def driftpara(self, s, dts):
        g = self.grid
        dp = {"vr": np.zeros(g.nr), "p1": np.zeros(g.nr), "p2": np.zeros((g.nr, g.ne), order="F"),
              "edot": np.zeros((g.nr, g.ne), order="F"), "mudot": np.zeros((g.nr, g.npa), order="F")}
        st = RoDriftPara(*[_p(dp[k]) for k in ("vr", "p1", "p2", "edot", "mudot")])
        p = self.params(dts)
        self.lib.ro_driftpara(C.byref(self.rg), C.byref(self.sp[s]), C.byref(p), C.byref(st))
        dp["_struct"] = st
        return dp

    def sweep(self, which, s, f2, vt, dts, fgeos=None, closed=False, cdrift=None):
        """Run one DRIFT* routine on f2 (Fortran array, in place); returns DtDrift*."""
        dp = self.driftpara(s, dts)
        p = self.params(dts, closed)
        args = [C.byref(self.rg), C.byref(self.sp[s]), C.byref(p), C.byref(dp["_struct"]), _p(vt)]
        cd = _p(cdrift) if cdrift is not None else None
        if which == "R":
            fg = _f(fgeos if fgeos is not None else np.zeros((self.grid.nt, self.grid.ne, self.grid.npa)))
            return self.lib.ro_driftr(*args, _p(fg), _p(f2), cd)
        fn = {"P": self.lib.ro_driftp, "E": self.lib.ro_drifte, "MU": self.lib.ro_driftmu}[which]
        return fn(*args, _p(f2), cd)

    def padif(self, f2, daa, dts):
        """WPADIF / FLCscatter on one species (Fortran array, in place)."""
        p = self.params(dts)
        self.lib.ro_padif(C.byref(self.rg), C.byref(p), _p(_f(daa)), _p(f2))

    def bounce_integrals(self, lines):
        """computehI's bounce integrals on field lines (workload.FieldLines):
        (H_cart, I_cart, HDens_cart, mirror B), each (NR, NT, NPA)."""
        g = self.grid
        shp = (g.nr, g.nt, g.npa)
        h, fi, hd, bm = (np.zeros(shp, order="F") for _ in range(4))
        b = _f(lines.b).copy(order="F")
        self.lib.ro_bounce_integrals(C.byref(self.rg), int(lines.chi.size), _p(_f(lines.chi)), _p(_f(lines.x)),
                                     _p(_f(lines.y)), _p(_f(lines.z)), _p(b), _p(_f(lines.dens)),
                                     int(lines.ieq), _p(h), _p(fi), _p(hd), _p(bm))
        return h, fi, hd, bm

    def compute_hI(self, lines, bnormal=1.0, dthi=0.0, fields=None):
        """computehI's integrals and RAM-variable fill: a dict of new field
        tables (as Fields, Fortran order) starting from ``fields`` (default
        this oracle's).  The oracle's own fields are left unchanged."""
        g = self.grid
        h, fi, hd, bm = self.bounce_integrals(lines)
        beq = _f(bm[:, :, 0])
        src = fields if fields is not None else {k[2:]: v for k, v in self._keep.items() if k.startswith("f_")}
        out = {k: _f(src[k]).copy(order="F") for k in ("fnhs", "fnis", "hdns", "bounhs", "bounis", "bnes", "dbdt",
                                                       "didt", "dibndt", "eir", "eip")}
        self.lib.ro_install_hI(C.byref(self.rg), _p(_f(g.pa)), _p(_f(g.pabn)), _p(h), _p(fi), _p(hd), _p(beq),
                               float(bnormal), float(dthi),
                               *[_p(out[k]) for k in ("fnhs", "fnis", "hdns", "bounhs", "bounis", "bnes", "dbdt",
                                                      "didt", "dibndt", "eir", "eip")])
        return out

    def cepara(self, s, dts, do_atmol=True):
        g = self.grid
        charge = np.zeros((g.nr, g.nt, g.ne, g.npa), order="F")
        atlos = np.zeros((g.nr, g.ne), order="F")
        p = self.params(dts, do_atmol=do_atmol)
        self.lib.ro_cepara(C.byref(self.rg), C.byref(self.sp[s]), C.byref(p), _p(charge), _p(atlos))
        return charge, atlos

    def sumrc(self, f2):
        return self.lib.ro_sumrc(C.byref(self.rg), _p(f2))

    def anisch(self, s, f2):
        g = self.grid
        pe = np.zeros((g.nr, g.nt), order="F")
        pa = np.zeros((g.nr, g.nt), order="F")
        self.lib.ro_anisch(C.byref(self.rg), C.byref(self.sp[s]), _p(f2), _p(pe), _p(pa))
        return pe, pa

    def flux(self, s, f2):
        g = self.grid
        out = np.zeros((g.nr, g.nt, g.ne, g.npa), order="F")
        self.lib.ro_flux(C.byref(self.rg), C.byref(self.sp[s]), _p(f2), _p(out))
        return out

    def half_step(self, s, f2, vt, fgeos, dts, order, closed=False, do_atmol=True):
        dp = self.driftpara(s, dts)
        p = self.params(dts, closed, do_atmol)
        charge, atlos = self.cepara(s, dts, do_atmol)
        self.lib.ro_half_step(C.byref(self.rg), C.byref(self.sp[s]), C.byref(p), C.byref(dp["_struct"]),
                              _p(vt), _p(_f(fgeos)), _p(charge), _p(atlos), _p(f2), int(order))

    def ram_run(self, f2s, fgeos, dts, kp=None, vt=None, closed=False, do_atmol=True,
                losses=None, want_flux=False, nthreads=1, species=None, daa=None):
        """One ram_run call over the species in ``species`` (default all);
        f2s/fgeos are lists indexed by species.  daa: optional {species:
        pitch-angle diffusion coefficient (NR,NT,NE,NPA)}, applied as WPADIF
        on both sides of the loss processes."""
        g = self.grid
        idx = list(range(self.ns)) if species is None else list(species)
        n = len(idx)
        sp_arr = (RoSpecies * n)(*[self.sp[s] for s in idx])
        p = self.params(dts, closed, do_atmol)
        fg = [_f(fgeos[s]) for s in idx]
        for s in idx:
            assert f2s[s].flags["F_CONTIGUOUS"] and f2s[s].dtype == np.float64
        PArr = _P * n
        pe = [np.zeros((g.nr, g.nt), order="F") for _ in idx]
        pa = [np.zeros((g.nr, g.nt), order="F") for _ in idx]
        fl = [np.zeros((g.nr, g.nt, g.ne, g.npa), order="F") for _ in idx] if want_flux else None
        vt_out = np.zeros((g.nr + 1, g.nt), order="F")
        vt_in = _f(vt) if vt is not None else None
        ls = (RoLosses * n)()
        if losses is not None:
            for t, s in enumerate(idx):
                ls[t].setrc, ls[t].lsdr, ls[t].lscha, ls[t].lsatm = losses[s]
        dn = C.c_double()
        dl = [_f(daa[s]) if daa is not None and s in daa else None for s in idx]
        self.lib.ro_ram_run2(C.byref(self.rg), n, sp_arr, C.byref(p), float(kp if kp is not None else 0.0),
                             _p(vt_in), _p(vt_out), PArr(*[_p(a) for a in fg]),
                             PArr(*[_p(f2s[s]) for s in idx]), PArr(*[_p(a) for a in pe]),
                             PArr(*[_p(a) for a in pa]), PArr(*[_p(a) for a in fl]) if fl else None,
                             ls, C.byref(dn), int(nthreads), PArr(*[_p(a) for a in dl]))
        out = {"vt": vt_out, "ppert": dict(zip(idx, pe)), "ppart": dict(zip(idx, pa)),
               "dts_next": dn.value,
               "losses": {s: (ls[t].setrc, ls[t].lsdr, ls[t].lscha, ls[t].lsatm) for t, s in enumerate(idx)},
               "lswae": {s: ls[t].lswae for t, s in enumerate(idx)}}
        if fl:
            out["flux"] = dict(zip(idx, fl))
        return out

    # ------------------------------------------------------------- adjoint
    _REC = {"R": "ro_driftr_rec", "P": "ro_driftp_rec", "E": "ro_drifte_rec", "MU": "ro_driftmu_rec"}

    def sweep_rec(self, which, s, f2, vt, dts, fgeos=None, closed=False):
        """One DRIFT* routine (in place) that also records its frozen branches.
        Returns a tape entry (which, s, cdrift, rec, gsrc|None)."""
        g = self.grid
        shape = (g.nr, g.nt, g.ne, g.npa)
        dp = self.driftpara(s, dts)
        p = self.params(dts, closed)
        cd = np.zeros(shape, order="F")
        rec = np.zeros(shape, dtype=np.uint8, order="F")
        args = [C.byref(self.rg), C.byref(self.sp[s]), C.byref(p), C.byref(dp["_struct"]), _p(vt)]
        if which == "R":
            gsrc = np.full((g.nt, g.ne, g.npa), -1, dtype=np.int32, order="F")
            self.lib.ro_driftr_rec(*args, _p(_f(fgeos)), _p(f2), _p(cd), _u8(rec), _ip(gsrc))
            return ("R", s, cd, rec, gsrc)
        getattr(self.lib, self._REC[which])(*args, _p(f2), _p(cd), _u8(rec))
        return (which, s, cd, rec, None)

    def sweep_adj(self, tape, lam, dts, gfgeos=None, closed=False):
        """Transpose of a recorded sweep applied to lam (Fortran, in place);
        DRIFTR adds its FGEOS gradient into gfgeos."""
        which, s, cd, rec, gsrc = tape
        p = self.params(dts, closed)
        rg = C.byref(self.rg)
        if which == "R":
            self.lib.ro_driftr_adj(rg, C.byref(p), _p(cd), _u8(rec), _ip(gsrc), _p(lam), _p(gfgeos))
        elif which == "P":
            self.lib.ro_driftp_adj(rg, C.byref(p), _p(cd), _u8(rec), _p(lam))
        elif which == "E":
            self.lib.ro_drifte_adj(rg, C.byref(self.sp[s]), C.byref(p), _p(cd), _u8(rec), _p(lam))
        else:
            self.lib.ro_driftmu_adj(rg, C.byref(p), _p(cd), _u8(rec), _p(lam))

    def loss_factor(self, s, dts, do_atmol=True):
        """Per-cell factor of CHAREXCHANGE, ATMOL, ATMOL, CHAREXCHANGE as
        ram_run applies them between the two sweep halves."""
        g = self.grid
        charge, atlos = self.cepara(s, dts, do_atmol)
        at = np.ones((g.nr, g.nt, g.ne, g.npa), order="F")
        if do_atmol:
            self.lib.ro_atmol(C.byref(self.rg), _p(at), _p(atlos))
        ch = charge if self.grid.species[s].cex_kind else np.ones_like(at)
        return ch, at

    def window_gradient(self, f2s, fgeos, dts, kps, obs, species=None, closed=False, do_atmol=True,
                        records=None, states=None):
        """Scalar adjoint of a window of len(kps) ram_run calls for one member.

        J = sum over obs of (log flux - log_obs)^2 with flux = F2/FFACTOR/FNHS
        (src/ModRamRun.f90:214) after call o["call"], bilinear in (L-shell,
        MLT) at 0-based bins (o["k"], o["l"]).  Forward: the reference call
        sequence of ram_run (src/ModRamRun.f90:77-225) with every sweep
        recorded; backward: the transposes in reverse order.  f2s is not
        modified.  With ``records`` a list, each call's branch record is
        appended as an (8 sweeps, species, NR*NT*NE*NPA) uint8 array; with
        ``states`` a list, each call's starting F2 as (species, NR*NT*NE*NPA).
        Returns (J, {s: dJ/dF2}, {s: dJ/dFGEOS})."""
        g = self.grid
        idx = list(range(self.ns)) if species is None else list(species)
        f = {s: np.array(f2s[s], dtype=np.float64, order="F", copy=True) for s in idx}
        fg = {s: _f(fgeos[s]) for s in idx}
        fac = {s: self.loss_factor(s, dts, do_atmol) for s in idx}
        out = np.asarray(self._keep["outside"]) == 1
        fnhs = self._keep["f_fnhs"]
        tapes, fm = [], {}
        J = 0.0
        for c, kp in enumerate(kps):
            vt = self.vt_vols(kp)
            tc = {}
            if states is not None:
                states.append(np.stack([f[s].reshape(-1, order="F").copy() for s in idx]))
            for s in idx:
                t = [self.sweep_rec("R", s, f[s], vt, dts, fg[s], closed),
                     self.sweep_rec("P", s, f[s], vt, dts, closed=closed),
                     self.sweep_rec("E", s, f[s], vt, dts, closed=closed),
                     self.sweep_rec("MU", s, f[s], vt, dts, closed=closed)]
                ch, at = fac[s]
                f[s] *= ch
                f[s] *= at
                f[s] *= at
                f[s] *= ch
                t += [self.sweep_rec("MU", s, f[s], vt, dts, closed=closed),
                      self.sweep_rec("E", s, f[s], vt, dts, closed=closed),
                      self.sweep_rec("P", s, f[s], vt, dts, closed=closed),
                      self.sweep_rec("R", s, f[s], vt, dts, fg[s], closed)]
                tc[s] = t
                f[s][:, g.nt - 1] = f[s][:, 0]
                f[s][out] = 1e-31
                self.anisch(s, f[s])
            tapes.append(tc)
            if records is not None:
                records.append(np.stack([np.stack([tc[s][q][3].reshape(-1, order="F") for s in idx])
                                         for q in range(8)]))
            for n, o in enumerate(obs):
                if o["call"] != c:
                    continue
                ff = np.asarray(self.grid.ffactor[o["s"]])
                v = sum(w * (f[o["s"]][i, j, o["k"], o["l"]] / ff[i, o["k"], o["l"]] / fnhs[i, j, o["l"]])
                        for i, j, w in obs_cells(g, o))
                fm[n] = v
                J += (math.log(v) - o["log_obs"]) ** 2
        lam = {s: np.zeros((g.nr, g.nt, g.ne, g.npa), order="F") for s in idx}
        gfg = {s: np.zeros((g.nt, g.ne, g.npa), order="F") for s in idx}
        for c in range(len(kps) - 1, -1, -1):
            for n, o in enumerate(obs):
                if o["call"] != c:
                    continue
                v = fm[n]
                gr = 2.0 * (math.log(v) - o["log_obs"]) / v
                ff = np.asarray(self.grid.ffactor[o["s"]])
                for i, j, w in obs_cells(g, o):
                    lam[o["s"]][i, j, o["k"], o["l"]] += gr * w / (ff[i, o["k"], o["l"]] * fnhs[i, j, o["l"]])
            for s in idx:
                lm = lam[s]
                # ANISCH: F2(I,J,K,1) = F2(I,J,K,2), I >= 2, K >= 2
                lm[1:, :, 1:, 1] += lm[1:, :, 1:, 0]
                lm[1:, :, 1:, 0] = 0.0
                lm[out] = 0.0
                lm[:, 0] += lm[:, g.nt - 1]
                lm[:, g.nt - 1] = 0.0
                t = tapes[c][s]
                for e in t[7:3:-1]:
                    self.sweep_adj(e, lm, dts, gfg[s], closed)
                ch, at = fac[s]
                lm *= ch
                lm *= at
                lm *= at
                lm *= ch
                for e in t[3::-1]:
                    self.sweep_adj(e, lm, dts, gfg[s], closed)
            tapes[c] = None
        return J, lam, gfg


# ----------------------------------------------------------- output products
BAD_DATA = -1.0E10  # BadDataFlag, src/ModRamSats.f90:35


def sat_samples(grid, flux, sats, species_of=None):
    """Virtual-spacecraft samples restated from fly_sats' flux block
    (src/ModRamSats.f90:640-666) on the equatorial RAM grid: SatFlux(S,E,PA)
    bilinear in (R, MLT) over the FLUX cells of obs_cells (BadDataFlag unless
    all four corners are > 0) and OmnFlux(S,E) = sum_PA SatFlux*4*pi*WMU for
    SatFlux > 0 (BadDataFlag if not > 0).  flux: {s: FLUX (NR,NT,NE,NPA)};
    sats: [(member, lshell, mlt)]; species_of: {member: species list}."""
    ns, ne, npa = len(grid.species), grid.ne, grid.npa
    wmu = np.asarray(grid.wmu)
    sf = np.full((len(sats), ns, ne, npa), BAD_DATA)
    om = np.full((len(sats), ns, ne), BAD_DATA)
    for t, (m, lsh, mlt) in enumerate(sats):
        cells = obs_cells(grid, {"lshell": lsh, "mlt": mlt})
        for s in range(ns):
            if species_of is not None and s not in species_of[m]:
                continue
            acc = np.zeros((ne, npa))
            pos = np.ones((ne, npa), dtype=bool)
            for i, j, w in cells:
                fl = np.asarray(flux[s])[i, j]
                pos &= fl > 0.0
                acc = acc + w * fl
            v = np.where(pos, acc, BAD_DATA)
            v[0, :] = BAD_DATA
            v[:, 0] = BAD_DATA
            sf[t, s] = v
            o = np.zeros(ne)
            for l in range(npa):
                o = np.where(v[:, l] > 0.0, o + v[:, l] * 4.0 * math.pi * wmu[l], o)
            om[t, s] = np.where(o > 0.0, o, BAD_DATA)
    return sf, om


def sum_pressure(ppert, ppart, species):
    """ram_sum_pressure (src/ModRamFunctions.f90:272-297) over `species`:
    PAllSum = sum_S 2/3 PPERT + 1/3 PPART, PParSum = sum_S PPART."""
    onethird, twothird = 1.0 / 3.0, 2.0 / 3.0
    pall = np.zeros_like(ppert[species[0]])
    ppar = np.zeros_like(ppart[species[0]])
    for s in species:
        pall = pall + twothird * ppert[s] + onethird * ppart[s]
        ppar = ppar + ppart[s]
    return pall, ppar
