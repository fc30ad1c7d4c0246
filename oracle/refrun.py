"""Harness of the translated reference: RAM's own kinetic-step routines.

TEST INFRASTRUCTURE ONLY: imported by tests/, tests/golden/make_ref_golden.py
and bench.py's reference arm, never by the product.

``oracle/f90c.py`` translates the reference's Fortran source files
(src/ModRamDrift.f90, src/ModRamLoss.f90, src/ModRamRun.f90 and the modules
they use) into ``oracle/_ref/ramref.c``; gcc builds it into
``oracle/_ref/libramref.so``.  This module fills the reference's module
variables from a workload as RAM's initialisation would (the array shapes
of ram_allocate, src/ModRamInit.f90:68-146; the species table of
ModRamSpecies through oracle/refdriver.f90) and calls the reference's own
``ram_run`` (src/ModRamRun.f90:16-225): VT from VOLS, CEPARA, DRIFTPARA,
the Strang-ordered sweeps, CHAREXCHANGE, ATMOL, SUMRC, the mask, DtsNext,
ANISCH and FLUX, in the reference's loop order and arithmetic.

Configuration: every process flag of src/ModRamParams.f90 keeps its default
(plasmasphere, Coulomb, WPI, EMIC and FLC off; electric field 'VOLS'), and
each species' WPI and EMIC switches are off (the electron WAVELO lifetimes
and the EMIC scattering are outside the kinetic step).  COULPARA, which
ram_run calls unconditionally but whose results only the (off) Coulomb
processes read, is the one procedure left as a counted no-op stub.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys
from pathlib import Path

import numpy as np

ORACLE_DIR = Path(__file__).resolve().parent
REF_DIR = ORACLE_DIR / "_ref"
C_PATH = REF_DIR / "ramref.c"
LIB_PATH = REF_DIR / "libramref.so"
LIB_CHECK_PATH = REF_DIR / "libramref_check.so"
DRIVER = ORACLE_DIR / "refdriver.f90"

# RAMSpecies index of each species name (src/ModRamSpecies.f90:43-130)
SPECIES_INDEX = {"Electron": 1, "Hydrogen": 2, "HeliumP1": 3, "OxygenP1": 4, "Nitrogen": 5, "Strontium": 6}
# the only stub ram_run may call with this configuration
ALLOWED_STUBS = {"coulpara"}


def ref_root():
    """The reference's source tree when it is present on this machine."""
    r = Path(os.environ.get("RAM_REF_ROOT", "/root/reference"))
    return r if (r / "src" / "ModRamDrift.f90").exists() else None


def build(force: bool = False):
    """Translate the reference (where its tree is present) and compile.
    Returns the library path, or None when neither the tree nor a
    translated C file is available."""
    sys.path.insert(0, str(ORACLE_DIR))
    import f90c  # noqa: E402
    root = ref_root()
    if root is not None:
        deps = [Path(f90c.__file__), DRIVER] + [root / f for f in f90c.REF_FILES]
        if force or not C_PATH.exists() or C_PATH.stat().st_mtime < max(d.stat().st_mtime for d in deps):
            f90c.translate(str(root), str(REF_DIR), [str(DRIVER)])
    if not C_PATH.exists():
        return None
    for lib, chk in ((LIB_PATH, False), (LIB_CHECK_PATH, True)):
        if force or not lib.exists() or lib.stat().st_mtime < C_PATH.stat().st_mtime:
            f90c.compile_c(C_PATH, lib, check=chk)
    return LIB_PATH


class RefArr(C.Structure):
    _fields_ = [("p", C.c_void_p), ("esz", C.c_int), ("rank", C.c_int),
                ("lb", C.c_long * 7), ("ub", C.c_long * 7), ("sm", C.c_long * 7)]


_libs = {}


def load(check: bool = False):
    key = bool(check)
    if key not in _libs:
        if build() is None:
            raise FileNotFoundError("translated reference unavailable: no reference tree and no oracle/_ref/ramref.c")
        lib = C.CDLL(str(LIB_CHECK_PATH if check else LIB_PATH), mode=getattr(C, "RTLD_LOCAL", 0))
        _sigs(lib)
        _libs[key] = lib
    return _libs[key]


class RefLib:
    """Accessors of a translated library: module variables by
    "module::name", integer-argument procedures by name."""

    def __init__(self, lib):
        self.lib = lib

    @classmethod
    def open(cls, path):
        lib = C.CDLL(str(path), mode=getattr(C, "RTLD_LOCAL", 0))
        _sigs(lib)
        lib.ref_init()
        return cls(lib)

    def _addr(self, name):
        b, r, e = C.c_int(), C.c_int(), C.c_int()
        p = self.lib.ref_addr(name.encode(), C.byref(b), C.byref(r), C.byref(e))
        if not p:
            raise KeyError(f"{name} is not a variable of the translated code")
        return p, b.value, r.value, e.value

    def set(self, name, value):
        p, b, r, e = self._addr(name)
        if r:
            raise TypeError(f"{name} is an array")
        if b == 1:
            C.c_double.from_address(p).value = float(value)
        elif b in (0, 2):
            C.c_int.from_address(p).value = int(value)
        else:
            raise TypeError(f"{name}: unsupported type")

    def set_str(self, name, value):
        """A character variable, blank-padded to its length."""
        p, b, r, e = self._addr(name)
        if b != 3 or r:
            raise TypeError(f"{name} is not a character scalar")
        raw = value.encode()[:e].ljust(e, b" ")
        C.memmove(p, raw, e)

    def get(self, name):
        p, b, r, e = self._addr(name)
        if r:
            return self.view(name)
        if b == 1:
            return C.c_double.from_address(p).value
        if b == 3:
            return C.string_at(p, e).decode()
        return C.c_int.from_address(p).value

    def alloc(self, name, shape, lb=None):
        lb = (C.c_long * len(shape))(*([1] * len(shape) if lb is None else lb))
        ub = (C.c_long * len(shape))(*[lb[k] + shape[k] - 1 for k in range(len(shape))])
        if self.lib.ref_alloc_var(name.encode(), len(shape), lb, ub) != 0:
            raise RuntimeError(f"allocating {name}: {self.lib.ref_error().decode()}")
        return self.view(name)

    def view(self, name):
        """numpy view (Fortran order) of an allocated array variable."""
        p, b, r, e = self._addr(name)
        d = RefArr.from_address(p)
        if not d.p:
            raise RuntimeError(f"{name} is not allocated")
        shape = tuple(int(d.ub[k] - d.lb[k] + 1) for k in range(d.rank))
        n = int(np.prod(shape))
        ct = {0: C.c_int, 1: C.c_double, 2: C.c_int}[b]
        buf = (ct * n).from_address(d.p)
        return np.ctypeslib.as_array(buf).reshape(shape, order="F")

    def call(self, name, *args):
        """Call a procedure with integer arguments; returns the arguments
        after the call (intent(out)/(inout) values)."""
        arr = (C.c_int * max(1, len(args)))(*args)
        rc = self.lib.ref_call(name.encode(), len(args), arr)
        if rc != 0:
            raise RuntimeError(f"{name}: rc {rc}: {self.lib.ref_error().decode()}")
        return list(arr)[:len(args)]

    def call_rc(self, name, *args):
        arr = (C.c_int * max(1, len(args)))(*args)
        rc = self.lib.ref_call(name.encode(), len(args), arr)
        return rc, self.lib.ref_error().decode()

    def stubs(self):
        return {self.lib.ref_stub_name(i).decode(): self.lib.ref_stub_count(i) for i in range(self.lib.ref_nstubs())}


def _sigs(lib):
    lib.ref_init.restype = C.c_int
    lib.ref_addr.restype = C.c_void_p
    lib.ref_addr.argtypes = [C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]
    lib.ref_alloc_var.argtypes = [C.c_char_p, C.c_int, C.POINTER(C.c_long), C.POINTER(C.c_long)]
    lib.ref_call.argtypes = [C.c_char_p, C.c_int, C.POINTER(C.c_int)]
    lib.ref_error.restype = C.c_char_p
    lib.ref_stub_name.restype = C.c_char_p
    lib.ref_stub_count.restype = C.c_long
    lib.ref_threads.argtypes = [C.c_int]


class RefRam(RefLib):
    """The reference's module state for one grid and field set.

    One instance at a time per library (the reference keeps its state in
    module variables); creating an instance resets that state."""

    def __init__(self, grid, fields, betalim=1.5, fraccfl=0.8, dtsmin=0.1, check=False, threads=1):
        super().__init__(load(check))
        self.grid = grid
        g = grid
        self.ns = ns = len(g.species)
        self.lib.ref_init()
        self.lib.ref_threads(int(threads))
        for k, v in (("ns", ns), ("nr", g.nr), ("nt", g.nt), ("ne", g.ne), ("npa", g.npa)):
            self.set("modramgrids::" + k, v)
        self.call("refdrv_species_begin", ns)
        for i, sp in enumerate(g.species, 1):
            self.call("refdrv_species_set", i, SPECIES_INDEX[sp.name])
            q = self._charge(i)
            if q != sp.charge:
                raise ValueError(f"species {sp.name}: charge {q} in the reference table, {sp.charge} in the grid")
        nr, nt, ne, npa = g.nr, g.nt, g.ne, g.npa
        slen = self.get("modramgrids::slen")
        # shapes of ram_allocate (src/ModRamInit.f90:68-146)
        shapes = {
            "f2": (ns, nr, nt, ne, npa), "flux": (ns, nr, nt, ne, npa), "charge": (ns, nr, nt, ne, npa),
            "ppert": (ns, nr, nt), "ppart": (ns, nr, nt),
            "fnhs": (nr + 1, nt, npa), "fnis": (nr + 1, nt, npa), "bounhs": (nr + 1, nt, npa),
            "bounis": (nr + 1, nt, npa), "didt": (nr + 1, nt, npa), "dibndt": (nr + 1, nt, npa),
            "hdns": (nr + 1, nt, npa), "bnes": (nr + 1, nt), "dbdt": (nr + 1, nt),
            "vt": (nr + 1, nt), "eir": (nr + 1, nt), "eip": (nr + 1, nt), "vtol": (nr + 1, nt), "vtn": (nr + 1, nt),
            "rmas": (ns,), "v": (ns, ne), "grel": (ns, ne), "grbnd": (ns, ne), "epp": (ns, ne), "ernh": (ns, ne),
            "upa": (nr,), "we": (ne,), "de": (ne,), "ekev": (ne,), "ebnd": (ne,), "phi": (nt,),
            "mu": (npa,), "dmu": (npa,), "wmu": (npa,), "lz": (nr + 1,), "rlz": (nr + 1,),
            "ffactor": (ns, nr, ne, npa), "outsidemgnp": (nr, nt), "atlos": (ns, nr, ne),
            "fgeos": (ns, nt, ne, npa), "dtdriftr": (ns,), "dtdriftp": (ns,), "dtdrifte": (ns,),
            "dtdriftmu": (ns,), "setrc": (ns,), "elorc": (ns,), "lsdr": (ns,), "lscha": (ns,), "lsatm": (ns,),
            "lscoe": (ns,), "lscsc": (ns,), "lswae": (ns,), "xne": (nr, nt),
            # ARRAYS' outputs (src/ModRamInit.f90:97-101) and the coefficient
            # arrays of WPADIF / FLCscatter and ram_sum_pressure
            "amla": (slen,), "be": (nr + 1, slen), "zrpabn": (nr, npa, slen), "pa": (npa,), "pabn": (npa,),
            "mlt": (nt,), "vbnd": (ns, ne), "facgr": (ns, ne), "pallsum": (nr, nt), "pparsum": (nr, nt),
            "ataw": (nr, nt, ne, npa), "atac": (nr, nt, ne, npa), "flc_coef": (4, nr, nt, ne, npa),
        }
        self.a = {}
        for name, shp in shapes.items():
            self.a[name] = self.alloc("modramvariables::" + name, shp)
        a = self.a
        for k in ("we", "de", "ekev", "ebnd", "phi", "mu", "dmu", "wmu", "lz", "rlz", "upa"):
            a[k][...] = np.asarray(getattr(g, k), dtype=np.float64)
        a["rmas"][...] = np.asarray(g.rmas)
        for k in ("v", "grel", "grbnd", "epp", "ernh", "ffactor"):
            a[k][...] = np.asarray(getattr(g, k))
        for k in ("fnhs", "fnis", "bounhs", "bounis", "didt", "dibndt", "hdns", "bnes", "dbdt", "eir", "eip"):
            a[k][...] = np.asarray(getattr(fields, k))
        a["outsidemgnp"][...] = np.asarray(fields.outside, dtype=np.int32)
        self.set("modramvariables::mdr", g.mdr)
        self.set("modramvariables::conf1", g.conf1)
        self.set("modramvariables::conf2", g.conf2)
        self.set("modramgrids::dphi", g.dphi)
        self.set("modramparams::betalim", betalim)
        self.set("modramvariables::fraccfl", fraccfl)
        self.set("modramtiming::dtsmin", dtsmin)

    def _charge(self, i):
        # species(i)%s_charge through the driver
        return self.call("refdrv_species_charge", i, 0)[1]

    # ------------------------------------------------------------ the step
    def ram_run(self, f2s, fgeos, dts, kp, uts=0.0, potential=None):
        """One reference ram_run over every species.  f2s: list of
        (NR,NT,NE,NPA) arrays, updated in place; fgeos: list of (NT,NE,NPA).
        potential: None for the Volland-Stern VT from Kp, else (VTOL, VTN,
        T, TOLV, DtEfi) for the interpolated branch
        VT = VTOL + (VTN-VTOL)*(T-TOLV)/DtEfi (src/ModRamRun.f90:46-52).
        Returns the outputs in the layout of the C oracle's ram_run."""
        a = self.a
        for s in range(self.ns):
            a["f2"][s] = f2s[s]
            a["fgeos"][s] = fgeos[s]
        if potential is None:
            self.set_str("modramparams::electric", "VOLS")
        else:
            vtol, vtn, t, tolv, dtefi = potential
            self.set_str("modramparams::electric", "WESC")
            a["vtol"][...] = vtol
            a["vtn"][...] = vtn
            self.set("modramtiming::t", t)
            self.set("modramvariables::tolv", tolv)
            self.set("modramtiming::dtefi", dtefi)
        self.set("modramtiming::dts", dts)
        self.set("modramvariables::kp", kp)
        self.set("modramtiming::uts", uts)
        self.lib.ref_stub_reset()
        self.call("ram_run")
        bad = set(self.stubs()) - ALLOWED_STUBS
        if bad:
            raise RuntimeError(f"ram_run reached procedures outside the translation: {sorted(bad)}")
        for s in range(self.ns):
            f2s[s][...] = a["f2"][s]
        rng = range(self.ns)
        return {
            "vt": a["vt"].copy(order="F"),
            "ppert": {s: a["ppert"][s].copy(order="F") for s in rng},
            "ppart": {s: a["ppart"][s].copy(order="F") for s in rng},
            "flux": {s: a["flux"][s].copy(order="F") for s in rng},
            "dts_next": self.get("modramtiming::dtsnext"),
            "losses": {s: (a["setrc"][s], a["lsdr"][s], a["lscha"][s], a["lsatm"][s]) for s in rng},
            "dtdrift": {s: (a["dtdriftr"][s], a["dtdriftp"][s], a["dtdrifte"][s], a["dtdriftmu"][s]) for s in rng},
            "charge": {s: a["charge"][s].copy(order="F") for s in rng},
            "atlos": {s: a["atlos"][s].copy(order="F") for s in rng},
        }

    def load_state(self, f2s, fgeos):
        for s in range(self.ns):
            self.a["f2"][s] = f2s[s]
            self.a["fgeos"][s] = fgeos[s]

    def step(self, dts, kp, uts=0.0):
        """One reference ram_run on the state held in the reference's own
        module arrays (no copies in or out): the timed form."""
        self.set("modramtiming::dts", dts)
        self.set("modramvariables::kp", kp)
        self.set("modramtiming::uts", uts)
        self.call("ram_run")

    # ------------------------------------------------------------ other routines
    def arrays(self):
        """The reference's ARRAYS (src/ModRamInit.f90:364-587) for every
        species: the grid it builds, read back from the module arrays."""
        for s in range(self.ns):
            self.call("arrays", s + 1)
        a = self.a
        out = {k: a[k].copy() for k in ("lz", "rlz", "phi", "mlt", "ekev", "ebnd", "we", "de", "mu", "dmu", "wmu",
                                         "pa", "pabn", "upa", "rmas", "grel", "grbnd", "v", "vbnd", "ffactor",
                                         "epp", "ernh")}
        for k in ("dl1", "mdr", "conf1", "conf2"):
            out[k] = self.get("modramvariables::" + k)
        out["dphi"] = self.get("modramgrids::dphi")
        return out

    def wpadif(self, s, f2, daa, dts):
        """The reference's WPADIF (src/ModRamWPI.f90:643-714) on species s
        (an electron species: ATAW = daa, ATAC = 0); f2 updated in place."""
        self.a["ataw"][...] = daa
        self.a["atac"][...] = 0.0
        self.a["f2"][s] = f2
        self.set("modramtiming::dts", dts)
        self.call("wpadif", s + 1)
        f2[...] = self.a["f2"][s]

    def flcscatter(self, s, f2, coef, dts):
        """The reference's FLCscatter (src/ModRamLoss.f90:513-575) on species
        s with FLC_coef(s,...) = coef, after the first boundary cycle
        (TimeRamElapsed >= Dt_bc); f2 updated in place."""
        self.a["flc_coef"][s] = coef
        self.a["f2"][s] = f2
        self.set("modramtiming::dts", dts)
        self.set("modramtiming::timeramelapsed", self.get("modramtiming::dt_bc"))
        self.call("flcscatter", s + 1)
        f2[...] = self.a["f2"][s]

    def sum_pressure(self, ppert, ppart):
        """The reference's ram_sum_pressure (src/ModRamFunctions.f90:272-297)
        over every species: (PAllSum, PParSum)."""
        for s in range(self.ns):
            self.a["ppert"][s] = ppert[s]
            self.a["ppart"][s] = ppart[s]
        self.call("ram_sum_pressure")
        return self.a["pallsum"].copy(), self.a["pparsum"].copy()

    def subroutine(self, name, s):
        """Call one species-indexed reference routine (DRIFTPARA, DRIFTR, ...,
        CEPARA, CHAREXCHANGE, ATMOL, SUMRC, ANISCH) on species s (0-based)."""
        self.call(name, s + 1)
