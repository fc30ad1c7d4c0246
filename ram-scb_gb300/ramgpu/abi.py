"""ctypes binding of the C ABI in include/ramgpu.h.

``RamGpu`` mirrors the reference's interface for this path: the RAM state
(F2 per species, field tables, FGEOS, VT) lives in the context, ``ram_run``
advances it by one call of src/ModRamRun.f90:16-225, and the outputs
(PPERT/PPART, FLUX, DtsNext, SUMRC losses) are read back afterwards.
Arrays cross the boundary in the reference's Fortran layout.  There is no
CPU fallback: if the CUDA library is missing the constructor raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import build as _build

RAMGPU_OK = 0
ERRORS = {-1: "RAMGPU_ERR_ARG", -2: "RAMGPU_ERR_CUDA", -3: "RAMGPU_ERR_STATE",
          -4: "RAMGPU_ERR_NUMERIC", -5: "RAMGPU_ERR_NOMEM"}
FLAG_CLOSED, FLAG_NO_ATMOL, FLAG_LOSSES = 1, 2, 4

# Every symbol include/ramgpu.h declares.
EXPORTS = (
    "ramgpu_create", "ramgpu_destroy", "ramgpu_last_error", "ramgpu_set_stream",
    "ramgpu_set_species", "ramgpu_set_grid", "ramgpu_set_fields", "ramgpu_set_boundary",
    "ramgpu_set_potential", "ramgpu_set_kp", "ramgpu_set_member_species",
    "ramgpu_set_member_active", "ramgpu_upload_f2", "ramgpu_download_f2",
    "ramgpu_upload_f2_all", "ramgpu_download_f2_all", "ramgpu_f2_device_ptr",
    "ramgpu_ram_run", "ramgpu_half_step", "ramgpu_ram_run_async", "ramgpu_moments",
    "ramgpu_flux", "ramgpu_cfl", "ramgpu_losses", "ramgpu_reset_losses", "ramgpu_launch_count",
    "ramgpu_apply_op", "ramgpu_set_timing", "ramgpu_kernel_times", "ramgpu_probe_fp64",
    "ramgpu_sumrc_noalloc", "ramgpu_set_graph", "ramgpu_set_launch_shape",
    "ramgpu_get_launch_shape", "ramgpu_autotune", "ramgpu_set_kp_all",
    "ramgpu_adj_forward", "ramgpu_adj_backward", "ramgpu_adj_digest", "ramgpu_adj_record",
    "ramgpu_fly_sats", "ramgpu_sum_pressure", "ramgpu_adj_replay", "ramgpu_set_pa_diffusion",
    "ramgpu_loss_wae", "ramgpu_bounce_integrals", "ramgpu_upload_f2_async", "ramgpu_download_f2_async",
    "ramgpu_moments_async", "ramgpu_synchronize", "ramgpu_set_coef_store", "ramgpu_compute_hI",
    "ramgpu_get_fields", "ramgpu_ram_run_host", "ramgpu_ram_run_ref", "ramgpu_set_ref_staging", "ramgpu_autotune_trials",
    "ramgpu_save_state", "ramgpu_load_state", "ramgpu_snapshot_info", "ramgpu_set_pipeline_chunks",
    "ramgpu_set_pipeline_groups", "ramgpu_pipeline_groups",
    "ramgpu_set_step_groups", "ramgpu_step_groups", "ramgpu_set_pipeline_trace", "ramgpu_pipeline_trace",
    "ramgpu_check", "ramgpu_set_check", "ramgpu_last_status",
    "ramgpu_set_adj_record_budget", "ramgpu_adj_segments", "ramgpu_set_adj_overlap", "ramgpu_bounds_report",
    "ramgpu_f2_stats", "ramgpu_probe_l2", "ramgpu_set_mu_lanes",
    "ramgpu_selftest_arith",
)
BAD_DATA = -1.0E10  # BadDataFlag of the satellite products
KCLASS = ("member_tables", "ghost_planes", "driftr", "driftp", "drifte", "driftmu", "finish",
          "anisch", "dts_tables", "sumrc", "padif")
OP_DRIFTR, OP_DRIFTP, OP_DRIFTE, OP_DRIFTMU, OP_CHAREXCHANGE, OP_ATMOL, OP_ANISCH, OP_PADIF = range(8)


class RamGpuError(RuntimeError):
    def __init__(self, msg, code=None):
        super().__init__(msg)
        self.code = code  # the RAMGPU_ERR_* value, when the library returned one


class Status(C.Structure):
    """ramgpu_status: the device status word."""
    _fields_ = [("f2_nonfinite", C.c_longlong), ("moments_nonfinite", C.c_longlong),
                ("cfl_over", C.c_longlong), ("clips", C.c_longlong), ("first_member", C.c_int),
                ("first_species", C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class SnapshotInfo(C.Structure):
    """ramgpu_snapshot_info_t: header of a snapshot file."""
    _fields_ = [("nr", C.c_int), ("nt", C.c_int), ("ne", C.c_int), ("npa", C.c_int), ("ns", C.c_int),
                ("n_members", C.c_int), ("flags", C.c_uint), ("time", C.c_double)]


def snapshot_info(path) -> dict:
    """Header of a snapshot file after its checksum is checked (no GPU)."""
    lib = load_library()
    info = SnapshotInfo()
    rc = lib.ramgpu_snapshot_info(str(path).encode(), C.byref(info))
    if rc != RAMGPU_OK:
        buf = C.create_string_buffer(256)
        lib.ramgpu_last_error(None, buf, 256)
        raise RamGpuError(f"snapshot_info: {buf.value.decode()}", rc)
    return {k: getattr(info, k) for k, _ in SnapshotInfo._fields_}


class Config(C.Structure):
    _fields_ = [("nr", C.c_int), ("nt", C.c_int), ("ne", C.c_int), ("npa", C.c_int),
                ("ns", C.c_int), ("n_members", C.c_int), ("betalim", C.c_double),
                ("fraccfl", C.c_double), ("dtsmin", C.c_double), ("flags", C.c_uint)]


_P = C.POINTER(C.c_double)


class GridStruct(C.Structure):
    _fields_ = [("lz", _P), ("rlz", _P), ("phi", _P), ("dl1", C.c_double), ("mdr", C.c_double),
                ("dphi", C.c_double), ("conf1", C.c_double), ("conf2", C.c_double),
                ("ekev", _P), ("ebnd", _P), ("we", _P), ("de", _P), ("mu", _P), ("dmu", _P),
                ("wmu", _P), ("upa", _P), ("rmas", _P), ("grel", _P), ("grbnd", _P), ("v", _P),
                ("epp", _P), ("ernh", _P), ("ffactor", _P)]


class ObsStruct(C.Structure):
    _fields_ = [("member", C.c_int), ("s", C.c_int), ("call", C.c_int), ("k", C.c_int),
                ("l", C.c_int), ("lshell", C.c_double), ("mlt", C.c_double), ("log_obs", C.c_double)]


class SatStruct(C.Structure):
    _fields_ = [("member", C.c_int), ("lshell", C.c_double), ("mlt", C.c_double)]


_lib = None


def load_library(path: str | Path | None = None, build_if_missing: bool = False):
    """Load libramgpu.so; raise if it is absent (no fallback path exists)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else _build.LIB_PATH
    if not p.exists():
        if build_if_missing:
            _build.build_library()
        else:
            raise RamGpuError(f"CUDA library {p} not built; run __graft_entry__.build()")
    lib = C.CDLL(str(p))
    vp = C.c_void_p
    i, d, u = C.c_int, C.c_double, C.c_uint
    dp = _P
    ip = C.POINTER(C.c_int)
    sig = {
        "ramgpu_create": ([C.POINTER(Config), C.POINTER(vp)], i),
        "ramgpu_destroy": ([vp], i),
        "ramgpu_last_error": ([vp, C.c_char_p, C.c_size_t], i),
        "ramgpu_set_stream": ([vp, vp], i),
        "ramgpu_set_species": ([vp, i, i, i], i),
        "ramgpu_set_grid": ([vp, C.POINTER(GridStruct)], i),
        "ramgpu_set_fields": ([vp] + [dp] * 11 + [ip], i),
        "ramgpu_set_boundary": ([vp, i, i, dp], i),
        "ramgpu_set_potential": ([vp, i, dp], i),
        "ramgpu_set_kp": ([vp, i, d], i),
        "ramgpu_set_member_species": ([vp, i, i, ip], i),
        "ramgpu_set_member_active": ([vp, i, i], i),
        "ramgpu_upload_f2": ([vp, i, i, dp], i),
        "ramgpu_download_f2": ([vp, i, i, dp], i),
        "ramgpu_upload_f2_all": ([vp, i, dp], i),
        "ramgpu_download_f2_all": ([vp, i, dp], i),
        "ramgpu_f2_device_ptr": ([vp, i, i, C.POINTER(dp)], i),
        "ramgpu_ram_run": ([vp, d], i),
        "ramgpu_half_step": ([vp, d, i], i),
        "ramgpu_ram_run_async": ([vp, d], i),
        "ramgpu_moments": ([vp, i, i, dp, dp], i),
        "ramgpu_flux": ([vp, i, i, dp], i),
        "ramgpu_cfl": ([vp, i, i, dp], i),
        "ramgpu_losses": ([vp, i, i, dp], i),
        "ramgpu_reset_losses": ([vp], i),
        "ramgpu_launch_count": ([vp], C.c_longlong),
        "ramgpu_apply_op": ([vp, d, i, i], i),
        "ramgpu_set_timing": ([vp, i], i),
        "ramgpu_kernel_times": ([vp, dp, C.POINTER(C.c_longlong)], i),
        "ramgpu_probe_fp64": ([dp], i),
        "ramgpu_sumrc_noalloc": ([vp, i, i, i, i, dp, dp, dp, vp, dp], i),
        "ramgpu_set_graph": ([vp, i], i),
        "ramgpu_set_launch_shape": ([vp, i, i, i], i),
        "ramgpu_get_launch_shape": ([vp, ip, ip], i),
        "ramgpu_autotune": ([vp, d, i, dp], i),
        "ramgpu_set_kp_all": ([vp, dp], i),
        "ramgpu_adj_forward": ([vp, i, d, dp, i, C.POINTER(ObsStruct), i, dp], i),
        "ramgpu_adj_backward": ([vp, dp, dp], i),
        "ramgpu_adj_digest": ([vp, C.POINTER(C.c_ulonglong)], i),
        "ramgpu_adj_record": ([vp, i, C.POINTER(C.c_ubyte)], i),
        "ramgpu_fly_sats": ([vp, C.POINTER(SatStruct), i, dp, dp], i),
        "ramgpu_adj_replay": ([vp, dp], i),
        "ramgpu_set_pa_diffusion": ([vp, i, dp], i),
        "ramgpu_loss_wae": ([vp, i, i, dp], i),
        "ramgpu_bounce_integrals": ([vp, i, dp, dp, dp, dp, dp, dp, i, dp, dp, dp, dp], i),
        "ramgpu_upload_f2_async": ([vp, i, i, dp], i),
        "ramgpu_download_f2_async": ([vp, i, i, dp], i),
        "ramgpu_moments_async": ([vp, i, i, dp, dp], i),
        "ramgpu_synchronize": ([vp], i),
        "ramgpu_set_coef_store": ([vp, i], i),
        "ramgpu_compute_hI": ([vp, i, dp, dp, dp, dp, dp, dp, i, dp, dp, d, d], i),
        "ramgpu_get_fields": ([vp] + [dp] * 11, i),
        "ramgpu_sum_pressure": ([vp, i, dp, dp], i),
        "ramgpu_ram_run_host": ([vp, d, vp, vp, vp], i),
        "ramgpu_ram_run_ref": ([vp, d, vp, vp, vp], i),
        "ramgpu_set_ref_staging": ([vp, i], i),
        "ramgpu_autotune_trials": ([vp, dp, dp], i),
        "ramgpu_save_state": ([vp, C.c_char_p, d], i),
        "ramgpu_set_pipeline_chunks": ([vp, i], i),
        "ramgpu_load_state": ([vp, C.c_char_p, dp], i),
        "ramgpu_snapshot_info": ([C.c_char_p, C.POINTER(SnapshotInfo)], i),
        "ramgpu_set_pipeline_groups": ([vp, i], i),
        "ramgpu_pipeline_groups": ([vp], i),
        "ramgpu_set_step_groups": ([vp, i], i),
        "ramgpu_step_groups": ([vp], i),
        "ramgpu_set_pipeline_trace": ([vp, i], i),
        "ramgpu_check": ([vp, C.POINTER(Status)], i),
        "ramgpu_set_check": ([vp, i], i),
        "ramgpu_last_status": ([vp, C.POINTER(Status)], i),
        "ramgpu_pipeline_trace": ([vp, ip, C.POINTER(C.c_float)], i),
        "ramgpu_set_adj_record_budget": ([vp, C.c_longlong], i),
        "ramgpu_adj_segments": ([vp, ip, ip], i),
        "ramgpu_set_adj_overlap": ([vp, i], i),
        "ramgpu_bounds_report": ([vp, ip, C.POINTER(C.c_longlong), ip, C.POINTER(C.c_longlong)], i),
        "ramgpu_f2_stats": ([vp, i, i, dp, dp, dp], i),
        "ramgpu_probe_l2": ([dp], i),
        "ramgpu_set_mu_lanes": ([vp, i], i),
        "ramgpu_selftest_arith": ([C.c_longlong, C.c_ulonglong, C.POINTER(C.c_longlong)], i),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    if path is None:
        _lib = lib
    return lib


def probe_fp64() -> float:
    """FP64 fma lane-operations per second of the current GPU."""
    lib = load_library()
    v = C.c_double()
    rc = lib.ramgpu_probe_fp64(C.byref(v))
    if rc != RAMGPU_OK:
        raise RamGpuError(f"ramgpu_probe_fp64: {ERRORS.get(rc, rc)}")
    return v.value


def probe_l2() -> float:
    """L2 read bandwidth of the current GPU in bytes per second."""
    lib = load_library()
    v = C.c_double()
    rc = lib.ramgpu_probe_l2(C.byref(v))
    if rc != RAMGPU_OK:
        raise RamGpuError(f"ramgpu_probe_l2: {ERRORS.get(rc, rc)}")
    return v.value


def selftest_arith(n: int, seed: int = 1) -> int:
    """Mismatches of the integer-pipe FP64 multiply against the FP64 unit on
    n random operand pairs (0 expected)."""
    lib = load_library()
    m = C.c_longlong()
    rc = lib.ramgpu_selftest_arith(int(n), int(seed), C.byref(m))
    if rc != RAMGPU_OK:
        raise RamGpuError(f"ramgpu_selftest_arith: {ERRORS.get(rc, rc)}")
    return m.value


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(_P)


def _fort(a, dtype=np.float64):
    return np.asfortranarray(np.asarray(a, dtype=dtype))


class RamGpu:
    """One GPU context holding the RAM state of ``n_members`` runs.

    grid, fields: ``ramgpu.workload.Grid`` / ``Fields``.  Species are taken
    from ``grid.species`` (charge and CEPARA branch)."""

    def __init__(self, grid, fields, n_members: int = 1, betalim: float = 1.5,
                 fraccfl: float = 0.8, dtsmin: float = 0.1, flags: int = 0, lib=None):
        self.lib = lib or load_library()
        self.grid = grid
        self.ns = len(grid.species)
        self.n_members = n_members
        self.fraccfl = fraccfl
        self._host_tables = None  # ram_run_host's address tables of the last buffer set
        self.member_species = [list(range(self.ns)) for _ in range(n_members)]
        cfg = Config(grid.nr, grid.nt, grid.ne, grid.npa, self.ns, n_members, betalim, fraccfl,
                     dtsmin, flags)
        h = C.c_void_p()
        rc = self.lib.ramgpu_create(C.byref(cfg), C.byref(h))
        if rc != RAMGPU_OK:
            buf = C.create_string_buffer(512)
            self.lib.ramgpu_last_error(None, buf, 512)
            raise RamGpuError(f"ramgpu_create: {ERRORS.get(rc, rc)}: {buf.value.decode()}")
        self.h = h
        for s, sp in enumerate(grid.species):
            self._ck(self.lib.ramgpu_set_species(self.h, s, sp.charge, sp.cex_kind), "set_species")
        self.set_grid(grid)
        self.set_fields(fields)

    # -------------------------------------------------------------- plumbing
    def _ck(self, rc, what):
        if rc != RAMGPU_OK:
            buf = C.create_string_buffer(512)
            self.lib.ramgpu_last_error(self.h, buf, 512)
            raise RamGpuError(f"{what}: {ERRORS.get(rc, rc)}: {buf.value.decode()}", code=rc)

    def close(self):
        self._host_tables = None
        if getattr(self, "h", None):
            self.lib.ramgpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---------------------------------------------------------------- inputs
    def set_grid(self, g):
        keep = {k: _fort(getattr(g, k)) for k in ("lz", "rlz", "phi", "ekev", "ebnd", "we", "de", "mu",
                                                  "dmu", "wmu", "upa", "rmas", "grel", "grbnd", "v",
                                                  "epp", "ernh", "ffactor")}
        gs = GridStruct()
        for k, a in keep.items():
            setattr(gs, k, _dptr(a))
        gs.dl1, gs.mdr, gs.dphi, gs.conf1, gs.conf2 = g.dl1, g.mdr, g.dphi, g.conf1, g.conf2
        self._ck(self.lib.ramgpu_set_grid(self.h, C.byref(gs)), "set_grid")

    def set_fields(self, f):
        arrs = [_fort(getattr(f, k)) for k in ("fnhs", "fnis", "bounhs", "bounis", "hdns", "didt",
                                               "dibndt", "bnes", "dbdt", "eir", "eip")]
        out = _fort(f.outside, np.int32)
        self._ck(self.lib.ramgpu_set_fields(self.h, *[_dptr(a) for a in arrs],
                                            out.ctypes.data_as(C.POINTER(C.c_int))), "set_fields")

    def set_boundary(self, member: int, s: int, fgeos):
        a = _fort(fgeos)
        self._ck(self.lib.ramgpu_set_boundary(self.h, member, s, _dptr(a)), "set_boundary")

    def set_kp(self, member: int, kp: float):
        self._ck(self.lib.ramgpu_set_kp(self.h, member, float(kp)), "set_kp")

    def set_kp_all(self, kp):
        a = np.ascontiguousarray(kp, dtype=np.float64)
        if a.size != self.n_members:
            raise ValueError("need one Kp per member")
        self._ck(self.lib.ramgpu_set_kp_all(self.h, _dptr(a)), "set_kp_all")

    def set_potential(self, member: int, vt):
        a = _fort(vt)
        self._ck(self.lib.ramgpu_set_potential(self.h, member, _dptr(a)), "set_potential")

    def set_member_species(self, member: int, species_list):
        a = np.asarray(species_list, dtype=np.int32)
        self._ck(self.lib.ramgpu_set_member_species(self.h, member, a.size,
                                                    a.ctypes.data_as(C.POINTER(C.c_int))),
                 "set_member_species")
        self.member_species[member] = sorted(int(x) for x in a)

    def set_member_active(self, member: int, active: bool):
        self._ck(self.lib.ramgpu_set_member_active(self.h, member, int(bool(active))), "set_member_active")

    # ----------------------------------------------------------------- state
    def upload_f2(self, member: int, s: int, f2):
        a = _fort(f2)
        self._ck(self.lib.ramgpu_upload_f2(self.h, member, s, _dptr(a)), "upload_f2")

    def download_f2(self, member: int, s: int) -> np.ndarray:
        g = self.grid
        a = np.empty((g.nr, g.nt, g.ne, g.npa), order="F")
        self._ck(self.lib.ramgpu_download_f2(self.h, member, s, _dptr(a)), "download_f2")
        return a

    def f2_device_ptr(self, member: int, s: int) -> int:
        p = _P()
        self._ck(self.lib.ramgpu_f2_device_ptr(self.h, member, s, C.byref(p)), "f2_device_ptr")
        return C.cast(p, C.c_void_p).value

    # ------------------------------------------------------------------ step
    def ram_run(self, dts: float):
        self._ck(self.lib.ramgpu_ram_run(self.h, float(dts)), "ram_run")

    def ram_run_async(self, dts: float):
        self._ck(self.lib.ramgpu_ram_run_async(self.h, float(dts)), "ram_run_async")

    def ram_run_host(self, dts: float, f2, ppert=None, ppart=None):
        """One ram_run call with F2 on the host (ramgpu_ram_run_host): f2[slot]
        (slot = member*NS + species; None = stays resident) is uploaded,
        advanced and written back in place; ppert/ppart[slot], when given,
        receive the moments.  Buffers: float64, contiguous, writable, NCELL
        (resp. NR*NT) values in the layout of upload_f2 / moments."""
        g = self.grid
        nslot = self.n_members * self.ns
        seqs = tuple(None if q is None else list(q) for q in (f2, ppert, ppart))
        # the address tables of the last buffer set are kept with references
        # to its arrays (so their ids cannot be reused): a call with the same
        # arrays, the usual case from a time loop, skips rebuilding them
        key = tuple(None if q is None else tuple(map(id, q)) for q in seqs)
        hit = self._host_tables is not None and self._host_tables[0] == key
        if hit:
            tabs = self._host_tables[1]
            sizes = (g.nr * g.nt * g.ne * g.npa, g.nr * g.nt, g.nr * g.nt)
            hit = all(a is None or (a.flags.writeable and a.size == n)
                      for q, n in zip(seqs, sizes) if q is not None for a in q)
        if not hit:
            vtab = C.c_void_p * nslot

            def table(seq, n, what):
                if seq is None:
                    return None
                if len(seq) != nslot:
                    raise RamGpuError(f"{what}: need {nslot} entries (member*NS + species)")
                addrs = []
                for k, a in enumerate(seq):
                    if a is None:
                        addrs.append(None)
                        continue
                    if not (isinstance(a, np.ndarray) and a.dtype == np.float64 and a.size == n
                            and a.flags.writeable and (a.flags.f_contiguous or a.flags.c_contiguous)):
                        raise RamGpuError(f"{what}[{k}]: need a contiguous writable float64 array of {n} values")
                    addrs.append(a.ctypes.data)
                return vtab(*addrs)

            ncell = g.nr * g.nt * g.ne * g.npa
            tabs = (table(seqs[0], ncell, "f2"), table(seqs[1], g.nr * g.nt, "ppert"),
                    table(seqs[2], g.nr * g.nt, "ppart"))
            self._host_tables = (key, tabs, seqs)
        self._ck(self.lib.ramgpu_ram_run_host(self.h, float(dts), *tabs), "ram_run_host")

    def ram_run_ref(self, dts: float, f2, ppert=None, ppart=None):
        """One ram_run call on arrays in the reference's own layout
        (ramgpu_ram_run_ref): f2[m] is member m's F2(NS,NR,NT,NE,NPA),
        ppert[m]/ppart[m] its PPERT/PPART(NS,NR,NT), each a Fortran-ordered
        (or flat) float64 array, updated in place; None skips a member."""
        g = self.grid
        nm = self.n_members
        sizes = (self.ns * g.ncell, self.ns * g.nr * g.nt, self.ns * g.nr * g.nt)
        seqs = tuple(None if q is None else list(q) for q in (f2, ppert, ppart))
        key = tuple(None if q is None else tuple(map(id, q)) for q in seqs)
        if getattr(self, "_ref_tables", None) is None or self._ref_tables[0] != key:
            vtab = C.c_void_p * nm

            def table(seq, n, what):
                if seq is None:
                    return None
                if len(seq) != nm:
                    raise RamGpuError(f"{what}: need {nm} entries (one per member)")
                addrs = []
                for k, a in enumerate(seq):
                    if a is None:
                        addrs.append(None)
                        continue
                    if not (isinstance(a, np.ndarray) and a.dtype == np.float64 and a.size == n
                            and a.flags.writeable and (a.flags.f_contiguous or a.flags.c_contiguous)):
                        raise RamGpuError(f"{what}[{k}]: need a contiguous writable float64 array of {n} values")
                    addrs.append(a.ctypes.data)
                return vtab(*addrs)

            tabs = tuple(table(q, n, w) for q, n, w in zip(seqs, sizes, ("f2", "ppert", "ppart")))
            self._ref_tables = (key, tabs, seqs)
        self._ck(self.lib.ramgpu_ram_run_ref(self.h, float(dts), *self._ref_tables[1]), "ram_run_ref")

    def save_state(self, path, time: float = 0.0):
        """The context's evolving state to a snapshot file (ramgpu_save_state)."""
        self._ck(self.lib.ramgpu_save_state(self.h, str(path).encode(), float(time)), "save_state")

    def load_state(self, path) -> float:
        """State from a snapshot file; returns the time saved with it."""
        t = C.c_double(0.0)
        self._ck(self.lib.ramgpu_load_state(self.h, str(path).encode(), C.byref(t)), "load_state")
        return t.value

    def set_ref_staging(self, mode):
        """How reference-layout arrays move (ramgpu_set_ref_staging): 0 (or
        False) in place where the device reaches them; 1 (or True) through
        the staging buffer and the copy engines, unpipelined; 2 page-locked
        arrays through the copy engines chunk by chunk, inside the pipeline."""
        self._ck(self.lib.ramgpu_set_ref_staging(self.h, int(mode)), "set_ref_staging")

    def upload_f2_all(self, member: int, f2):
        """Member's whole F2(NS,NR,NT,NE,NPA) in the reference layout."""
        a = np.asfortranarray(np.asarray(f2, dtype=np.float64))
        if a.size != self.ns * self.grid.ncell:
            raise RamGpuError("upload_f2_all: need NS*NR*NT*NE*NPA values")
        self._ck(self.lib.ramgpu_upload_f2_all(self.h, int(member), _dptr(a)), "upload_f2_all")

    def download_f2_all(self, member: int) -> np.ndarray:
        g = self.grid
        out = np.zeros((self.ns, g.nr, g.nt, g.ne, g.npa), order="F")
        self._ck(self.lib.ramgpu_download_f2_all(self.h, int(member), _dptr(out)), "download_f2_all")
        return out

    def set_pipeline_chunks(self, chunks: int):
        """Chunks of L planes the host calls pipeline F2 over (0: item groups)."""
        self._ck(self.lib.ramgpu_set_pipeline_chunks(self.h, int(chunks)), "set_pipeline_chunks")

    def set_pipeline_groups(self, groups: int):
        """Item groups ram_run_host pipelines its copies over."""
        self._ck(self.lib.ramgpu_set_pipeline_groups(self.h, int(groups)), "set_pipeline_groups")

    def pipeline_groups(self) -> int:
        return int(self.lib.ramgpu_pipeline_groups(self.h))

    def set_step_groups(self, groups: int):
        """Item groups whose sweeps ram_run runs on concurrent streams."""
        self._ck(self.lib.ramgpu_set_step_groups(self.h, int(groups)), "set_step_groups")

    def step_groups(self) -> int:
        return int(self.lib.ramgpu_step_groups(self.h))

    def check(self) -> dict:
        """Status word of the active items now (ramgpu_check); a non-finite
        value is reported in the dict, not raised."""
        st = Status()
        rc = self.lib.ramgpu_check(self.h, C.byref(st))
        if rc not in (RAMGPU_OK, -4):
            self._ck(rc, "check")
        return st.as_dict()

    def set_check(self, enable: bool):
        """Append the status pass to every ram_run / ram_run_host; the
        synchronous calls then raise RamGpuError (code -4) after a call that
        left a non-finite value."""
        self._ck(self.lib.ramgpu_set_check(self.h, int(bool(enable))), "set_check")

    def last_status(self) -> dict:
        st = Status()
        rc = self.lib.ramgpu_last_status(self.h, C.byref(st))
        if rc not in (RAMGPU_OK, -4):
            self._ck(rc, "last_status")
        return st.as_dict()

    def set_pipeline_trace(self, enable: bool):
        self._ck(self.lib.ramgpu_set_pipeline_trace(self.h, int(bool(enable))), "set_pipeline_trace")

    def pipeline_trace(self) -> np.ndarray:
        """(groups, 3) ms after the last traced ram_run_host call started:
        uploads landed, sweeps done, read-back done."""
        G = C.c_int()
        ms = np.zeros(24, dtype=np.float32)
        self._ck(self.lib.ramgpu_pipeline_trace(self.h, C.byref(G), ms.ctypes.data_as(C.POINTER(C.c_float))),
                 "pipeline_trace")
        return ms[:3 * G.value].reshape(G.value, 3).astype(np.float64)

    def half_step(self, dts: float, order: int):
        self._ck(self.lib.ramgpu_half_step(self.h, float(dts), int(order)), "half_step")

    def apply_op(self, dts: float, op: int, cfl: bool = False):
        """One reference operator (DRIFTR..ANISCH) on every active item."""
        self._ck(self.lib.ramgpu_apply_op(self.h, float(dts), int(op), int(bool(cfl))), "apply_op")

    # --------------------------------------------------------------- outputs
    def moments(self, member: int, s: int):
        g = self.grid
        pe = np.empty((g.nr, g.nt), order="F")
        pa = np.empty((g.nr, g.nt), order="F")
        self._ck(self.lib.ramgpu_moments(self.h, member, s, _dptr(pe), _dptr(pa)), "moments")
        return pe, pa

    def flux(self, member: int, s: int) -> np.ndarray:
        g = self.grid
        a = np.empty((g.nr, g.nt, g.ne, g.npa), order="F")
        self._ck(self.lib.ramgpu_flux(self.h, member, s, _dptr(a)), "flux")
        return a

    def fly_sats(self, sats):
        """Virtual-spacecraft samples of the current state.  sats: iterable of
        (member, lshell [RE], mlt [h]).  Returns (SatFlux, OmnFlux) with shapes
        (nsat, NS, NE, NPA) and (nsat, NS, NE); BadDataFlag where undefined."""
        g = self.grid
        sats = list(sats)
        arr = (SatStruct * max(1, len(sats)))(*[SatStruct(int(m), float(lv), float(t)) for m, lv, t in sats])
        fl = np.zeros(len(sats) * self.ns * g.ne * g.npa)
        om = np.zeros(len(sats) * self.ns * g.ne)
        self._ck(self.lib.ramgpu_fly_sats(self.h, arr, len(sats), _dptr(fl), _dptr(om)), "fly_sats")
        return (fl.reshape(len(sats), g.npa, g.ne, self.ns).transpose(0, 3, 2, 1),
                om.reshape(len(sats), g.ne, self.ns).transpose(0, 2, 1))

    def sum_pressure(self, member: int = 0):
        """(PAllSum, PParSum), each (NR, NT), from the moments of the last ram_run."""
        g = self.grid
        pa = np.empty((g.nr, g.nt), order="F")
        pp = np.empty((g.nr, g.nt), order="F")
        self._ck(self.lib.ramgpu_sum_pressure(self.h, int(member), _dptr(pa), _dptr(pp)), "sum_pressure")
        return pa, pp

    def bounce_integrals(self, lines):
        """computehI's bounce integrals on field lines (workload.FieldLines):
        (H_cart, I_cart, HDens_cart, mirror B), each (NR, NT, NPA)."""
        g = self.grid
        shp = (g.nr, g.nt, g.npa)
        h, fi, hd, bm = (np.zeros(shp, order="F") for _ in range(4))
        arrs = [_fort(a) for a in (lines.chi, lines.x, lines.y, lines.z, lines.b, lines.dens)]
        self._ck(self.lib.ramgpu_bounce_integrals(self.h, int(lines.chi.size), *[_dptr(a) for a in arrs],
                                                  int(lines.ieq), _dptr(h), _dptr(fi), _dptr(hd), _dptr(bm)),
                 "bounce_integrals")
        return h, fi, hd, bm

    def compute_hI(self, lines, pa, pabn, bnormal: float = 1.0, dthi: float = 0.0):
        """computehI on the device from field lines (workload.FieldLines):
        fills the context's field tables."""
        arrs = [_fort(a) for a in (lines.chi, lines.x, lines.y, lines.z, lines.b, lines.dens)]
        pa_, pb_ = _fort(pa), _fort(pabn)
        self._ck(self.lib.ramgpu_compute_hI(self.h, int(lines.chi.size), *[_dptr(a) for a in arrs],
                                            int(lines.ieq), _dptr(pa_), _dptr(pb_), float(bnormal),
                                            float(dthi)), "compute_hI")

    def get_fields(self):
        """The context's field tables: dict of FNHS, FNIS, BOUNHS, BOUNIS, HDNS,
        dIdt, dIbndt (NR+1,NT,NPA) and BNES, dBdt, EIR, EIP (NR+1,NT)."""
        g = self.grid
        names3 = ("fnhs", "fnis", "bounhs", "bounis", "hdns", "didt", "dibndt")
        names2 = ("bnes", "dbdt", "eir", "eip")
        out = {n: np.zeros((g.nr + 1, g.nt, g.npa), order="F") for n in names3}
        out.update({n: np.zeros((g.nr + 1, g.nt), order="F") for n in names2})
        self._ck(self.lib.ramgpu_get_fields(self.h, *[_dptr(out[n]) for n in names3 + names2]), "get_fields")
        return out

    def set_pa_diffusion(self, s: int, daa=None):
        """Pitch-angle diffusion coefficient D(I,J,K,L) of species s (None removes it)."""
        if daa is None:
            self._ck(self.lib.ramgpu_set_pa_diffusion(self.h, s, None), "set_pa_diffusion")
        else:
            a = _fort(daa)
            self._ck(self.lib.ramgpu_set_pa_diffusion(self.h, s, _dptr(a)), "set_pa_diffusion")

    def loss_wae(self, member: int, s: int) -> float:
        v = C.c_double()
        self._ck(self.lib.ramgpu_loss_wae(self.h, member, s, C.byref(v)), "loss_wae")
        return v.value

    def cfl(self, member: int, s: int) -> np.ndarray:
        a = np.empty(5)
        self._ck(self.lib.ramgpu_cfl(self.h, member, s, _dptr(a)), "cfl")
        return a

    def losses(self, member: int, s: int) -> np.ndarray:
        a = np.empty(4)
        self._ck(self.lib.ramgpu_losses(self.h, member, s, _dptr(a)), "losses")
        return a

    def reset_losses(self):
        self._ck(self.lib.ramgpu_reset_losses(self.h), "reset_losses")

    def set_timing(self, enable: bool):
        self._ck(self.lib.ramgpu_set_timing(self.h, int(bool(enable))), "set_timing")

    def kernel_times(self):
        """{class: (total_ms, launches)} of the launches timed since the last call."""
        ms = np.zeros(16)
        cnt = np.zeros(16, dtype=np.int64)
        self._ck(self.lib.ramgpu_kernel_times(self.h, _dptr(ms), cnt.ctypes.data_as(C.POINTER(C.c_longlong))),
                 "kernel_times")
        return {KCLASS[k]: (float(ms[k]), int(cnt[k])) for k in range(len(KCLASS)) if cnt[k]}

    def set_coef_store(self, mask):
        """Sweeps (bit 0 R, 1 P, 2 E, 3 MU; True = 4, False = 0) whose forward
        face coefficients are kept for the reverse half."""
        m = (4 if mask else 0) if isinstance(mask, bool) else int(mask)
        self._ck(self.lib.ramgpu_set_coef_store(self.h, m), "set_coef_store")

    def set_graph(self, enable: bool):
        self._ck(self.lib.ramgpu_set_graph(self.h, int(bool(enable))), "set_graph")

    def set_launch_shape(self, sweep: int, threads: int, persistent_ctas: int = 0):
        self._ck(self.lib.ramgpu_set_launch_shape(self.h, sweep, threads, persistent_ctas),
                 "set_launch_shape")

    def launch_shape(self):
        t = np.zeros(4, dtype=np.int32)
        p = np.zeros(4, dtype=np.int32)
        self._ck(self.lib.ramgpu_get_launch_shape(self.h, t.ctypes.data_as(C.POINTER(C.c_int)),
                                                  p.ctypes.data_as(C.POINTER(C.c_int))), "launch_shape")
        return [(int(a), int(b)) for a, b in zip(t, p)]

    def autotune(self, dts: float, reps: int = 3):
        """Pick threads/CTA and persistent-vs-plain grid per sweep, then the
        number of item groups, by timing whole steps; returns the chosen
        shapes and the best step time of each sweep's round [ms]."""
        ms = np.zeros(4)
        self._ck(self.lib.ramgpu_autotune(self.h, float(dts), int(reps), _dptr(ms)), "autotune")
        return self.launch_shape(), ms

    def autotune_trials(self):
        """Best whole-step trial of the last autotune per sweep (R, P, E, MU):
        (plain-grid ms, persistent-grid ms); 0 where not tried."""
        a, b = np.zeros(4), np.zeros(4)
        self._ck(self.lib.ramgpu_autotune_trials(self.h, _dptr(a), _dptr(b)), "autotune_trials")
        return a, b

    # --------------------------------------------------------------- adjoint
    def adj_forward(self, ncalls: int, dts: float, kp, k_ckpt: int, obs):
        """Checkpointed forward pass of a window; kp: (ncalls, n_members) or
        (ncalls,) Kp; obs: list of dicts with member, s, call, k, l (0-based),
        lshell [RE], mlt [h], log_obs.  Returns J per member."""
        kpa = np.asarray(kp, dtype=np.float64)
        if kpa.ndim == 1:
            kpa = np.repeat(kpa[:, None], self.n_members, axis=1)
        kpa = np.ascontiguousarray(kpa.reshape(ncalls, self.n_members))
        arr = (ObsStruct * max(1, len(obs)))()
        for t, o in enumerate(obs):
            arr[t] = ObsStruct(o["member"], o["s"], o["call"], o["k"], o["l"], o["lshell"], o["mlt"],
                               o["log_obs"])
        J = np.zeros(self.n_members)
        self._ck(self.lib.ramgpu_adj_forward(self.h, int(ncalls), float(dts), _dptr(kpa), int(k_ckpt),
                                             arr, len(obs), _dptr(J)), "adj_forward")
        return J

    def adj_backward(self):
        """(dJ/dF2 at the window start, dJ/dFGEOS): arrays of shape
        (members, ns, NR, NT, NE, NPA) and (members, ns, NT, NE, NPA), each
        trailing block in Fortran order like F2(S,:,:,:,:) / FGEOS(S,:,:,:)."""
        g = self.grid
        gf = np.zeros(self.n_members * self.ns * g.ncell)
        gb = np.zeros(self.n_members * self.ns * g.nt * g.ne * g.npa)
        self._ck(self.lib.ramgpu_adj_backward(self.h, _dptr(gf), _dptr(gb)), "adj_backward")
        gf = gf.reshape(self.n_members, self.ns, g.npa, g.ne, g.nt, g.nr).transpose(0, 1, 5, 4, 3, 2)
        gb = gb.reshape(self.n_members, self.ns, g.npa, g.ne, g.nt).transpose(0, 1, 4, 3, 2)
        return gf, gb

    def adj_record(self, call: int, nitems: int) -> np.ndarray:
        """Branch record of one call: (8 sweeps, items, NR*NT*NE*NPA) bytes."""
        g = self.grid
        out = np.zeros((8, nitems, g.ncell), dtype=np.uint8)
        self._ck(self.lib.ramgpu_adj_record(self.h, int(call), out.ctypes.data_as(C.POINTER(C.c_ubyte))),
                 "adj_record")
        return out

    def adj_replay(self) -> np.ndarray:
        """J per member of the last window replayed from the current F2 with
        the recorded branches frozen (needs k_ckpt >= ncalls)."""
        J = np.zeros(self.n_members)
        self._ck(self.lib.ramgpu_adj_replay(self.h, _dptr(J)), "adj_replay")
        return J

    def set_mu_lanes(self, lanes: int):
        """Lanes per DRIFTMU line (2: lane pairs, NPA >= 12; 1)."""
        self._ck(self.lib.ramgpu_set_mu_lanes(self.h, int(lanes)), "set_mu_lanes")

    def set_adj_record_budget(self, nbytes: int):
        """Device bytes the adjoint's branch-record ring may use (< 0: half of
        the free device memory; small: one segment, every earlier segment is
        recomputed)."""
        self._ck(self.lib.ramgpu_set_adj_record_budget(self.h, int(nbytes)), "set_adj_record_budget")

    def f2_stats(self, member: int, s: int):
        """(smallest F2, largest F2, number content sum F2*WE*WMU over the
        updated cells) of (member, s), one device pass (ramgpu_f2_stats)."""
        a, b, c = C.c_double(), C.c_double(), C.c_double()
        self._ck(self.lib.ramgpu_f2_stats(self.h, int(member), int(s), C.byref(a), C.byref(b), C.byref(c)),
                 "f2_stats")
        return a.value, b.value, c.value

    def bounds_report(self) -> dict:
        """The bounds-checked build's log (ramgpu_bounds_report): checked
        (1 in libramgpu_bounds.so), failures, the first failed check and its
        line."""
        ck, ch = C.c_int(), C.c_int()
        fl, va = C.c_longlong(), C.c_longlong()
        self._ck(self.lib.ramgpu_bounds_report(self.h, C.byref(ck), C.byref(fl), C.byref(ch), C.byref(va)),
                 "bounds_report")
        return {"checked": ck.value, "failures": fl.value, "check": ch.value, "value": va.value}

    def set_adj_overlap(self, on: bool):
        """Recompute segment s-1 on a second stream while segment s is
        transposed in adj_backward (default on; the ring then keeps at least
        two segments)."""
        self._ck(self.lib.ramgpu_set_adj_overlap(self.h, 1 if on else 0), "set_adj_overlap")

    def adj_segments(self):
        """(checkpoint segments, segments whose records are kept) of the last
        adj_forward."""
        a, b = C.c_int(), C.c_int()
        self._ck(self.lib.ramgpu_adj_segments(self.h, C.byref(a), C.byref(b)), "adj_segments")
        return a.value, b.value

    def adj_digest(self) -> int:
        v = C.c_ulonglong()
        self._ck(self.lib.ramgpu_adj_digest(self.h, C.byref(v)), "adj_digest")
        return int(v.value)

    def set_stream(self, stream_ptr: int):
        self._ck(self.lib.ramgpu_set_stream(self.h, C.c_void_p(stream_ptr)), "set_stream")

    def launch_count(self) -> int:
        return int(self.lib.ramgpu_launch_count(self.h))
