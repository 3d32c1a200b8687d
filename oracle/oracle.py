"""ctypes front end of the CPU oracle (phinum_oracle.c) and of the reference
pin (oracle/_ref/libphinum_ref_*.so, built by oracle/build_ref.sh).

TEST INFRASTRUCTURE.  Only tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg import this module.  Arrays are float64 in the reference's
layout: Nc*N*N*(N+2) values, index Nc*(x + N*y + N*N*z) + a, z-slabs 0 and
N+1 are ghosts (lattice.cpp:76-78, util.cpp:34-37).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
MAX_NC = 4
AVG_FIELDS = (["t"] + [f"phi{a}" for a in range(MAX_NC)] + [f"pi{a}" for a in range(MAX_NC)] +
              ["phi2", "pi2", "phipi", "phi4", "phi6", "energy", "interaction", "charge",
               "min_phi", "max_phi", "max_abs_phi", "min_pos", "max_pos", "max_abs_pos",
               "gradient", "reserved0", "reserved1"])
AVG_LEN = len(AVG_FIELDS)
AVG = {k: i for i, k in enumerate(AVG_FIELDS)}
ISLAND_FIELDS = ["index", "size", "volume", "pot_en", "kin_en", "grad_en", "av_phi",
                 "peak_pos", "peak_value", "seed_pos"]
ISL = {k: i for i, k in enumerate(ISLAND_FIELDS)}

_D = ctypes.c_double
_I = ctypes.c_int
_PD = ctypes.POINTER(ctypes.c_double)
_PI = ctypes.POINTER(ctypes.c_int)


@dataclass
class Params:
    """Reference run parameters (parameters.cpp:84-201)."""
    N: int = 8
    Nc: int = 1
    theory: int = 0
    mass_mode: int = 1
    lambda_mode: int = -1
    a: float = 0.25
    dt: float = 0.08
    T0: float = 0.0
    m_sqr: float = 1.0
    kappa: float = 3.0 ** 0.5
    h: float = 0.0
    g: float = 2.0            # theory 4
    p_mono: float = -0.5      # theory 5
    m_mono_sqr: float = 1.0   # theory 3
    expansion: int = 0        # 1: radiation-era expanding box
    H0: float = 0.0171156     # H_0 (parameters.cpp:177)


class _CParams(ctypes.Structure):
    _fields_ = [("N", _I), ("Nc", _I), ("theory", _I), ("mass_mode", _I), ("lambda_mode", _I),
                ("expansion", _I), ("a", _D), ("dt", _D), ("T0", _D), ("m_sqr", _D), ("kappa", _D),
                ("h", _D), ("g", _D), ("p_mono", _D), ("m_mono_sqr", _D), ("H0", _D)]


class _CClock(ctypes.Structure):
    _fields_ = [("tau", _D), ("dtau", _D), ("last_mom", _D), ("last_field", _D),
                ("steps", _I), ("pad_", _I), ("tau_c", _D), ("sf", _D), ("last_mom_c", _D),
                ("last_field_c", _D)]


class _CClock32(ctypes.Structure):
    _fields_ = [("tau", ctypes.c_float), ("dtau", ctypes.c_float), ("last_mom", ctypes.c_float),
                ("last_field", ctypes.c_float), ("steps", _I), ("pad_", _I)]


class _CIc(ctypes.Structure):
    _fields_ = [("seed", ctypes.c_long), ("justnoise", _I), ("pad_", _I), ("QS", _D), ("scale2", _D),
                ("amplitude", _D), ("noise", _D), ("phi0", _D * 2), ("pi0", _D * 2), ("m2_long", _D),
                ("m2_trans", _D), ("initialize", _I), ("withcharge", _I), ("chi", _D), ("famp", _D), ("lambda_", _D),
                ("temperature", _D), ("phi0s", _D), ("pi0s", _D)]


# SetInitialConditions parameters: the reference globals' names; initialize
# and withcharge are its compile-time switches (parameters.cpp:205, :51), the
# last six the globals of initialize 0-2 (phi0s, pi0s: its phi0, pi0)
IC_DEFAULTS = dict(seed=1, justnoise=0, QS=1.0, scale2=1.0, amplitude=0.0, noise=0.5, phi0=(0.0, 0.0),
                   pi0=(0.0, 0.0), initialize=3, withcharge=0, chi=1.0, famp=0.5, lambda_=1.0, temperature=1.0,
                   phi0s=0.0, pi0s=0.0)


def _cp(p: Params) -> _CParams:
    return _CParams(p.N, p.Nc, p.theory, p.mass_mode, p.lambda_mode, int(p.expansion), p.a, p.dt, p.T0,
                    p.m_sqr, p.kappa, p.h, p.g, p.p_mono, p.m_mono_sqr, p.H0)


def _ptr(a: np.ndarray, kind=_PD):
    return a.ctypes.data_as(kind)


def field_len(p: Params) -> int:
    return p.Nc * p.N * p.N * (p.N + 2)


def to_ref_layout(field: np.ndarray, Nc: int = 1) -> np.ndarray:
    """[Nc][z][y][x] (or [z][y][x]) -> reference layout with ghost slabs."""
    f = np.asarray(field, dtype=np.float64)
    if f.ndim == 3:
        f = f[None]
    nc, n = f.shape[0], f.shape[1]
    out = np.zeros((n + 2, n, n, nc))
    out[1:n + 1] = np.moveaxis(f, 0, -1)
    out[0] = out[n]
    out[n + 1] = out[1]
    return out.reshape(-1)


def from_ref_layout(flat: np.ndarray, N: int, Nc: int = 1) -> np.ndarray:
    """reference layout -> [Nc][z][y][x] interior."""
    f = np.asarray(flat).reshape(N + 2, N, N, Nc)[1:N + 1]
    return np.ascontiguousarray(np.moveaxis(f, -1, 0))


# ----------------------------------------------------------------- build ---
def lib_path(fast: bool = False) -> str:
    return os.path.join(HERE, "libphinum_oracle_fast.so" if fast else "libphinum_oracle.so")


def build(force: bool = False) -> None:
    """Compile phinum_oracle.c twice: an exact build (no fast-math, no FP
    contraction; the parity checker) and a timing build with the reference's
    own optimisation flags minus the x86-only ones (run_PC.pbs:1)."""
    src = os.path.join(HERE, "phinum_oracle.c")
    variants = [
        (lib_path(False), ["-O2", "-ffp-contract=off", "-fno-fast-math"]),
        (lib_path(True), ["-O3", "-ffast-math", "-funroll-all-loops", "-fprefetch-loop-arrays"]),
    ]
    procs = []
    for out, flags in variants:
        if not force and os.path.exists(out) and os.path.getmtime(out) >= max(
                os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "phinum_oracle.h"))):
            continue
        for omp in (["-fopenmp"], []):
            cmd = ["gcc", "-std=c99", "-fPIC", "-shared", *flags, *omp, src, "-o", out + ".tmp", "-lm"]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode == 0:
                os.replace(out + ".tmp", out)
                break
        else:
            raise RuntimeError("oracle build failed:\n" + r.stderr)
    del procs


_libs: dict = {}


def _load(fast: bool = False):
    key = "fast" if fast else "exact"
    if key not in _libs:
        path = lib_path(fast)
        build()  # rebuilds only when the C source is newer than the library
        lib = ctypes.CDLL(path)
        lib.orc_evolve.argtypes = [ctypes.POINTER(_CParams), ctypes.POINTER(_CClock), _PD, _PD, _I, _I]
        lib.orc_reset.argtypes = [ctypes.POINTER(_CParams), ctypes.POINTER(_CClock)]
        lib.orc_averages.argtypes = [ctypes.POINTER(_CParams), ctypes.POINTER(_CClock), _PD, _PD, _PD]
        lib.orc_run_loop.argtypes = [ctypes.POINTER(_CParams), ctypes.POINTER(_CClock), _PD, _PD, _I, _D,
                                     _PD, _I, _I]
        lib.orc_run_loop.restype = _I
        lib.orc_spectrum_bins.argtypes = [ctypes.POINTER(_CParams), _PI, _PD]
        lib.orc_spectrum.argtypes = [ctypes.POINTER(_CParams), _PD, _PD, _PD, _PD, _PD, _PI]
        lib.orc_spectrum.restype = _I
        lib.orc_spectrum_uniform.argtypes = [ctypes.POINTER(_CParams), _PD, _PD, _I, _PD, _PD, _PD, _PI]
        lib.orc_spectrum_uniform.restype = _I
        lib.orc_initial_conditions.argtypes = [ctypes.POINTER(_CParams), ctypes.POINTER(_CIc), _PD, _PD]
        lib.orc_initial_conditions.restype = _I
        lib.orc_apply_filter.argtypes = [ctypes.POINTER(_CParams), _PD, _PD, _D, _I, _PD, _I, _D]
        lib.orc_apply_filter.restype = _I
        lib.orc_spectrum_columns.argtypes = [ctypes.POINTER(_CParams), _PD, _PD, _PD, _PI, _I, _PD]
        lib.orc_islands_at.argtypes = [ctypes.POINTER(_CParams), ctypes.POINTER(_CClock), _PD, _PD, _D, _I, _I,
                                       _PI, _PD, _I]
        lib.orc_islands_at.restype = _I
        lib.orc_site_energy_at.argtypes = [ctypes.POINTER(_CParams), ctypes.POINTER(_CClock), _PD, _PD,
                                           ctypes.c_long, _I, _I, _I]
        lib.orc_site_energy_at.restype = _D
        lib.orc_max_threads.restype = _I
        _PF = ctypes.POINTER(ctypes.c_float)
        lib.orc_reset_f32.argtypes = [ctypes.POINTER(_CParams), ctypes.POINTER(_CClock32)]
        lib.orc_evolve_f32.argtypes = [ctypes.POINTER(_CParams), ctypes.POINTER(_CClock32), _PF, _PF, _I, _I]
        _libs[key] = lib
    return _libs[key]


class Clock:
    """numeric:: time keeping (tau, dtau, last kick/drift times, steps)."""

    def __init__(self, p: Params, fast: bool = False):
        self.p, self._c, self.fast = p, _CClock(), fast
        _load(fast).orc_reset(ctypes.byref(_cp(p)), ctypes.byref(self._c))

    @property
    def tau(self) -> float:
        return self._c.tau

    @property
    def steps(self) -> int:
        return self._c.steps

    @property
    def tau_c(self) -> float:
        """Conformal time (tau for the static box)."""
        return self._c.tau_c

    @property
    def sf(self) -> float:
        """Scale factor (1 for the static box)."""
        return self._c.sf


class Clock32:
    """The single-precision build's clock (float tau, dtau, update stamps)."""

    def __init__(self, p: Params, fast: bool = False):
        self.p, self._c, self.fast = p, _CClock32(), fast
        _load(fast).orc_reset_f32(ctypes.byref(_cp(p)), ctypes.byref(self._c))

    @property
    def tau(self) -> float:
        return self._c.tau

    @property
    def steps(self) -> int:
        return self._c.steps


def evolve_f32(p: Params, phi: np.ndarray, pi: np.ndarray, nsteps: int, clock: Clock32 | None = None,
               nthreads: int = 1, fast: bool = False) -> Clock32:
    """n x evolve() of the reference's single-precision build (theories 0, 1,
    static box) in place on reference-layout float32 arrays."""
    assert phi.dtype == np.float32 and pi.dtype == np.float32 and phi.flags.c_contiguous
    assert phi.size == field_len(p) and pi.size == field_len(p) and p.theory in (0, 1) and not p.expansion
    clock = clock or Clock32(p, fast)
    pf = ctypes.POINTER(ctypes.c_float)
    _load(fast).orc_evolve_f32(ctypes.byref(_cp(p)), ctypes.byref(clock._c), phi.ctypes.data_as(pf),
                               pi.ctypes.data_as(pf), int(nsteps), int(nthreads))
    return clock


def max_threads(fast: bool = True) -> int:
    return int(_load(fast).orc_max_threads())


def evolve(p: Params, phi: np.ndarray, pi: np.ndarray, nsteps: int, clock: Clock | None = None,
           nthreads: int = 1, fast: bool = False) -> Clock:
    """n x evolve() in place on reference-layout float64 arrays."""
    assert phi.dtype == np.float64 and pi.dtype == np.float64 and phi.flags.c_contiguous
    assert phi.size == field_len(p) and pi.size == field_len(p)
    clock = clock or Clock(p, fast)
    _load(fast).orc_evolve(ctypes.byref(_cp(p)), ctypes.byref(clock._c), _ptr(phi), _ptr(pi),
                           int(nsteps), int(nthreads))
    return clock


def averages(p: Params, phi: np.ndarray, pi: np.ndarray, clock: Clock | None = None) -> np.ndarray:
    out = np.zeros(AVG_LEN)
    _load().orc_averages(ctypes.byref(_cp(p)), ctypes.byref(clock._c) if clock else None, _ptr(phi),
                         _ptr(pi), _ptr(out))
    return out


def run_loop(p: Params, phi: np.ndarray, pi: np.ndarray, nsteps: int, tso: float,
             max_rows: int = 10000, nthreads: int = 1):
    clock = Clock(p)
    rows = np.zeros((max_rows, AVG_LEN))
    n = _load().orc_run_loop(ctypes.byref(_cp(p)), ctypes.byref(clock._c), _ptr(phi), _ptr(pi),
                             int(nsteps), float(tso), _ptr(rows), max_rows, int(nthreads))
    return rows[:n], clock


def false_vacuum_decayed(interaction: float, theory: int) -> bool:
    """false_vacuum_decayed() (fieldanalysis.cpp:887-893): for theories 0, 1
    and 4 the vacuum has decayed when <V> < 0, <V> is NaN, or <V> * 0 != 0
    (an infinity); the other theories never stop."""
    v = float(interaction)
    if theory not in (0, 1, 4):
        return False
    return v < 0 or v != v or v * 0.0 != 0.0


def stop_step(rows: np.ndarray, theory: int, step_of_row) -> int:
    """Where main.cpp:77-90 breaks: false_vacuum_decayed() reads the averages
    of the last row computed, so the loop stops at the first row whose
    interaction decays it, before that step's evolve().  step_of_row(i) is
    row i's step count; -1 when no row decays it."""
    for i in range(rows.shape[0]):
        if false_vacuum_decayed(rows[i, 15], theory):
            return int(step_of_row(i))
    return -1


def spectrum_bins(p: Params):
    nb, bs = _I(), _D()
    _load().orc_spectrum_bins(ctypes.byref(_cp(p)), ctypes.byref(nb), ctypes.byref(bs))
    return nb.value, bs.value


def spectrum(p: Params, phi: np.ndarray, pi: np.ndarray):
    nb, _ = spectrum_bins(p)
    F, K, Q = (np.zeros(nb * p.Nc) for _ in range(3))
    C = np.zeros(nb, dtype=np.int32)
    r = _load().orc_spectrum(ctypes.byref(_cp(p)), _ptr(phi), _ptr(pi), _ptr(F), _ptr(K), _ptr(Q),
                             _ptr(C, _PI))
    if r < 0:
        raise RuntimeError("bin array too small")
    return F, K, Q, C


def spectrum_uniform(p: Params, phi: np.ndarray, pi: np.ndarray, nbins: int = 64):
    """Config-mode spectrum: nbins uniform |p| bins on [0, p_max]."""
    F, K, Q = (np.zeros(nbins * p.Nc) for _ in range(3))
    C = np.zeros(nbins, dtype=np.int32)
    _load().orc_spectrum_uniform(ctypes.byref(_cp(p)), _ptr(phi), _ptr(pi), int(nbins), _ptr(F), _ptr(K), _ptr(Q),
                                 _ptr(C, _PI))
    return F, K, Q, C


def initial_conditions(p: Params, **kw):
    """SetInitialConditions (initialize 0-4, withcharge 0/1; default 3, 0)
    with srand48(seed): Phi, Pi in the reference layout (Pi's ghost slabs
    zero).  M2_long = M2_trans = M_sqr."""
    q = dict(IC_DEFAULTS, **kw)
    c = _CIc(int(q["seed"]), int(q["justnoise"]), 0, q["QS"], q["scale2"], q["amplitude"], q["noise"],
             (_D * 2)(*q["phi0"]), (_D * 2)(*q["pi0"]), p.m_sqr, p.m_sqr, int(q["initialize"]),
             int(q["withcharge"]), q["chi"], q["famp"], q["lambda_"], q["temperature"], q["phi0s"], q["pi0s"])
    phi, pi = np.zeros(field_len(p)), np.zeros(field_len(p))
    if _load().orc_initial_conditions(ctypes.byref(_cp(p)), ctypes.byref(c), _ptr(phi), _ptr(pi)) != 0:
        raise ValueError("initialize/withcharge combination the reference does not define")
    return phi, pi


def apply_filter(p: Params, phi: np.ndarray, pi: np.ndarray, r: float, which: int, table=None, dp: float = 0.0):
    """apply_filter on copies of Phi, Pi (reference layout); returns them."""
    phi, pi = np.array(phi, dtype=np.float64), np.array(pi, dtype=np.float64)
    t = np.ascontiguousarray(table if table is not None else np.zeros(1), dtype=np.float64)
    _load().orc_apply_filter(ctypes.byref(_cp(p)), _ptr(phi), _ptr(pi), float(r), int(which), _ptr(t), t.size,
                             float(dp))
    return phi, pi


def spectrum_columns(p: Params, F, K, Q, C) -> np.ndarray:
    nb = C.size
    cols = np.zeros((nb, 7))
    _load().orc_spectrum_columns(ctypes.byref(_cp(p)), _ptr(F), _ptr(K), _ptr(Q),
                                 _ptr(np.ascontiguousarray(C, dtype=np.int32), _PI), nb, _ptr(cols))
    return cols


def site_energy(p: Params, phi: np.ndarray, pi: np.ndarray, clock: Clock | None = None) -> np.ndarray:
    """rho(x) for every interior site, [z][y][x] (slow; small lattices only).
    The expanding box reads the scale factor from clock."""
    N = p.N
    out = np.zeros((N, N, N))
    lib = _load()
    cp = ctypes.byref(_cp(p))
    ck = ctypes.byref(clock._c) if clock else None
    for z in range(N):
        for y in range(N):
            for x in range(N):
                K = p.Nc * (x + N * y + N * N * (z + 1))
                out[z, y, x] = lib.orc_site_energy_at(cp, ck, _ptr(phi), _ptr(pi), K, x, y, z + 1)
    return out


def islands(p: Params, phi: np.ndarray, pi: np.ndarray, thres: float, mode: int = 0, zper: int = 0,
            max_islands: int = 1 << 20, clock: Clock | None = None):
    """Returns (labels in reference layout, island records [n][10]).  The
    expanding box reads the scale factor from clock."""
    labels = np.zeros(field_len(p), dtype=np.int32)
    recs = np.zeros((max_islands, len(ISLAND_FIELDS)))
    n = _load().orc_islands_at(ctypes.byref(_cp(p)), ctypes.byref(clock._c) if clock else None, _ptr(phi),
                               _ptr(pi), float(thres), int(mode), int(zper), _ptr(labels, _PI), _ptr(recs),
                               max_islands)
    if n == -2:
        raise ValueError(f"no Delta mask for theory {p.theory}")
    if n < 0:
        raise MemoryError("oracle islands: allocation failed")
    return labels, recs[:min(n, max_islands)]


def delta(p: Params, phi: np.ndarray, pi: np.ndarray, clock: Clock | None = None) -> np.ndarray:
    """Delta of every component of every interior site (withEnergyPS 1,
    fieldanalysis.cpp:446-560), the reference layout's interior: Nc N^3
    values.  Theories 2-5 only, as the reference compiles them."""
    lib = _load()
    lib.orc_delta_at.restype = ctypes.c_int
    out = np.zeros(p.Nc * p.N ** 3)
    r = lib.orc_delta_at(ctypes.byref(_cp(p)), ctypes.byref(clock._c) if clock else None, _ptr(phi), _ptr(pi),
                         _ptr(out))
    if r:
        raise ValueError(f"no Delta for theory {p.theory} (the reference's withEnergyPS forms need theory 2-5)")
    return out


def spectrum_energy(p: Params, phi: np.ndarray, pi: np.ndarray, clock: Clock | None = None):
    """The density-contrast spectrum (momentumspace.cpp:165-183, 233-270):
    (D[bin*Nc + a], counts)."""
    lib = _load()
    lib.orc_spectrum_energy_at.restype = ctypes.c_int
    nb, _ = spectrum_bins(p)
    D = np.zeros(nb * p.Nc)
    C = np.zeros(nb, dtype=np.int32)
    r = lib.orc_spectrum_energy_at(ctypes.byref(_cp(p)), ctypes.byref(clock._c) if clock else None, _ptr(phi),
                                   _ptr(pi), _ptr(D), _ptr(C, _PI))
    if r == -2:
        raise ValueError(f"no Delta for theory {p.theory}")
    if r < 0:
        raise MemoryError("oracle energy spectrum: allocation failed")
    return D, C


# ------------------------------------------------------ the reference pin ---
REF_DIR = os.path.join(HERE, "_ref")


def ref_dir() -> str:
    """The reference tree the pin builds from: REF_DIR, with the default of
    oracle/build_ref.sh."""
    return os.environ.get("REF_DIR", "/root/reference")


def ref_path(theory: int = 0, precision: str = "f64", expansion: int = 0, variant: str = "") -> str:
    """variant: "" (initialize 3), "_ic0", "_ic1", "_ic2", "_ic4" (other
    initialize switches), "_ic2q", "_ic3q" (withcharge 1)."""
    return os.path.join(REF_DIR, f"libphinum_ref_t{theory}_{precision}{'_exp' if expansion else ''}{variant}.so")


def ref_available(theory: int = 0, precision: str = "f64", expansion: int = 0, variant: str = "") -> bool:
    return os.path.exists(ref_path(theory, precision, expansion, variant))


class Reference:
    """The reference's own sources (single rank, shims) behind ctypes.  One
    instance per process and variant: the reference keeps global state."""

    def __init__(self, p: Params, precision: str = "f64", variant: str = ""):
        self.p = p
        lib = ctypes.CDLL(ref_path(p.theory, precision, p.expansion, variant))
        lib.ref_init.argtypes = [_I, _I, _D, _D, _D, _I, _D, _I, _D, _D, _D]
        lib.ref_init.restype = _I
        lib.ref_set_fields.argtypes = [_PD, _PD]
        lib.ref_get_fields.argtypes = [_PD, _PD]
        lib.ref_evolve.argtypes = [_I]
        lib.ref_time.argtypes = [_PD, _PI]
        lib.ref_averages.argtypes = [_PD]
        lib.ref_run_loop.argtypes = [_I, _D, _PD, _I]
        lib.ref_run_loop.restype = _I
        lib.ref_binsize.restype = _D
        lib.ref_spectrum.argtypes = [_PD, _PD, _PD, _PI]
        lib.ref_islands.argtypes = [_D, _PI, _PD, _I]
        lib.ref_islands.restype = _I
        lib.ref_save_config.argtypes = [_I]
        lib.ref_apply_filter.argtypes = [_D, _I, _PD, _I, _D]
        lib.ref_apply_filter.restype = _I
        lib.ref_track_step.argtypes = [_D, _PI]
        lib.ref_track_step.restype = _I
        lib.ref_track_island.argtypes = [_I, _PD]
        lib.ref_track_island.restype = _I
        lib.ref_initial_conditions.argtypes = [ctypes.c_long, _I, _D, _D, _D, _D, _D, _D, _D, _D]
        lib.ref_initial_conditions.restype = _I
        self.lib = lib
        lib.ref_set_extra.argtypes = [_D, _D, _D]
        lib.ref_set_extra(p.g, p.p_mono, p.m_mono_sqr)
        lib.ref_set_h0.argtypes = [_D]
        lib.ref_set_h0(p.H0)
        lib.ref_expansion_state.argtypes = [_PD, _PD]
        r = lib.ref_init(p.N, p.Nc, p.a, p.dt, p.T0, p.mass_mode, p.m_sqr, p.lambda_mode, 1.0,
                         p.kappa, p.h)
        if r != 0:
            raise RuntimeError(f"ref_init failed ({r}); one Reference per process")

    def initial_conditions(self, **kw):
        """The reference's SetInitialConditions with srand48(seed) (the
        build's initialize / withcharge switches); returns Phi, Pi."""
        q = dict(IC_DEFAULTS, **kw)
        self.lib.ref_set_ic_extra.argtypes = [_D] * 6
        self.lib.ref_set_ic_extra(q["chi"], q["famp"], q["lambda_"], q["temperature"], q["phi0s"], q["pi0s"])
        r = self.lib.ref_initial_conditions(int(q["seed"]), int(q["justnoise"]), q["QS"], q["scale2"],
                                            q["amplitude"], q["noise"], q["phi0"][0], q["phi0"][1],
                                            q["pi0"][0], q["pi0"][1])
        if r != 0:
            raise RuntimeError("ref_initial_conditions failed")
        return self.get_fields()

    def apply_filter(self, r: float, which: int, table=None, dp: float = 0.0):
        """The reference's apply_filter on its current fields; returns Phi, Pi."""
        t = np.ascontiguousarray(table if table is not None else np.zeros(1), dtype=np.float64)
        if self.lib.ref_apply_filter(float(r), int(which), _ptr(t), t.size, float(dp)) != 0:
            raise RuntimeError("ref_apply_filter failed")
        return self.get_fields()

    def save_config(self, name: int):
        """The reference's SaveConfig: files in the working directory."""
        self.lib.ref_save_config(int(name))

    def track_reset(self):
        self.lib.ref_track_reset()

    def track_step(self, thres: float):
        """Full_Analysis() on the current fields; returns the tracked islands
        as an (n, 44) array: index, status, disp, L, then 5 x (at_time, centre,
        V, PotEn, KinEn, GradEn, avPhi, Peak_value), unused entries zero."""
        n = self.lib.ref_track_step(float(thres), None)
        out = np.zeros((n, 44))
        for i in range(n):
            self.lib.ref_track_island(i, _ptr(out[i]))
        return out

    def set_fields(self, phi, pi):
        self.lib.ref_set_fields(_ptr(np.ascontiguousarray(phi, np.float64)),
                                _ptr(np.ascontiguousarray(pi, np.float64)))

    def get_fields(self):
        n = field_len(self.p)
        phi, pi = np.zeros(n), np.zeros(n)
        self.lib.ref_get_fields(_ptr(phi), _ptr(pi))
        return phi, pi

    def reset(self):
        self.lib.ref_reset()

    def evolve(self, n: int):
        self.lib.ref_evolve(int(n))

    def time(self):
        t, s = _D(), _I()
        self.lib.ref_time(ctypes.byref(t), ctypes.byref(s))
        return t.value, s.value

    def expansion_state(self):
        """(conformal time, scale factor); (tau, 1) for the static box."""
        tc, sf = _D(), _D()
        self.lib.ref_expansion_state(ctypes.byref(tc), ctypes.byref(sf))
        return tc.value, sf.value

    def averages(self) -> np.ndarray:
        out = np.zeros(AVG_LEN)
        self.lib.ref_averages(_ptr(out))
        return out

    def run_loop(self, nsteps: int, tso: float, max_rows: int = 10000) -> np.ndarray:
        rows = np.zeros((max_rows, AVG_LEN))
        n = self.lib.ref_run_loop(int(nsteps), float(tso), _ptr(rows), max_rows)
        return rows[:n]

    def false_vacuum_decayed(self, interaction: float) -> bool:
        """The reference's false_vacuum_decayed() with avgInteraction set."""
        self.lib.ref_false_vacuum_decayed.argtypes = [_D]
        self.lib.ref_false_vacuum_decayed.restype = _I
        return bool(self.lib.ref_false_vacuum_decayed(float(interaction)))

    def run_until_decayed(self, nsteps: int, tso: float, max_rows: int = 10000):
        """main.cpp:77-90 with the false-vacuum break: (rows, stop step or -1)."""
        self.lib.ref_run_until_decayed.argtypes = [_I, _D, _PD, _I, _PI]
        self.lib.ref_run_until_decayed.restype = _I
        rows = np.zeros((max_rows, AVG_LEN))
        stop = _I()
        n = self.lib.ref_run_until_decayed(int(nsteps), float(tso), _ptr(rows), max_rows, ctypes.byref(stop))
        return rows[:n], stop.value

    def spectrum(self):
        nb = self.lib.ref_nbins()
        F, K, Q = (np.zeros(nb * self.p.Nc) for _ in range(3))
        C = np.zeros(nb, dtype=np.int32)
        self.lib.ref_spectrum(_ptr(F), _ptr(K), _ptr(Q), _ptr(C, _PI))
        return F, K, Q, C

    def islands(self, thres: float, max_islands: int = 1 << 16):
        labels = np.zeros(field_len(self.p), dtype=np.int32)
        stats = np.zeros((max_islands, 8))
        n = self.lib.ref_islands(float(thres), _ptr(labels, _PI), _ptr(stats), max_islands)
        return labels, stats[:min(n, max_islands)]

    def island_thres(self) -> float:
        """The threshold of the last Full_Analysis (EnergybasedID: 4 <rho>)."""
        self.lib.ref_island_thres.restype = _D
        return self.lib.ref_island_thres()

    def delta(self) -> np.ndarray:
        """withEnergyPS builds: Delta of the current fields (interior)."""
        out = np.zeros(self.p.Nc * self.p.N ** 3)
        self.lib.ref_delta(_ptr(out))
        return out

    def spectrum_energy(self):
        """withEnergyPS builds: Calculate_CorrelationFunctions' TotalCorrD
        (note: the reference turns Delta into the density contrast in place)."""
        F, K, Q, C = self.spectrum()
        D = np.zeros(self.lib.ref_nbins() * self.p.Nc)
        self.lib.ref_spectrum_d(_ptr(D))
        return D, C
