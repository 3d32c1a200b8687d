"""Python mirror of the reference's hot-path entry points over the C ABI.

One `Lattice` is one reference run: `LocalLattice` fields on the GPU plus the
reference clock.  Method names follow the reference functions they replace:

    reset()                     dynamics.cpp:28-50
    evolve(n)                   n x evolve(), dynamics.cpp:196-237
    volume_averages()           CalculateExtrema + CalculateVolumeAverages,
                                fieldanalysis.cpp:319-699
    run_loop(n, TSO)            main.cpp:685-699 with Print_AveragesExtrema's cadence
    correlation_functions()     Calculate_CorrelationFunctions, momentumspace.cpp:140-278
    full_analysis(thres)        Full_Analysis seeding, islands.cpp:778-840

Arrays are numpy float64 in the reference layout (Nc*N*N*(N+2), ghost slabs).
Errors raise PhnError carrying the library's status code.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _lib as L


@dataclass
class Params:
    """Reference run parameters (parameters.cpp:84-201)."""
    N: int = 64
    Nc: int = 1
    theory: int = 0
    mass_mode: int = 1
    lambda_mode: int = -1
    precision: int = L.FP64
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

    def c(self) -> L.PhnParams:
        return L.PhnParams(self.N, self.Nc, self.theory, self.mass_mode, self.lambda_mode, self.precision,
                           self.a, self.dt, self.T0, self.m_sqr, self.kappa, self.h, self.g, self.p_mono,
                           self.m_mono_sqr, int(self.expansion), 0, self.H0)

    @property
    def field_len(self) -> int:
        return self.Nc * self.N * self.N * (self.N + 2)


def _pd(a: np.ndarray):
    return a.ctypes.data_as(L._PD)


def _pi(a: np.ndarray):
    return a.ctypes.data_as(L._PI)


def avg_array(a: L.PhnAverages) -> np.ndarray:
    return np.frombuffer(bytes(a), dtype=np.float64).copy()


class Lattice:
    def __init__(self, p: Params):
        self.p = p
        self.lib = L.load()
        h = ctypes.c_void_p()
        L.check(self.lib.phn_create(ctypes.byref(p.c()), ctypes.byref(h)))
        self.h = h

    def close(self):
        if self.h:
            self.lib.phn_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------- fields
    def upload(self, phi: np.ndarray, pi: np.ndarray):
        """Reference-layout fields; float32 arrays go through phn_upload_f32
        (the reference's single-precision build), anything else as float64."""
        if phi.dtype == np.float32 and pi.dtype == np.float32:
            phi, pi = np.ascontiguousarray(phi), np.ascontiguousarray(pi)
            assert phi.size == self.p.field_len and pi.size == self.p.field_len
            L.check(self.lib.phn_upload_f32(self.h, phi.ctypes.data, pi.ctypes.data))
            return
        phi = np.ascontiguousarray(phi, dtype=np.float64)
        pi = np.ascontiguousarray(pi, dtype=np.float64)
        assert phi.size == self.p.field_len and pi.size == self.p.field_len
        L.check(self.lib.phn_upload(self.h, _pd(phi), _pd(pi)))

    def download(self, dtype=np.float64):
        """Reference-layout fields as float64, or as float32 through
        phn_download_f32."""
        phi = np.zeros(self.p.field_len, dtype=dtype)
        pi = np.zeros(self.p.field_len, dtype=dtype)
        if np.dtype(dtype) == np.float32:
            L.check(self.lib.phn_download_f32(self.h, phi.ctypes.data, pi.ctypes.data))
        else:
            L.check(self.lib.phn_download(self.h, _pd(phi), _pd(pi)))
        return phi, pi

    def initial_conditions(self, seed: int = 1, justnoise: int = 0, QS: float = 1.0, scale2: float = 1.0,
                           amplitude: float = 0.0, noise: float = 0.5, phi0=(0.0, 0.0), pi0=(0.0, 0.0),
                           m2_long: float | None = None, m2_trans: float | None = None, initialize: int = 3,
                           withcharge: int = 0, chi: float = 1.0, famp: float = 0.5, lambda_: float = 1.0,
                           temperature: float = 1.0, phi0s: float = 0.0, pi0s: float = 0.0):
        """SetInitialConditions on the device with the reference's drand48
        stream from srand48(seed): initialize 3 without charge through
        phn_initial_conditions, any other initialize / withcharge through
        phn_initial_conditions_mode (phi0s, pi0s: the phi0, pi0 of
        initialize 0-2).  M2_long and M2_trans default to M_sqr
        (renormalization.cpp:17-18)."""
        m2l = self.p.m_sqr if m2_long is None else m2_long
        m2t = self.p.m_sqr if m2_trans is None else m2_trans
        ic = L.PhnIcParams(int(seed), int(justnoise), QS, scale2, amplitude, noise, (ctypes.c_double * 2)(*phi0),
                           (ctypes.c_double * 2)(*pi0), m2l, m2t)
        if initialize == 3 and not withcharge:
            L.check(self.lib.phn_initial_conditions(self.h, ctypes.byref(ic)))
            return
        md = L.PhnIcMode(int(initialize), int(withcharge), chi, famp, lambda_, temperature, phi0s, pi0s)
        L.check(self.lib.phn_initial_conditions_mode(self.h, ctypes.byref(ic), ctypes.byref(md)))

    def apply_filter(self, r_filter: float, which: int, table=None, dp: float = 0.0):
        """apply_filter (filter.cpp:53-133): 0 top hat, 1 Gaussian, 2 table, 3 sharp cut."""
        t = np.ascontiguousarray(table if table is not None else np.zeros(1), dtype=np.float64)
        L.check(self.lib.phn_apply_filter(self.h, float(r_filter), int(which), _pd(t), t.size, float(dp)))

    def save_config(self, name: int, directory: str = ".", rank: int = 0, nthreads: int = 0):
        """SaveConfig: field-<name>-<rank>.out (and moment-<name>.out) in the reference's format."""
        L.check(self.lib.phn_save_config(self.h, directory.encode(), int(name), int(rank), int(nthreads)))

    def load_config(self, name: int, directory: str = ".", rank: int = 0, nthreads: int = 0) -> float:
        """ExtractConfig: reads the files back; returns the time stamp (the reference's T0)."""
        t0 = ctypes.c_double()
        L.check(self.lib.phn_load_config(self.h, directory.encode(), int(name), int(rank), ctypes.byref(t0),
                                         int(nthreads)))
        return t0.value

    # -------------------------------------------------------------- clock
    def reset(self):
        L.check(self.lib.phn_reset(self.h))

    def evolve(self, n: int):
        L.check(self.lib.phn_evolve(self.h, int(n)))

    def time(self):
        t, s = ctypes.c_double(), ctypes.c_int()
        L.check(self.lib.phn_time(self.h, ctypes.byref(t), ctypes.byref(s)))
        return t.value, s.value

    def conformal_time(self):
        """(conformal time, scale factor); (tau, 1) for the static box."""
        tc, sf = ctypes.c_double(), ctypes.c_double()
        L.check(self.lib.phn_conformal_time(self.h, ctypes.byref(tc), ctypes.byref(sf)))
        return tc.value, sf.value

    # ----------------------------------------------------------- analysis
    def volume_averages(self, allow_nonfinite: bool = False) -> np.ndarray:
        a = L.PhnAverages()
        r = self.lib.phn_volume_averages(self.h, ctypes.byref(a))
        if not (allow_nonfinite and r == L.ERR_NONFINITE):
            L.check(r)
        return avg_array(a)

    def run_loop(self, nsteps: int, tso: float, max_rows: int = 100000) -> np.ndarray:
        rows = (L.PhnAverages * max_rows)()
        n = ctypes.c_int()
        L.check(self.lib.phn_run_loop(self.h, int(nsteps), float(tso), rows, max_rows, ctypes.byref(n)))
        out = np.frombuffer(bytes(rows), dtype=np.float64).reshape(max_rows, L.AVG_LEN)
        return out[:n.value].copy()

    def spectrum_bins(self):
        nb, bs = ctypes.c_int(), ctypes.c_double()
        L.check(self.lib.phn_spectrum_bins(self.h, ctypes.byref(nb), ctypes.byref(bs)))
        return nb.value, bs.value

    def correlation_functions(self):
        nb, _ = self.spectrum_bins()
        F, K, Q = (np.zeros(nb * self.p.Nc) for _ in range(3))
        C = np.zeros(nb, dtype=np.int32)
        L.check(self.lib.phn_spectrum(self.h, _pd(F), _pd(K), _pd(Q), _pi(C), nb))
        return F, K, Q, C

    def spectrum_uniform(self, nbins: int = 64):
        """The configuration's radial spectrum: nbins uniform |p| bins on [0, p_max]."""
        F, K, Q = (np.zeros(nbins * self.p.Nc) for _ in range(3))
        C = np.zeros(nbins, dtype=np.int32)
        L.check(self.lib.phn_spectrum_uniform(self.h, int(nbins), _pd(F), _pd(K), _pd(Q), _pi(C)))
        return F, K, Q, C

    def spectrum_timing(self):
        """Device time of the last spectrum call: (transforms ms, binning ms)."""
        t, b = ctypes.c_double(), ctypes.c_double()
        L.check(self.lib.phn_spectrum_timing(self.h, ctypes.byref(t), ctypes.byref(b)))
        return t.value, b.value

    def spectrum_energy(self):
        """The density-contrast spectrum (withEnergyPS 1): (D[bin*Nc + a], counts)."""
        nb, bs = ctypes.c_int(), ctypes.c_double()
        L.check(self.lib.phn_spectrum_bins(self.h, ctypes.byref(nb), ctypes.byref(bs)))
        D = np.zeros(nb.value * self.p.Nc)
        C = np.zeros(nb.value, dtype=np.int32)
        L.check(self.lib.phn_spectrum_energy(self.h, _pd(D), _pi(C), nb.value))
        return D, C

    def full_analysis(self, thres: float, mode: int = L.ISLAND_REFERENCE, z_periodic: bool = False,
                      labels: bool = True, max_out: int = 1 << 20, out=None):
        """phn_islands: (labels or None, records).  `out`, a caller-owned
        C-contiguous float64 array of shape (rows, 10) (page-locked with
        phn_pin_host for a DMA copy), receives the records in place of a new
        array; the result is then a view of its first rows."""
        lab = np.zeros(self.p.N * self.p.N * (self.p.N + 2), dtype=np.int32) if labels else None
        if out is not None:
            if out.dtype != np.float64 or out.ndim != 2 or out.shape[1] != len(L.ISLAND_FIELDS) or \
                    not out.flags["C_CONTIGUOUS"]:
                raise ValueError("out: a C-contiguous float64 array of shape (rows, %d)" % len(L.ISLAND_FIELDS))
            recs, max_out = out, out.shape[0]
        else:
            recs = np.zeros((max_out, len(L.ISLAND_FIELDS)))
        n = ctypes.c_int()
        r = self.lib.phn_islands(self.h, float(thres), int(mode), int(bool(z_periodic)),
                                 _pi(lab) if labels else None, _pd(recs), max_out, ctypes.byref(n))
        L.check(r)
        if out is not None:
            return lab, recs[:n.value]
        return lab, recs if n.value == max_out else recs[:n.value].copy()

    def full_analysis_device(self, thres: float, mode: int = L.ISLAND_REFERENCE, z_periodic: bool = False):
        """phn_islands_device: (number of islands, device address of their
        records); the records live in the handle until its next island call."""
        n, d = ctypes.c_int(), ctypes.c_void_p()
        L.check(self.lib.phn_islands_device(self.h, float(thres), int(mode), int(bool(z_periodic)), ctypes.byref(d),
                                            ctypes.byref(n)))
        return n.value, d.value

    def stats(self):
        n, ms, st = ctypes.c_longlong(), ctypes.c_double(), ctypes.c_int()
        L.check(self.lib.phn_stats(self.h, ctypes.byref(n), ctypes.byref(ms), ctypes.byref(st)))
        return n.value, ms.value, st.value

    def synchronize(self):
        L.check(self.lib.phn_synchronize(self.h))


class Tracker:
    """Island tracking over a run (phn_tracker_*): Full_Analysis with its
    history.  islands(set) returns an (n, 44) array per island: index,
    status, disp, history length, then 5 x (at_time, centre, volume, PotEn,
    KinEn, GradEn, avPhi, Peak_value)."""

    def __init__(self, rank: int = 0):
        self.lib = L.load()
        h = ctypes.c_void_p()
        L.check(self.lib.phn_tracker_create(int(rank), ctypes.byref(h)))
        self.h = h

    def close(self):
        if self.h:
            self.lib.phn_tracker_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def update(self, lat: "Lattice", thres: float, mode: int = L.ISLAND_REFERENCE, z_periodic: bool = False,
               labels: bool = False):
        lab = np.zeros(lat.p.N * lat.p.N * (lat.p.N + 2), dtype=np.int32) if labels else None
        L.check(self.lib.phn_tracker_update(self.h, lat.h, float(thres), int(mode), int(bool(z_periodic)),
                                            _pi(lab) if labels else None))
        return lab

    def update_records(self, tau: float, comps: np.ndarray, center_island: np.ndarray):
        """The bookkeeping alone: comps as phn_islands records (n, 10),
        center_island aligned with centers(); returns each island's owner."""
        comps = np.ascontiguousarray(comps, dtype=np.float64)
        ci = np.ascontiguousarray(center_island, dtype=np.int32)
        owner = np.zeros(max(1, comps.shape[0]), dtype=np.int32)
        L.check(self.lib.phn_tracker_update_records(self.h, float(tau), comps.ctypes.data_as(ctypes.c_void_p),
                                                    comps.shape[0], _pi(ci), _pi(owner)))
        return owner[:comps.shape[0]]

    def centers(self) -> np.ndarray:
        n = ctypes.c_int()
        L.check(self.lib.phn_tracker_count(self.h, L.TRACK_ALIVE, ctypes.byref(n)))
        out = np.zeros(max(1, n.value), dtype=np.int64)
        L.check(self.lib.phn_tracker_centers(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong)),
                                             n.value, ctypes.byref(n)))
        return out[:n.value]

    def islands(self, which: int = L.TRACK_ALIVE) -> np.ndarray:
        n = ctypes.c_int()
        L.check(self.lib.phn_tracker_count(self.h, int(which), ctypes.byref(n)))
        out = np.zeros((n.value, 44))
        rec = L.PhnTrackIsland()
        for i in range(n.value):
            L.check(self.lib.phn_tracker_get(self.h, int(which), i, ctypes.byref(rec)))
            a = np.frombuffer(bytes(rec), dtype=np.float64)
            out[i, :4] = a[:4]
            out[i, 4:] = a[4:].reshape(8, 5).T.ravel()
        return out


class Ensemble:
    """Many lattices evolved together (phn_ensemble_*): one persistent kernel
    per step over all members, step loop in a CUDA graph."""

    def __init__(self, members: list):
        self.members = members
        self.lib = L.load()
        arr = (L.PhnParams * len(members))(*[m.c() for m in members])
        h = ctypes.c_void_p()
        L.check(self.lib.phn_ensemble_create(arr, len(members), ctypes.byref(h)))
        self.h = h

    def close(self):
        if self.h:
            self.lib.phn_ensemble_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, m: int, phi: np.ndarray, pi: np.ndarray):
        phi = np.ascontiguousarray(phi, dtype=np.float64)
        pi = np.ascontiguousarray(pi, dtype=np.float64)
        L.check(self.lib.phn_ensemble_upload(self.h, m, _pd(phi), _pd(pi)))

    def download(self, m: int):
        n = self.members[m].field_len
        phi, pi = np.zeros(n), np.zeros(n)
        L.check(self.lib.phn_ensemble_download(self.h, m, _pd(phi), _pd(pi)))
        return phi, pi

    def reset(self):
        L.check(self.lib.phn_ensemble_reset(self.h))

    def evolve(self, n: int):
        L.check(self.lib.phn_ensemble_evolve(self.h, int(n)))

    def averages(self) -> np.ndarray:
        out = (L.PhnAverages * len(self.members))()
        L.check(self.lib.phn_ensemble_averages(self.h, out))
        return np.frombuffer(bytes(out), dtype=np.float64).reshape(len(self.members), L.AVG_LEN).copy()

    def islands(self, m: int, thres: float, mode: int = L.ISLAND_REFERENCE, z_periodic: bool = False,
                max_out: int = 0):
        n = ctypes.c_int()
        recs = np.zeros((max(max_out, 1), len(L.ISLAND_FIELDS)))
        L.check(self.lib.phn_ensemble_islands(self.h, m, float(thres), int(mode), int(bool(z_periodic)), None,
                                              _pd(recs) if max_out else None, max_out, ctypes.byref(n)))
        return n.value, recs[:min(n.value, max_out)].copy()

    def autotune(self, steps: int = 5):
        t, ms = ctypes.c_int(), ctypes.c_double()
        L.check(self.lib.phn_ensemble_autotune(self.h, steps, ctypes.byref(t), ctypes.byref(ms)))
        return t.value, ms.value

    def set_tile(self, t: int):
        L.check(self.lib.phn_ensemble_set_tile(self.h, t))

    def stats(self):
        n, ms, st = ctypes.c_longlong(), ctypes.c_double(), ctypes.c_int()
        L.check(self.lib.phn_ensemble_stats(self.h, ctypes.byref(n), ctypes.byref(ms), ctypes.byref(st)))
        return n.value, ms.value, st.value


def device_count() -> int:
    lib = L.load()
    n = ctypes.c_int()
    r = lib.phn_device_count(ctypes.byref(n))
    return n.value if r == L.OK else 0


class Adjoint:
    """Forward/backward pair of the hand-written adjoint (phn_adjoint_*).

    `width` is the sigmoid width of the objective in the reference's energy
    units; the default 0.6 is width 0.1 in the units of the
    phi^2/2 - phi^4/4 + g phi^6/6 form (Phi = sqrt(6) phi, energies 6x)."""

    def __init__(self, p: Params, nsteps: int, every: int = 50, width: float = 0.6,
                 forward_precision: int = None):
        self.p = p
        self.lib = L.load()
        h = ctypes.c_void_p()
        L.check(self.lib.phn_adjoint_create(ctypes.byref(p.c()), int(nsteps), int(every), float(width),
                                            ctypes.byref(h)))
        self.h = h
        if forward_precision is not None:
            L.check(self.lib.phn_adjoint_set_forward_precision(self.h, int(forward_precision)))

    def close(self):
        if self.h:
            self.lib.phn_adjoint_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def forward(self, phi: np.ndarray, pi: np.ndarray) -> float:
        phi = np.ascontiguousarray(phi, dtype=np.float64)
        pi = np.ascontiguousarray(pi, dtype=np.float64)
        J = ctypes.c_double()
        L.check(self.lib.phn_adjoint_forward(self.h, _pd(phi), _pd(pi), ctypes.byref(J)))
        return J.value

    def backward(self):
        """Returns (dJ/dPhi0, dJ/dPi0, [dJ/dshift, dJ/dc6, dJ/dh]) in the reference layout."""
        n = self.p.field_len
        dphi, dpi = np.zeros(n), np.zeros(n)
        g = np.zeros(3)
        L.check(self.lib.phn_adjoint_backward(self.h, _pd(dphi), _pd(dpi), _pd(g)))
        return dphi, dpi, g

    def info(self):
        J, f, b = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        L.check(self.lib.phn_adjoint_info(self.h, ctypes.byref(J), ctypes.byref(f), ctypes.byref(b)))
        return J.value, f.value, b.value
