"""Generates the golden fixtures in tests/golden/ from the reference's OWN
sources (oracle/_ref, built by oracle/build_ref.sh from the reference tree).

    sh oracle/build_ref.sh && python tests/golden/make_golden.py
    python tests/golden/make_golden.py --cases e0_n12 n12_exp   # chosen cases only

The initial-condition fixtures (tests/golden/ic/) hold the reference's own
SetInitialConditions output (initialize 3) for chosen srand48 seeds: the
harness redirects its time(NULL) seed (oracle/ref_driver.cpp).

Every case runs in a fresh process because the reference keeps its lattice in
globals.  Inputs come from tests/golden/inputs.py (bit-reproducible on any
platform), so the fixtures store seeds for the large cases and full arrays only
for the small ones.  FP64 fields of the large cases are stored as SHA-256
digests of their little-endian bytes: a bit-exact implementation reproduces
them exactly.
"""
from __future__ import annotations

import hashlib
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

SQRT6 = 6.0 ** 0.5

# Reference parameterisation of the two potentials (field rescaled by sqrt(6)):
#   phi^6:        V = phi^2/2 - phi^4/4 + g phi^6/6, g = 0.1   -> theory 0,
#                 Mmode=1, M=1, Lmode=-1, Kappa = sqrt(0.3/g) = sqrt(3)
#   tilted DW:    V = (phi^2-1)^2/4 + eps phi, eps = 0.05       -> theory 1,
#                 Mmode=-1, M=1, Lmode=1, h = sqrt(6) eps
PHI6 = dict(theory=0, mass_mode=1, lambda_mode=-1, m_sqr=1.0, kappa=3.0 ** 0.5, h=0.0)
TDW = dict(theory=1, mass_mode=-1, lambda_mode=1, m_sqr=1.0, kappa=1.0, h=SQRT6 * 0.05)
# theories 2-5 with the couplings parameters.cpp:122-170 sets
COS = dict(theory=2, mass_mode=1, lambda_mode=1, m_sqr=0.49, kappa=1.0, h=0.0)
MONO = dict(theory=3, mass_mode=1, lambda_mode=1, m_sqr=9.0, kappa=1.0, h=0.0, m_mono_sqr=1.0)
CUBIC = dict(theory=4, mass_mode=1, lambda_mode=1, m_sqr=1.0, kappa=1.0, h=0.0, g=2.0)
POWER = dict(theory=5, mass_mode=1, lambda_mode=1, m_sqr=1.0, kappa=1.0, h=0.0, p_mono=-0.5)
EXP = dict(expansion=1, H0=0.0171156)

CASES = {
    # name: (params, seed, phi0, steps, tso, full arrays?, checkpoints)
    "t0_n8": (dict(N=8, Nc=1, **PHI6), 1, SQRT6, 100, 0.25, True, (1, 10, 100)),
    "t1_n8": (dict(N=8, Nc=1, **TDW), 2, -SQRT6, 100, 0.25, True, (1, 10, 100)),
    "t0_n12": (dict(N=12, Nc=1, **PHI6), 3, SQRT6, 60, 0.3, True, (1, 60)),
    "t0_n16_nc2": (dict(N=16, Nc=2, **PHI6), 4, SQRT6, 50, 0.25, True, (1, 50)),
    "t1_n32": (dict(N=32, Nc=1, **TDW), 5, -SQRT6, 500, 1.0, False, (1, 100, 500)),
    "c0_n64": (dict(N=64, Nc=1, **PHI6), 6, SQRT6, 2000, 1.0, False, (1, 500, 2000)),
    "t2_n8": (dict(N=8, Nc=1, **COS), 7, 1.5, 100, 0.25, True, (1, 10, 100)),
    "t3_n8": (dict(N=8, Nc=1, **MONO), 8, 2.0, 100, 0.25, True, (1, 10, 100)),
    "t4_n8": (dict(N=8, Nc=1, **CUBIC), 9, 1.0, 100, 0.25, True, (1, 10, 100)),
    "t4_n16": (dict(N=16, Nc=1, **CUBIC), 10, 1.0, 300, 0.5, False, (1, 100, 300)),
    "t5_n8": (dict(N=8, Nc=1, **POWER), 11, 2.0, 100, 0.25, True, (1, 10, 100)),
    # three and four field components (O(3) and O(4) models)
    "t0_n8_nc3": (dict(N=8, Nc=3, **PHI6), 38, SQRT6, 100, 0.25, True, (1, 100)),
    "t1_n12_nc4": (dict(N=12, Nc=4, **TDW), 39, -SQRT6, 100, 0.25, True, (1, 100)),
    # theories 2-5 with several components (their forces and averages use the
    # component sums locPhiSqr and, for theory 4, locPhi)
    "t2_n8_nc2": (dict(N=8, Nc=2, **COS), 41, 1.5, 100, 0.25, True, (1, 10, 100)),
    "t3_n8_nc3": (dict(N=8, Nc=3, **MONO), 42, 2.0, 100, 0.25, True, (1, 100)),
    "t4_n8_nc2": (dict(N=8, Nc=2, **CUBIC), 43, 1.0, 100, 0.25, True, (1, 10, 100)),
    "t5_n8_nc4": (dict(N=8, Nc=4, **POWER), 44, 2.0, 100, 0.25, True, (1, 100)),
    "e4_n8_nc2": (dict(N=8, Nc=2, **CUBIC, **EXP), 45, 1.0, 100, 0.25, True, (1, 100)),
    # the radiation-era expanding box (expansion 1) at the reference's H_0
    "e0_n12": (dict(N=12, Nc=1, **PHI6, **EXP), 31, SQRT6, 300, 0.5, True, (1, 100, 300)),
    "e0_n8_nc2": (dict(N=8, Nc=2, **PHI6, **EXP), 32, SQRT6, 100, 0.25, True, (1, 100)),
    "e1_n8": (dict(N=8, Nc=1, **TDW, **EXP), 33, -SQRT6, 200, 0.25, True, (1, 200)),
    "e2_n8": (dict(N=8, Nc=1, **COS, **EXP), 34, 1.5, 100, 0.25, True, (1, 100)),
    "e3_n8": (dict(N=8, Nc=1, **MONO, **EXP), 35, 2.0, 100, 0.25, True, (1, 100)),
    "e4_n16": (dict(N=16, Nc=1, **CUBIC, **EXP, T0=2.0), 36, 1.0, 400, 0.5, False, (1, 100, 400)),
    "e5_n8": (dict(N=8, Nc=1, **POWER, **EXP), 37, 2.0, 100, 0.25, True, (1, 100)),
}


# SetInitialConditions cases: name -> (lattice params, initial-condition params)
IC_CASES = {
    "n8_phi6": (dict(N=8, Nc=1, **PHI6), dict(seed=7, noise=3.0, scale2=6.2832, phi0=(SQRT6, 0.0))),
    "n12_nc2": (dict(N=12, Nc=2, **PHI6), dict(seed=123, noise=0.5, QS=6.0, scale2=10.0, amplitude=1.5,
                                                 phi0=(1.0, -0.5), pi0=(0.2, 0.1))),
    "n16_tdw": (dict(N=16, Nc=1, **TDW), dict(seed=20260, noise=3.0, scale2=6.2832, phi0=(-SQRT6, 0.0))),
    "n16_noise": (dict(N=16, Nc=1, **PHI6), dict(seed=-5, justnoise=1, scale2=0.0, noise=1.0)),
    "n12_exp": (dict(N=12, Nc=1, **PHI6, **EXP), dict(seed=41, noise=0.3, QS=3.0, scale2=5.0, phi0=(1.5, 0.0),
                                                      pi0=(0.1, 0.0))),
    "n16_exp_nc2": (dict(N=16, Nc=2, **PHI6, **EXP, T0=3.0),
                    dict(seed=42, noise=0.5, QS=4.0, scale2=6.0, phi0=(2.0, -0.5), pi0=(0.0, 0.3))),
    # the other `initialize` switches and the charged variant (withcharge 1),
    # from the reference builds oracle/_ref/libphinum_ref_t0_f64_ic*.so
    "n12_ic0": (dict(N=12, Nc=1, **dict(PHI6, m_sqr=0.7)),
                dict(seed=51, initialize=0, famp=0.5, lambda_=1.7, temperature=0.6, phi0s=0.9, pi0s=0.3,
                     variant="_ic0")),
    "n12_ic1_nc2": (dict(N=12, Nc=2, **dict(PHI6, m_sqr=0.7)),
                    dict(seed=52, initialize=1, QS=5.0, amplitude=0.8, noise=0.4, chi=1.3, phi0s=0.9, pi0s=0.3,
                         variant="_ic1")),
    "n12_ic2_nc3": (dict(N=12, Nc=3, **dict(PHI6, m_sqr=0.7)),
                    dict(seed=53, initialize=2, QS=5.0, scale2=7.0, amplitude=0.8, noise=0.4, phi0s=0.9, pi0s=0.3,
                         variant="_ic2")),
    "n12_ic4_nc2": (dict(N=12, Nc=2, **dict(PHI6, m_sqr=0.7)),
                    dict(seed=54, initialize=4, QS=5.0, scale2=7.0, noise=0.4, temperature=0.6, phi0=(1.0, 0.5),
                         pi0=(0.2, -0.1), variant="_ic4")),
    "n12_ic2q_nc2": (dict(N=12, Nc=2, **dict(PHI6, m_sqr=0.7)),
                     dict(seed=55, initialize=2, withcharge=1, QS=5.0, scale2=7.0, amplitude=0.8, noise=0.4,
                          phi0s=0.9, pi0s=0.3, variant="_ic2q")),
    "n16_ic3q_nc2": (dict(N=16, Nc=2, **dict(PHI6, m_sqr=0.7)),
                     dict(seed=56, initialize=3, withcharge=1, QS=5.0, scale2=7.0, amplitude=0.8, noise=0.4,
                          phi0=(1.0, 0.5), pi0=(0.2, -0.1), variant="_ic3q")),
    "n12_ic3q_nc1": (dict(N=12, Nc=1, **dict(PHI6, m_sqr=0.7)),
                     dict(seed=57, initialize=3, withcharge=1, QS=5.0, scale2=7.0, amplitude=0.8, noise=0.4,
                          phi0=(1.0, 0.0), variant="_ic3q")),
}


# Island tracking (Full_Analysis over a run): N, input seed, mask quantile,
# steps, steps between analyses
TRACK_CASES = {"n24_phi6": (dict(N=24, Nc=1, **PHI6), 3, 0.95, 2500, 50)}


def run_track_case(name: str) -> None:
    """The reference's Full_Analysis() every `every` steps from t = 0 (as
    main.cpp:68-83 calls it).  Per call: the tracked islands' integer data
    (index, status, disp, history length, centres, sizes), the labels' digest,
    per-column sums of the float data, and the full float data for the first
    two and the last ten calls."""
    from oracle import oracle as O
    import inputs
    pd, seed, q, steps, every = TRACK_CASES[name]
    p = O.Params(a=0.25, dt=0.08, T0=0.0, **pd)
    phi_i, pi_i = inputs.lattice_fields(p.N, 1, seed, phi0=SQRT6)
    thr = float(np.quantile(np.sqrt(phi_i ** 2 + pi_i ** 2), q))
    R = O.Reference(p)
    R.set_fields(O.to_ref_layout(phi_i), O.to_ref_layout(pi_i))
    R.reset()
    R.track_reset()
    ncalls = steps // every + 1
    ints, offs, sums, lab_sha, full = [], [0], [], [], {}
    cell = p.a ** 3
    labels = np.zeros(p.N * p.N * (p.N + 2), dtype=np.int32)
    for c in range(ncalls):
        n = R.lib.ref_track_step(thr, labels.ctypes.data_as(O._PI))
        T = np.zeros((n, 44))
        for i in range(n):
            R.lib.ref_track_island(i, T[i].ctypes.data_as(O._PD))
        H = T[:, 4:].reshape(n, 5, 8)
        iv = np.zeros((n, 14), dtype=np.int64)
        iv[:, :4] = T[:, :4].astype(np.int64)
        iv[:, 4:9] = H[:, :, 1].astype(np.int64)
        iv[:, 9:14] = np.rint(H[:, :, 2] / cell).astype(np.int64)
        ints.append(iv)
        offs.append(offs[-1] + n)
        sums.append(H[:, :, [0, 3, 4, 5, 6, 7]].sum(axis=(0, 1)))
        lab_sha.append(hashlib.sha256(labels.astype("<i4").tobytes()).hexdigest())
        if c < 2 or c >= ncalls - 10:
            full[f"floats_{c}"] = H[:, :, [0, 3, 4, 5, 6, 7]]
        if c + 1 < ncalls:
            R.evolve(every)
    np.savez_compressed(os.path.join(HERE, "track", f"{name}.npz"), params=json.dumps(pd), seed=seed, thres=thr,
                        every=every, ncalls=ncalls, ints=np.concatenate(ints), offs=np.array(offs),
                        sums=np.array(sums), labels_sha=np.array(lab_sha), **full)
    print(f"track/{name}: calls={ncalls} islands per call max={max(np.diff(offs))} total={offs[-1]}")


# Checkpoint files (SaveConfig): lattice params, input seed, precision build
CONFIG_CASES = {"n8_f64": (dict(N=8, Nc=1, **PHI6), 11, "f64"), "n8_nc2_f64": (dict(N=8, Nc=2, **PHI6), 12, "f64"),
                "n8_f32": (dict(N=8, Nc=1, **PHI6), 13, "f32")}


def run_config_case(name: str) -> None:
    """The reference's SaveConfig(3) on seeded fields, run in a scratch
    directory: SHA-256 of field-3-0.out and the text of moment-3.out."""
    import tempfile
    from oracle import oracle as O
    import inputs
    pd, seed, prec = CONFIG_CASES[name]
    p = O.Params(a=0.25, dt=0.08, T0=0.0, **pd)
    phi_i, pi_i = inputs.lattice_fields(p.N, p.Nc, seed, phi0=SQRT6)
    R = O.Reference(p, prec)
    R.set_fields(O.to_ref_layout(phi_i, p.Nc), O.to_ref_layout(pi_i, p.Nc))
    R.reset()
    R.evolve(3)
    phi, pi = R.get_fields()
    with tempfile.TemporaryDirectory() as tmp:
        cwd = os.getcwd()
        os.chdir(tmp)
        try:
            R.save_config(3)
            raw = open("field-3-0.out", "rb").read()
            moment = open("moment-3.out").read()
        finally:
            os.chdir(cwd)
    out = os.path.join(HERE, "config")
    os.makedirs(out, exist_ok=True)
    np.savez_compressed(os.path.join(out, f"{name}.npz"), params=json.dumps(pd), prec=prec, phi=phi, pi=pi,
                        sha=hashlib.sha256(raw).hexdigest(), nbytes=len(raw), moment=moment)
    print(f"config/{name}: {len(raw)} bytes, moment {moment.strip()}")


# Momentum-space filter: lattice params, input seed, r_filter, which
FILTER_CASES = {"n8_tophat": (dict(N=8, Nc=1, **PHI6), 21, 0.6, 0), "n8_gauss": (dict(N=8, Nc=1, **PHI6), 22, 0.6, 1),
                "n12_table": (dict(N=12, Nc=1, **PHI6), 23, 0.6, 2),
                "n12_nc2_ktophat": (dict(N=12, Nc=2, **PHI6), 24, 0.6, 3),
                "n16_tophat": (dict(N=16, Nc=1, **TDW), 25, 0.9, 0)}
FILTER_TABLE_DP = 0.01


def filter_table() -> np.ndarray:
    """The tabulated window of the which = 2 case (25000 entries, spacing 0.01)."""
    return np.exp(-np.arange(25000) * 0.001) * (1.0 + 0.1 * np.cos(np.arange(25000) * 0.01))


def run_filter_case(name: str) -> None:
    """The reference's apply_filter on seeded fields."""
    from oracle import oracle as O
    import inputs
    pd, seed, r, which = FILTER_CASES[name]
    p = O.Params(a=0.25, dt=0.08, T0=0.0, **pd)
    phi_i, pi_i = inputs.lattice_fields(p.N, p.Nc, seed, phi0=SQRT6)
    R = O.Reference(p)
    R.set_fields(O.to_ref_layout(phi_i, p.Nc), O.to_ref_layout(pi_i, p.Nc))
    phi, pi = R.apply_filter(r, which, filter_table(), FILTER_TABLE_DP)
    os.makedirs(os.path.join(HERE, "filter"), exist_ok=True)
    np.savez_compressed(os.path.join(HERE, "filter", f"{name}.npz"), params=json.dumps(pd), seed=seed, r=r,
                        which=which, dp=FILTER_TABLE_DP, phi=phi, pi=pi)
    print(f"filter/{name}")


# The false-vacuum break of main.cpp:85-89: lattice params, input seed, phi0,
# steps, TSO, a site of Pi set to NaN (-1: none).  The tilted well with a
# strong tilt rolls from phi0 = 0.8 towards negative phi, and <V> turns
# negative mid-run; a NaN in Pi reaches phi with the first drift, so the
# reference stops at its second row.
FVD_CASES = {
    "fvd_t1_n16": (dict(N=16, Nc=1, theory=1, mass_mode=-1, lambda_mode=1, m_sqr=1.0, kappa=1.0, h=0.6),
                   51, 0.8, 400, 0.2, -1),
    "fvd_t0_n16_nan": (dict(N=16, Nc=1, **PHI6), 52, SQRT6, 100, 0.2, 16 * 16 * 5 + 16 * 3 + 7),
}


def run_fvd_case(name: str) -> None:
    """The reference's run loop with its false_vacuum_decayed() break: the
    rows it printed and the step count at the break."""
    from oracle import oracle as O
    import inputs
    pd, seed, phi0, steps, tso, nan_site = FVD_CASES[name]
    p = O.Params(**{"a": 0.25, "dt": 0.08, "T0": 0.0, **pd})
    phi_i, pi_i = inputs.lattice_fields(p.N, p.Nc, seed, phi0=phi0)
    Phi, Pi = O.to_ref_layout(phi_i, p.Nc), O.to_ref_layout(pi_i, p.Nc)
    if nan_site >= 0:
        Pi[nan_site] = np.nan
    R = O.Reference(p)
    R.set_fields(Phi, Pi)
    rows, stop = R.run_until_decayed(steps, tso)
    os.makedirs(os.path.join(HERE, "fvd"), exist_ok=True)
    np.savez_compressed(os.path.join(HERE, "fvd", f"{name}.npz"), params=json.dumps(pd), seed=seed, phi0=phi0,
                        steps=steps, tso=tso, nan_site=nan_site, rows=rows, stop=stop)
    print(f"fvd/{name}: rows={len(rows)} stop={stop}")


# The reference's single-precision build (doubleprecision -1): lattice
# params, input seed, phi0, steps.  Float fields after the steps.
F32_CASES = {
    "f32_t0_n12_nc2": (dict(N=12, Nc=2, **PHI6), 61, SQRT6, 100),
    "f32_t1_n12": (dict(N=12, Nc=1, **TDW), 62, -SQRT6, 100),
}


def run_f32_case(name: str) -> None:
    from oracle import oracle as O
    import inputs
    pd, seed, phi0, steps = F32_CASES[name]
    p = O.Params(**{"a": 0.25, "dt": 0.08, "T0": 0.0, **pd})
    phi_i, pi_i = inputs.lattice_fields(p.N, p.Nc, seed, phi0=phi0)
    R = O.Reference(p, "f32")
    R.set_fields(O.to_ref_layout(phi_i, p.Nc), O.to_ref_layout(pi_i, p.Nc))
    R.reset()
    R.evolve(steps)
    phi, pi = R.get_fields()
    tau, n = R.time()
    os.makedirs(os.path.join(HERE, "f32"), exist_ok=True)
    np.savez_compressed(os.path.join(HERE, "f32", f"{name}.npz"), params=json.dumps(pd), seed=seed, phi0=phi0,
                        steps=steps, phi=phi.astype(np.float32), pi=pi.astype(np.float32), tau=tau)
    print(f"f32/{name}: tau={tau}")


# The energy-density analysis (withEnergyPS 1, EnergybasedID 1) of the
# reference builds that compile it: lattice params, input seed, phi0, steps
# before the analysis.  Delta, the island labels and records of a first
# Full_Analysis (threshold 4 <rho>, set by the reference itself) and the
# density-contrast spectrum.
EPS_CASES = {
    "eps_t2_n12": (dict(N=12, Nc=1, **COS), 71, 1.0, 40),
    "eps_t3_n12": (dict(N=12, Nc=1, **MONO), 72, 0.0, 40),
    "eps_t4_n12": (dict(N=12, Nc=1, **CUBIC), 73, 0.5, 40),
    "eps_t5_n12": (dict(N=12, Nc=1, **POWER), 74, 1.0, 40),
    "eps_t3_n12_exp": (dict(N=12, Nc=1, **MONO, **EXP), 75, 0.0, 40),
}


def run_eps_case(name: str) -> None:
    from oracle import oracle as O
    import inputs
    pd, seed, phi0, steps = EPS_CASES[name]
    p = O.Params(**{"a": 0.25, "dt": 0.08, "T0": 0.0, **pd})
    phi_i, pi_i = inputs.lattice_fields(p.N, p.Nc, seed, phi0=phi0)
    R = O.Reference(p, "f64", "_eps")
    R.set_fields(O.to_ref_layout(phi_i, p.Nc), O.to_ref_layout(pi_i, p.Nc))
    R.reset()
    R.evolve(steps)
    phi, pi = R.get_fields()
    delta = R.delta()
    labels, stats = R.islands(0.0)  # Full_Analysis replaces the threshold by 4 <rho>
    thres = R.island_thres()
    D, C = R.spectrum_energy()
    os.makedirs(os.path.join(HERE, "eps"), exist_ok=True)
    np.savez_compressed(os.path.join(HERE, "eps", f"{name}.npz"), params=json.dumps(pd), seed=seed, phi0=phi0,
                        steps=steps, phi=phi, pi=pi, delta=delta, labels=labels, stats=stats, thres=thres, D=D,
                        counts=C)
    print(f"eps/{name}: thres={thres:.6g} islands={len(stats)} D[1]={D[1]:.6g}")


def run_ic_case(name: str) -> None:
    from oracle import oracle as O
    pd, ic = IC_CASES[name]
    ic = dict(ic)
    variant = ic.pop("variant", "")
    p = O.Params(**{"a": 0.25, "dt": 0.08, "T0": 0.0, **pd})
    R = O.Reference(p, "f64", variant)
    phi, pi = R.initial_conditions(**ic)
    os.makedirs(os.path.join(HERE, "ic"), exist_ok=True)
    np.savez_compressed(os.path.join(HERE, "ic", f"{name}.npz"), params=json.dumps(pd), ic=json.dumps(ic),
                        phi=phi, pi=pi)
    print(f"ic/{name}: |phi|max={np.abs(phi).max():.4g} |pi|max={np.abs(pi).max():.4g}")


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()


def island_threshold(phi, pi) -> float:
    """A threshold that puts about 12% of sites in the reference mask."""
    r = np.sqrt(phi[0] ** 2 + pi[0] ** 2)
    return float(np.quantile(r, 0.88))


def run_case(name: str) -> None:
    from oracle import oracle as O
    import inputs
    pd, seed, phi0, steps, tso, full, checkpoints = CASES[name]
    p = O.Params(**{"a": 0.25, "dt": 0.08, "T0": 0.0, **pd})
    phi_i, pi_i = inputs.lattice_fields(p.N, p.Nc, seed, phi0=phi0)
    R = O.Reference(p)
    out = {"params": json.dumps(pd), "seed": seed, "phi0": phi0, "steps": steps, "tso": tso,
           "a": p.a, "dt": p.dt}
    if full:
        out["phi_init"], out["pi_init"] = phi_i, pi_i
    # SO rows over the whole run (main.cpp:685-699 cadence)
    R.set_fields(O.to_ref_layout(phi_i, p.Nc), O.to_ref_layout(pi_i, p.Nc))
    out["rows"] = R.run_loop(steps, tso)
    # fields at the checkpoints (fresh start, explicit evolve counts)
    R.set_fields(O.to_ref_layout(phi_i, p.Nc), O.to_ref_layout(pi_i, p.Nc))
    R.reset()
    done = 0
    for c in checkpoints:
        R.evolve(c - done)
        done = c
        ph, pp = R.get_fields()
        phi_c, pi_c = O.from_ref_layout(ph, p.N, p.Nc), O.from_ref_layout(pp, p.N, p.Nc)
        out[f"phi_sha_{c}"] = digest(phi_c)
        out[f"pi_sha_{c}"] = digest(pi_c)
        out[f"avg_{c}"] = R.averages()
        if full:
            out[f"phi_{c}"], out[f"pi_{c}"] = phi_c, pi_c
    out["tau_end"], out["steps_end"] = R.time()
    # spectrum and islands on the final state
    F, K, Q, C = R.spectrum()
    out["spec_F"], out["spec_K"], out["spec_Q"], out["spec_counts"] = F, K, Q, C
    if p.Nc == 1:
        thr = island_threshold(phi_c, pi_c)
        labels, stats = R.islands(thr)
        lab = O.from_ref_layout(labels.astype(np.float64), p.N, 1)[0].astype(np.int32)
        out["island_thres"] = thr
        out["island_stats"] = stats
        out["island_labels_sha"] = hashlib.sha256(lab.astype("<i4").tobytes()).hexdigest()
        if full:
            out["island_labels"] = lab
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
    print(f"{name}: rows={len(out['rows'])} islands={len(out.get('island_stats', []))}")


def main() -> None:
    from oracle import oracle as O
    if len(sys.argv) > 2 and sys.argv[1] == "--case":
        run_case(sys.argv[2])
        return
    if len(sys.argv) > 2 and sys.argv[1] == "--ic-case":
        run_ic_case(sys.argv[2])
        return
    if len(sys.argv) > 2 and sys.argv[1] == "--track-case":
        os.makedirs(os.path.join(HERE, "track"), exist_ok=True)
        run_track_case(sys.argv[2])
        return
    if len(sys.argv) > 1 and sys.argv[1] == "--track":
        for name in TRACK_CASES:
            subprocess.run([sys.executable, os.path.abspath(__file__), "--track-case", name], check=True)
        return
    if len(sys.argv) > 2 and sys.argv[1] == "--filter-case":
        run_filter_case(sys.argv[2])
        return
    if len(sys.argv) > 1 and sys.argv[1] == "--filter":
        for name in FILTER_CASES:
            subprocess.run([sys.executable, os.path.abspath(__file__), "--filter-case", name], check=True)
        return
    if len(sys.argv) > 2 and sys.argv[1] == "--config-case":
        run_config_case(sys.argv[2])
        return
    if len(sys.argv) > 1 and sys.argv[1] == "--config":
        for name in CONFIG_CASES:
            subprocess.run([sys.executable, os.path.abspath(__file__), "--config-case", name], check=True)
        return
    if len(sys.argv) > 2 and sys.argv[1] == "--eps-case":
        run_eps_case(sys.argv[2])
        return
    if len(sys.argv) > 1 and sys.argv[1] == "--eps":
        for name in EPS_CASES:
            subprocess.run([sys.executable, os.path.abspath(__file__), "--eps-case", name], check=True)
        return
    if len(sys.argv) > 2 and sys.argv[1] == "--f32-case":
        run_f32_case(sys.argv[2])
        return
    if len(sys.argv) > 1 and sys.argv[1] == "--f32":
        for name in F32_CASES:
            subprocess.run([sys.executable, os.path.abspath(__file__), "--f32-case", name], check=True)
        return
    if len(sys.argv) > 2 and sys.argv[1] == "--fvd-case":
        run_fvd_case(sys.argv[2])
        return
    if len(sys.argv) > 1 and sys.argv[1] == "--fvd":
        for name in FVD_CASES:
            subprocess.run([sys.executable, os.path.abspath(__file__), "--fvd-case", name], check=True)
        return
    if len(sys.argv) > 1 and sys.argv[1] == "--ic":
        for name in IC_CASES:
            subprocess.run([sys.executable, os.path.abspath(__file__), "--ic-case", name], check=True)
        return
    if not O.ref_available(0) or not O.ref_available(1):
        sys.exit("reference pin not built: run oracle/build_ref.sh first")
    only = sys.argv[2:] if len(sys.argv) > 2 and sys.argv[1] == "--cases" else None
    if only:
        for name in only:
            flag = "--ic-case" if name in IC_CASES else "--case"
            subprocess.run([sys.executable, os.path.abspath(__file__), flag, name], check=True)
        return
    for name in CASES:
        subprocess.run([sys.executable, os.path.abspath(__file__), "--case", name], check=True)
    for name in IC_CASES:
        subprocess.run([sys.executable, os.path.abspath(__file__), "--ic-case", name], check=True)
    for name in TRACK_CASES:
        subprocess.run([sys.executable, os.path.abspath(__file__), "--track-case", name], check=True)
    for name in CONFIG_CASES:
        subprocess.run([sys.executable, os.path.abspath(__file__), "--config-case", name], check=True)
    for name in FILTER_CASES:
        subprocess.run([sys.executable, os.path.abspath(__file__), "--filter-case", name], check=True)
    for name in FVD_CASES:
        subprocess.run([sys.executable, os.path.abspath(__file__), "--fvd-case", name], check=True)
    for name in F32_CASES:
        subprocess.run([sys.executable, os.path.abspath(__file__), "--f32-case", name], check=True)
    for name in EPS_CASES:
        subprocess.run([sys.executable, os.path.abspath(__file__), "--eps-case", name], check=True)


if __name__ == "__main__":
    main()
