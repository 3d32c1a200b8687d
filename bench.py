"""Benchmark of the lattice hot path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (one "step" = one leapfrog step over the whole lattice): the phi^6
oscillon potential (reference theory 0, Kappa = sqrt(3)) on a 512^3 periodic
lattice, a = 0.25, dtau = 0.02, FP32 fields, with the volume averages and
extrema fused into every 50th step (TSO = 1.0).  Inputs are seeded synthetic
Gaussian fields with the configuration's spectrum (phinum_gb300/initial.py:
phi0 = sqrt(6), vacuum amplitude per mode, modes above pi/(2 dx) zeroed);
1.5 GB of fields, far above the 129 MB L2, so no flush is needed between steps.

value     site-updates/s over K steps, fields resident in HBM, device time
          (CUDA events on the handle's stream), max over ranks x ranks.
e2e       the same metric through the C ABI with host buffers: each e2e
          iteration uploads phi, pi (reference layout, pinned float arrays as
          the reference's single-precision build holds them; e2e.f64_host:
          double arrays, its default build), runs one TSO interval (50 steps +
          one SO row) and downloads phi, pi.
roofline  the autotuned step kernel: 16 algorithmic bytes per site (read phi,
          pi; write pi, phi') over its mean launch time, against the measured
          HBM copy bandwidth in MEASURED_PEAKS.json; traffic from the kernel's
          ncu summary when that summary covers the same sources and variant.
clocks    SM clock and clock-event reasons: nvidia-smi every 200 ms and NVML
          every millisecond during the timed region.
cpu_baseline / --impl reference
          the reference loop restated in C (the oracle), compiled with the
          reference's -O3 -ffast-math flags, OpenMP over z-slabs, all host
          threads, a bounded number of steps of the same lattice: the float
          build (doubleprecision -1, pinned bit-identical to the reference's
          own float build) like for like with this FP32 line, and the double
          build (cpu_baseline_fp64) for the FP64 GPU line; like_for_like holds
          both ratios.
Multi-GPU: replicas only -- every rank evolves its own lattice; no collective
on the data path.

--form precision|adjoint|ensemble|initial|io|analysis|c1 prints one JSON
object for the compensated-FP32 run, the adjoint, the ensemble, the initial
conditions, the checkpoint files, the spectrum/island passes or the 256^3
drop-in configuration (both potentials, three precisions and the host
oracle) instead of the benchmark line.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))

METRIC = "site-updates/s"
N_MAIN = 512
TSO_STEPS = 50
BYTES_PER_SITE = {0: 32, 1: 16, 2: 32}  # FP64, FP32, compensated FP32


def env_rank():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)), int(os.environ.get("WORLD_SIZE", 1))


class Dist:
    """Barrier and max-reduce across ranks (gloo on CPU tensors); trivial at N=1."""

    def __init__(self):
        self.rank, self.local, self.world = env_rank()
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.world > 1:
            self.dist.barrier()

    def max(self, v: float) -> float:
        if self.world == 1:
            return v
        import torch
        t = torch.tensor([v], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.dist.destroy_process_group()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx, self.samples, self.proc = gpu_index, [], None
        self.nvml = NvmlPoller(gpu_index)

    def __enter__(self):
        self.nvml.start()
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                self.samples.append(parts)

    def __exit__(self, *exc):
        self.nvml.stop()
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        reasons = {names[j] for s in self.samples for j in range(4) if s[5 + j].lower() == "active"}
        # NVML polled every millisecond inside the timed region (nvidia-smi's
        # 200 ms period misses regions of a few milliseconds)
        sm += [float(m) for m, _ in self.nvml.samples]
        reasons |= {n for _, bits in self.nvml.samples for n, b in NvmlPoller.REASONS.items() if bits & b}
        if self.nvml.max_mhz:
            mx.append(float(self.nvml.max_mhz))
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.samples), "samples_nvml": len(self.nvml.samples)}


class NvmlPoller:
    """SM clock and clock-event reasons read through NVML (libnvidia-ml, the
    driver's library) every millisecond on a thread while the timed work runs
    in ctypes calls, which release the GIL.  Reads only; no setting changes."""

    REASONS = {"sw_power_cap": 0x4, "hw_slowdown": 0x8, "sw_thermal_slowdown": 0x20,
               "hw_thermal_slowdown": 0x40}

    def __init__(self, index: int):
        import ctypes
        self.samples, self.max_mhz, self.h, self.lib = [], None, None, None
        self._stop = threading.Event()
        try:
            lib = ctypes.CDLL("libnvidia-ml.so.1")
            if lib.nvmlInit_v2() != 0:
                return
            h = ctypes.c_void_p()
            if lib.nvmlDeviceGetHandleByIndex_v2(int(index), ctypes.byref(h)) != 0:
                return
            self.reasons_fn = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
                lib.nvmlDeviceGetCurrentClocksThrottleReasons
            mhz = ctypes.c_uint()
            if lib.nvmlDeviceGetMaxClockInfo(h, 1, ctypes.byref(mhz)) == 0:  # NVML_CLOCK_SM
                self.max_mhz = mhz.value
            self.lib, self.h = lib, h
        except (OSError, AttributeError):
            self.lib = None

    def _run(self):
        import ctypes
        mhz, bits = ctypes.c_uint(), ctypes.c_ulonglong()
        while not self._stop.is_set():
            if self.lib.nvmlDeviceGetClockInfo(self.h, 1, ctypes.byref(mhz)) == 0 and \
                    self.reasons_fn(self.h, ctypes.byref(bits)) == 0:
                self.samples.append((mhz.value, bits.value))
            time.sleep(0.001)

    def start(self):
        if self.lib is not None:
            self._stop.clear()
            self.t = threading.Thread(target=self._run, daemon=True)
            self.t.start()

    def stop(self):
        if self.lib is not None:
            self._stop.set()
            self.t.join(timeout=5)


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ncu summaries of the FP32 step kernels at 512^3 (PHN_PATH_TMA, PHN_PATH_X4)
# and the sources each kernel is compiled from
PROFILE_OF_PATH = {2: ("leapfrog_f32_512.md", ("leapfrog_tma.cu", "tma.cuh", "kick.cuh")),
                   3: ("leapfrog_f32_x4_512.md", ("leapfrog_x4.cu", "kick.cuh"))}


def source_digest(files) -> str:
    """SHA-256 (first 16 hex digits) of the kernel's source files, in order."""
    import hashlib
    h = hashlib.sha256()
    for f in files:
        with open(os.path.join(ROOT, "phinum_gb300", "csrc", f), "rb") as fh:
            h.update(fh.read())
    return h.hexdigest()[:16]


def traffic_from_profile(path_kind: int, variant: int):
    """DRAM bytes per launch (ncu dram__bytes_read.sum + dram__bytes_write.sum)
    of the FP32 step kernel at 512^3 from its committed ncu summary, which
    records the traffic, the variant captured and the digest of the sources it
    was compiled from.  ncu cannot run inside a timed benchmark, so the figure
    is used only when the summary covers this variant and these exact sources;
    otherwise (None, why)."""
    if path_kind not in PROFILE_OF_PATH:
        return None, "no ncu summary for this kernel"
    name, files = PROFILE_OF_PATH[path_kind]
    path = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(path):
        return None, f"profiles/{name} missing"
    digest, per_variant = None, {}
    for line in open(path):
        key, _, val = line.partition(":")
        key, val = key.strip(), val.split()
        if key == "source_sha256_16" and val:
            digest = val[0]
        elif key == "variant_traffic_bytes_per_launch" and len(val) >= 2:
            per_variant[val[0]] = val[1]  # "<variant> <bytes>"
    if digest != source_digest(files):
        return None, f"profiles/{name} was captured on other sources (stale)"
    if str(variant) not in per_variant:
        return None, f"profiles/{name} covers variants {sorted(per_variant)}, this run uses {variant}"
    try:
        return float(per_variant[str(variant)]), f"profiles/{name} (ncu, same sources and variant)"
    except ValueError:
        return None, f"profiles/{name} has no traffic line for variant {variant}"


_FIELDS = {}


def make_fields(N: int, seed: int = 2026):
    """Seeded Gaussian fields with the configuration's spectrum (vacuum
    amplitude 1/(2 omega L^3) per mode in the config's units, x6 in the
    reference's, modes above k_max = pi/(2 dx) zeroed), in the reference layout."""
    if N not in _FIELDS:
        from phinum_gb300 import initial, layout
        phi, pi = initial.gaussian_fields(N, a=0.25, phi0=6.0 ** 0.5, noise=3.0, scale2=2 * np.pi, seed=seed)
        _FIELDS[N] = (layout.to_ref_layout(phi), layout.to_ref_layout(pi))
    return _FIELDS[N]


def measure_gpu(args, dist: Dist):
    from phinum_gb300 import lattice as PL
    from phinum_gb300 import _lib as L

    N = args.n
    phi, pi = make_fields(N)
    lib = L.load()
    sites = N ** 3
    out = {}

    # ---------------------------------------------------------------- value
    lat = PL.Lattice(PL.Params(N=N, precision=L.FP32))
    lat.upload(phi, pi)
    # the project's autotuner picks the FP32 step kernel for this lattice: the
    # plain kernel or a variant of the TMA or x4 kernels (state unchanged; all
    # compute identical fields)
    import ctypes
    tv, tms, pk = ctypes.c_int(), ctypes.c_double(), ctypes.c_int()
    if args.variant is None:
        L.check(lib.phn_autotune(lat.h, 30, ctypes.byref(tv), ctypes.byref(tms)))
    else:
        L.check(lib.phn_set_variant(lat.h, args.variant))
        tv.value = args.variant
    L.check(lib.phn_get_path(lat.h, ctypes.byref(pk)))
    out["variant"] = tv.value
    kernel_name = {L.PATH_PLAIN: "phn::step_f32", L.PATH_TMA: f"phn::step_f32_tma (variant {tv.value})",
                   L.PATH_X4: f"phn::step_f32_x4 (variant {tv.value})"}[pk.value]
    lat.run_loop(max(3, args.warmup), 1.0)
    lat.synchronize()
    n0, _, _ = lat.stats()
    dist.barrier()
    lat.synchronize()
    with ClockSampler(dist.local) as cs:
        t0 = time.perf_counter()
        rows = lat.run_loop(args.steps, 1.0, max_rows=args.steps // TSO_STEPS + 2)
        lat.synchronize()
        wall = time.perf_counter() - t0
    dist.barrier()
    n1, ms, nsteps = lat.stats()
    dev_s = dist.max(ms / 1e3)
    out["value"] = sites * args.steps * dist.world / dev_s
    out["ms_per_step"] = dev_s * 1e3 / args.steps
    out["wall_s"] = wall
    out["rows"] = int(rows.shape[0])
    out["gpu_launches"] = int(n1 - n0)
    out["clocks"] = cs.summary()
    out["energy_drift"] = float(abs(rows[-1, 14] - rows[0, 14]) / abs(rows[0, 14])) if rows.shape[0] > 1 else None

    # ------------------------------------------------- roofline: plain step
    lat.evolve(20)
    k_plain = max(50, min(400, args.steps))
    lat.evolve(k_plain)
    _, ms_plain, _ = lat.stats()
    t_launch = ms_plain / 1e3 / k_plain
    # an observed step: every step of the loop is due a row (TSO = dtau), so
    # each costs the fused step with the averages, the fold and the row's read
    k_obs = 50
    lat.run_loop(k_obs, 0.02, max_rows=k_obs + 2)
    _, ms_obs, _ = lat.stats()
    out["observed_step"] = {"ms": ms_obs / k_obs, "plain_ms": t_launch * 1e3,
                            "ratio": (ms_obs / k_obs) / (t_launch * 1e3),
                            "what": "run loop with a row due every step (fused averages + fold + row read) "
                                    "against the plain step, same kernel variant"}
    achieved = BYTES_PER_SITE[1] * sites / t_launch / 1e9
    peak, kind = peaks()
    traffic, traffic_src = traffic_from_profile(pk.value, tv.value) if N == 512 else (None, "not 512^3")
    out["roofline"] = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                       "frac": round(achieved / peak, 4),
                       "traffic": traffic, "traffic_source": traffic_src,
                       "kernel": kernel_name, "peak_kind": f"{kind} hbm_gbs",
                       "algorithmic_bytes_per_launch": BYTES_PER_SITE[1] * sites,
                       "mean_launch_ms": round(t_launch * 1e3, 4)}
    lat.close()

    if args.no_e2e:
        out["e2e"] = None
        out["also"] = {}
        return out

    # ---------------------------------------------------------------- e2e
    elat = PL.Lattice(PL.Params(N=N, precision=L.FP32))
    # the kernel the autotuner chose above
    L.check(lib.phn_set_path(elat.h, L.PATH_PLAIN) if tv.value < 0 else lib.phn_set_variant(elat.h, tv.value))

    def e2e_leg(host_dtype, upload, download, n=9):
        """Per iteration: upload phi, pi from pinned host arrays in the
        reference layout, one TSO interval (50 steps + one fused SO row, the
        row read back), download phi, pi.  The host fields are fresh arrays
        (the same values) pinned just before the iterations, as a caller
        prepares them; one warm-up iteration, then n timed back to back."""
        hphi, hpi = phi.astype(host_dtype), pi.astype(host_dtype)
        ophi, opi = np.empty_like(hphi), np.empty_like(hpi)
        for a in (hphi, hpi, ophi, opi):
            L.check(lib.phn_pin_host(a.ctypes.data, a.nbytes))
        its, phases = [], []
        try:
            for it in range(n + 1):
                dist.barrier()
                t0 = time.perf_counter()
                L.check(upload(elat.h, hphi.ctypes.data, hpi.ctypes.data))
                t1 = time.perf_counter()
                elat.run_loop(TSO_STEPS, 1.0, max_rows=2)
                t2 = time.perf_counter()
                L.check(download(elat.h, ophi.ctypes.data, opi.ctypes.data))
                t3 = time.perf_counter()
                if it:
                    its.append(t3 - t0)
                    phases.append((t1 - t0, t2 - t1, t3 - t2))
        finally:
            for a in (hphi, hpi, ophi, opi):
                lib.phn_unpin_host(a.ctypes.data)
        med = dist.max(float(np.median(its)))
        return {"value": sites * TSO_STEPS * dist.world / med, "unit": METRIC,
                "h2d_bytes_per_step": int(hphi.nbytes + hpi.nbytes),
                "d2h_bytes_per_step": int(ophi.nbytes + opi.nbytes + 26 * 8),
                "iteration_s": {"median": float(np.median(its)), "min": float(min(its)), "max": float(max(its)),
                                "n": len(its), "all": [round(t, 4) for t in its],
                                "upload_steps_download": [[round(x, 4) for x in ph] for ph in phases]}}

    # the reference's single-precision build (doubleprecision -1) keeps float
    # host arrays: phn_upload_f32 / phn_download_f32, like for like with the
    # FP32 device arithmetic and the FP32 CPU baseline
    e2e = e2e_leg(np.float32, lib.phn_upload_f32, lib.phn_download_f32)
    e2e["step"] = (f"upload phi,pi (float host arrays, reference layout: the doubleprecision -1 build) + "
                   f"{TSO_STEPS} leapfrog steps with one fused SO row + download phi,pi")
    # its default double build: FP64 host arrays, converted on the device
    f64 = e2e_leg(np.float64, lambda h, a, b: lib.phn_upload(h, ctypes.cast(a, L._PD), ctypes.cast(b, L._PD)),
                  lambda h, a, b: lib.phn_download(h, ctypes.cast(a, L._PD), ctypes.cast(b, L._PD)))
    f64["step"] = "as e2e with FP64 host arrays (the reference's default doubleprecision 0 build)"
    e2e["f64_host"] = f64
    out["e2e"] = e2e
    elat.close()

    # ------------------------------------------- the other precisions/sizes
    also = {}
    if args.no_extra:
        out["also"] = also
        return out
    for label, n, prec, k in (("n256_fp32", 256, L.FP32, 400), ("n256_fp64", 256, L.FP64, 40),
                              ("n512_fp64", 512, L.FP64, 10), ("n512_kahan_fp32", 512, L.FP32_KAHAN, 200)):
        if args.quick and n == 512 and prec != L.FP32:
            continue
        ph, pp = (phi, pi) if n == N else make_fields(n)
        lat = PL.Lattice(PL.Params(N=n, precision=prec))
        lat.upload(ph, pp)
        kernel = tune(lib, lat)
        lat.evolve(3)
        lat.evolve(k)
        _, ms_k, _ = lat.stats()
        t = ms_k / 1e3 / k
        also[label] = {"site_updates_per_s": n ** 3 / t, "ms_per_step": t * 1e3, "kernel": kernel,
                       "hbm_gbs_algorithmic": BYTES_PER_SITE[prec] * n ** 3 / t / 1e9,
                       "frac_of_measured_hbm": BYTES_PER_SITE[prec] * n ** 3 / t / 1e9 / peak}
        lat.close()
    if not args.quick:
        also["ensemble_c3"] = measure_ensemble(2000, 100)
        also["analysis"] = analysis_form(N, precisions=("fp32",))["fp32"]
        adj = adjoint_form(128, 1000, reps_unchecked=3, light=True)
        also["adjoint_c4_fp32"] = {k: adj[k] for k in ("cost_ratio", "forward_plain_ms", "adjoint_forward_ms",
                                                       "adjoint_backward_ms", "timing", "fp32_vs_fp64_field_rel_l2")}
        also["adjoint_c4_fp32_pair_forward"] = adj["fp32_pair"]
        # the form held to "at most 3x a forward solve at a gradient error
        # below 1e-4" (both figures from the same solve)
        pf = adj["fp32_pair"]
        also["adjoint_c4_target"] = {
            "form": "FP32 reverse sweep, forward in FP32 pairs", "cost_ratio": pf["cost_ratio"],
            "field_gradient_rel_l2_vs_fp64": pf["vs_fp64_field_rel_l2"],
            "met": bool(pf["cost_ratio"] <= 3.0 and pf["vs_fp64_field_rel_l2"] < 1e-4)}
    out["also"] = also
    return out


def tune(lib, lat, steps: int = 20) -> str:
    """The project's autotuner on a live lattice (state unchanged; every
    kernel of a precision computes the same bits); returns the kernel's name."""
    import ctypes
    from phinum_gb300 import _lib as L
    v, ms, pk = ctypes.c_int(), ctypes.c_double(), ctypes.c_int()
    L.check(lib.phn_autotune(lat.h, steps, ctypes.byref(v), ctypes.byref(ms)))
    L.check(lib.phn_get_path(lat.h, ctypes.byref(pk)))
    return {L.PATH_PLAIN: "plain", L.PATH_TMA: f"tma variant {v.value}", L.PATH_X4: f"x4 variant {v.value}"}[pk.value]


def measure_ensemble(steps: int, steps_per_lattice: int):
    """Batched form: 256 realizations, 128 x 32^3 + 96 x 64^3 + 32 x 128^3,
    phi0 ~ U[0.8, 1.2] and g ~ U[0.05, 0.2] (config units; x sqrt(6) and
    Kappa = sqrt(0.3/g) in the reference's), FP32, one persistent kernel per
    step in CUDA-graph chunks, autotuned tile; against one handle per lattice
    (one launch per lattice per step)."""
    import ctypes
    from phinum_gb300 import initial, layout
    from phinum_gb300 import lattice as PL
    rng = np.random.default_rng(2026)
    sizes = [32] * 128 + [64] * 96 + [128] * 32
    params, fields = [], []
    for i, N in enumerate(sizes):
        phi0 = rng.uniform(0.8, 1.2) * 6 ** 0.5
        g = rng.uniform(0.05, 0.2)
        params.append(PL.Params(N=N, precision=1, theory=0, kappa=(0.3 / g) ** 0.5))
        phi, pi = initial.gaussian_fields(N, phi0=phi0, seed=i)
        fields.append((layout.to_ref_layout(phi), layout.to_ref_layout(pi)))
    sites = sum(N ** 3 for N in sizes)
    ens = PL.Ensemble(params)
    for m, (phi, pi) in enumerate(fields):
        ens.upload(m, phi, pi)
    tile, _ = ens.autotune(5)
    ens.evolve(50)
    n0, _, _ = ens.stats()
    ens.evolve(steps)
    n1, ms, _ = ens.stats()
    ens_rate = sites * steps / (ms / 1e3)
    ens.close()
    lats = []
    for p, f in zip(params, fields):
        lat = PL.Lattice(p)
        lat.upload(*f)
        lats.append(lat)
    for lat in lats:
        lat.evolve(2)
    lib = lats[0].lib
    for lat in lats:
        lat.synchronize()
    # per-lattice launches, two orders: (a) each lattice runs its steps in one
    # phn_evolve call (asynchronous launches, one synchronisation per lattice);
    # (b) all lattices advance one step at a time (one phn_evolve per lattice
    # per step).  The speed-up is quoted against the faster of the two.
    t0 = time.perf_counter()
    for lat in lats:
        lib.phn_evolve(lat.h, steps_per_lattice)
    for lat in lats:
        lat.synchronize()
    batched_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    for _ in range(steps_per_lattice):
        for lat in lats:
            lib.phn_evolve(lat.h, 1)
    for lat in lats:
        lat.synchronize()
    interleaved_s = time.perf_counter() - t0
    pl_rate = sites * steps_per_lattice / min(batched_s, interleaved_s)
    for lat in lats:
        lat.close()
    return {"members": len(sizes), "sites": sites, "steps": steps, "tile": tile,
            "site_updates_per_s": ens_rate, "ms_per_step": ms / steps, "launches_per_step": (n1 - n0) / steps,
            "per_lattice_site_updates_per_s": pl_rate, "per_lattice_steps": steps_per_lattice,
            "per_lattice_wall_s": {"one_call_per_lattice": batched_s, "one_call_per_lattice_step": interleaved_s},
            "speedup_vs_per_lattice": ens_rate / pl_rate,
            "hbm_gbs_algorithmic": 16 * sites * steps / (ms / 1e3) / 1e9}


def precision_form(N: int, steps: int, check_step: int = 500, tso_steps: int = 50):
    """Precision form (config C2): the same seeded 512^3 phi^6 run in FP64
    (the GPU oracle: bit-identical to the reference's FP64 arithmetic), plain
    FP32 and compensated FP32.  Reports, against FP64: the relative L2 error
    of phi after `check_step` steps, the per-bin relative error of the field
    spectrum F(|p|) at that step, and the relative energy drift
    |E(t) - E(0)| / |E(0)| over `steps` steps (E from the fused SO rows every
    `tso_steps` steps, FP64 sums)."""
    from phinum_gb300 import _lib as L
    from phinum_gb300 import lattice as PL
    phi, pi = make_fields(N)
    res = {}
    ref_phi = ref_F = None
    for name, prec in (("fp64", L.FP64), ("kahan_fp32", L.FP32_KAHAN), ("fp32", L.FP32)):
        lat = PL.Lattice(PL.Params(N=N, precision=prec))
        lat.upload(phi, pi)
        kernel = tune(L.load(), lat)
        t0 = time.perf_counter()
        energies = []
        done = 0
        e_check = None
        while done < steps:
            energies.append(lat.volume_averages()[14])  # SO row before the next evolve()
            lat.evolve(tso_steps)
            done += tso_steps
            if done == check_step:
                fphi, _ = lat.download()
                F, K, Q, C = lat.correlation_functions()
                e_check = (fphi, F)
        energies.append(lat.volume_averages()[14])
        wall = time.perf_counter() - t0
        lat.close()
        E = np.asarray(energies)
        r = {"energy0": float(E[0]), "energy_end": float(E[-1]),
             "drift_end": float(abs(E[-1] - E[0]) / abs(E[0])),
             "drift_max": float(np.max(np.abs(E - E[0])) / abs(E[0])), "wall_s": wall, "kernel": kernel}
        if name == "fp64":
            ref_phi, ref_F = e_check
        else:
            fphi, F = e_check
            r["l2_phi_rel_at_check"] = float(np.linalg.norm(fphi - ref_phi) / np.linalg.norm(ref_phi))
            nz = ref_F > 0
            rel = np.abs(F[nz] - ref_F[nz]) / ref_F[nz]
            r["spectrum_rel_err_max"] = float(rel.max())
            r["spectrum_rel_err_median"] = float(np.median(rel))
        res[name] = r
    res["kahan_drift_over_fp64_drift"] = res["kahan_fp32"]["drift_end"] / max(res["fp64"]["drift_end"], 1e-300)
    res["fp32_drift_over_fp64_drift"] = res["fp32"]["drift_end"] / max(res["fp64"]["drift_end"], 1e-300)
    return {"form": "precision", "N": N, "steps": steps, "check_step": check_step, "tso_steps": tso_steps,
            "workload": f"phi^6 (theory 0, Kappa=sqrt(3)), {N}^3, a=0.25, dtau=0.02, seeded Gaussian fields",
            "results": res}


def adjoint_form(N: int, steps: int, every: int = 50, ndir: int = 20, h_fd: float = 1e-3,
                 c6_steps=(1e-4, 1e-5, 1e-6, 1e-7), width_cfg: float = 0.1, check: bool = True,
                 reps_unchecked: int = 1, light: bool = False):
    """Adjoint form (config C4): phi^6, N^3, FP32, `steps` steps, checkpoints
    every `every`; J = sum rho sigmoid((rho - 2<rho>)/0.1) of the final state,
    in the configuration's units.  The kernels work in the reference's units
    (Phi = sqrt(6) phi, so rho_ref = 6 rho): the same objective is
    J_ref = sum rho_ref sigmoid((rho_ref - 2<rho_ref>)/0.6) = 6 J.
    Gradients w.r.t. the initial phi field, its homogeneous part phi0 and the
    phi^6 coupling, checked against the FP64 adjoint and against central
    finite differences of the FP64 forward (step h_fd) on `ndir` random unit
    directions; cost = (forward with checkpoints + backward) / plain forward.
    The FP32 adjoint runs with three forwards: FP32, FP64, and FP32 pairs
    (double-float arithmetic on the FP32 pipe).
    check=False times the all-FP32 adjoint only (`reps_unchecked` timed
    solves); light=True times the all-FP32 and the pair-forward adjoints and
    compares both with one FP64 adjoint (no finite differences)."""
    from phinum_gb300 import lattice as PL
    phi, pi = make_fields(N)
    sl = slice(N * N, -N * N)
    kappa = 3 ** 0.5
    # plain forward solves (the production step kernels, same steps) and the
    # adjoint pair, FP32 and FP64: one warm-up solve, then the median of
    # `reps` timed solves (device events)
    width = 6 * width_cfg  # the configuration's width in the reference's energy units
    out = {"form": "adjoint", "N": N, "steps": steps, "every": every, "width_config_units": width_cfg,
           "width_reference_units": width}
    res = {}
    # fp32_fwd64: the FP32 adjoint with its forward solve in FP64
    # (phn_adjoint_set_forward_precision); its plain forward is the FP64 one
    if light:
        legs = (("fp32", 1, reps_unchecked, None), ("fp32_pair", 1, reps_unchecked, 3), ("fp64", 0, 1, None))
    elif check:
        legs = (("fp32", 1, 5, None), ("fp64", 0, 2, None), ("fp32_fwd64", 1, 2, 0), ("fp32_pair", 1, 5, 3))
    else:
        legs = (("fp32", 1, reps_unchecked, None),)
    for name, prec, reps, fwd_prec in legs:
        plain = []
        if fwd_prec == 3:
            plain = [res["fp32"]["plain_ms"]]  # its cost against the plain FP32 forward
        elif fwd_prec is None:
            lat = PL.Lattice(PL.Params(N=N, precision=prec, kappa=kappa))
            for r in range(reps + 1):
                lat.upload(phi, pi)
                lat.evolve(steps)
                if r:
                    plain.append(lat.stats()[1])
            lat.close()
        else:
            plain = [res["fp64"]["plain_ms"]]
        with PL.Adjoint(PL.Params(N=N, precision=prec, kappa=kappa), steps, every, width,
                        forward_precision=fwd_prec) as adj:
            fl, bl = [], []
            for r in range(reps + 1):
                adj.forward(phi, pi)
                dphi, dpi, g = adj.backward()
                J, fms, bms = adj.info()
                if r:
                    fl.append(fms)
                    bl.append(bms)
        res[name] = {"J": J, "dphi": dphi, "g": g, "plain_ms": float(np.median(plain)),
                     "forward_ms": float(np.median(fl)), "backward_ms": float(np.median(bl))}
    r32 = res["fp32"]
    out["cost_ratio"] = (r32["forward_ms"] + r32["backward_ms"]) / r32["plain_ms"]
    out["forward_plain_ms"] = r32["plain_ms"]
    out["adjoint_forward_ms"] = r32["forward_ms"]
    out["adjoint_backward_ms"] = r32["backward_ms"]
    out["timing"] = ("device events; median of 5 (FP32) / 2 (FP64) solves after one warm-up solve; "
                     "adjoint = forward with checkpoints and J + backward (seed and reverse sweep)")
    if light:
        r64, rp = res["fp64"], res["fp32_pair"]
        d64 = r64["dphi"][sl]
        out["timing"] = (f"device events; median of {reps_unchecked} solve(s) after one warm-up solve; "
                         "errors against one FP64 adjoint")
        out["fp32_vs_fp64_field_rel_l2"] = float(np.linalg.norm(r32["dphi"][sl] - d64) / np.linalg.norm(d64))
        out["fp32_pair"] = {
            "what": "FP32 adjoint with its forward in FP32 pairs (double-float arithmetic on the FP32 pipe)",
            "cost_ratio": (rp["forward_ms"] + rp["backward_ms"]) / r32["plain_ms"],
            "adjoint_forward_ms": rp["forward_ms"], "adjoint_backward_ms": rp["backward_ms"],
            "vs_fp64_field_rel_l2": float(np.linalg.norm(rp["dphi"][sl] - d64) / np.linalg.norm(d64)),
            "vs_fp64_dphi0_rel": float(abs(rp["g"][0] - r64["g"][0]) / abs(r64["g"][0])),
            "vs_fp64_dc6_rel": float(abs(rp["g"][1] - r64["g"][1]) / abs(r64["g"][1])),
            "J_rel_to_fp64": float(abs(rp["J"] - r64["J"]) / abs(r64["J"]))}
        return out
    if not check:
        out["timing"] = (f"device events; median of {reps_unchecked} solve(s) after one warm-up solve "
                         "(no gradient checks)")
        return out
    r64 = res["fp64"]
    d32, d64 = res["fp32"]["dphi"][sl], res["fp64"]["dphi"][sl]
    out["J_fp32"], out["J_fp64"] = res["fp32"]["J"], res["fp64"]["J"]
    out["fp64"] = {"cost_ratio": (r64["forward_ms"] + r64["backward_ms"]) / r64["plain_ms"],
                   "forward_plain_ms": r64["plain_ms"], "adjoint_forward_ms": r64["forward_ms"],
                   "adjoint_backward_ms": r64["backward_ms"]}
    out["fp32_vs_fp64_field_rel_l2"] = float(np.linalg.norm(d32 - d64) / np.linalg.norm(d64))
    g32, g64 = res["fp32"]["g"], res["fp64"]["g"]
    out["fp32_vs_fp64_dphi0_rel"] = float(abs(g32[0] - g64[0]) / abs(g64[0]))
    out["fp32_vs_fp64_dc6_rel"] = float(abs(g32[1] - g64[1]) / abs(g64[1]))
    rp = res["fp32_pair"]
    dpp, gpp = rp["dphi"][sl], rp["g"]
    out["fp32_pair"] = {
        "what": "FP32 adjoint with its forward in FP32 pairs (double-float arithmetic on the FP32 pipe)",
        "cost_ratio": (rp["forward_ms"] + rp["backward_ms"]) / r32["plain_ms"],
        "adjoint_forward_ms": rp["forward_ms"], "adjoint_backward_ms": rp["backward_ms"],
        "J_rel_to_fp64": float(abs(rp["J"] - res["fp64"]["J"]) / abs(res["fp64"]["J"])),
        "vs_fp64_field_rel_l2": float(np.linalg.norm(dpp - d64) / np.linalg.norm(d64)),
        "vs_fp64_dphi0_rel": float(abs(gpp[0] - g64[0]) / abs(g64[0])),
        "vs_fp64_dc6_rel": float(abs(gpp[1] - g64[1]) / abs(g64[1]))}
    rm = res["fp32_fwd64"]
    dm, gm = rm["dphi"][sl], rm["g"]
    out["fp32_fwd64"] = {
        "what": "FP32 adjoint (checkpoints, reverse sweep) with an FP64 forward solve",
        "cost_ratio_vs_fp64_forward": (rm["forward_ms"] + rm["backward_ms"]) / r64["plain_ms"],
        "cost_ratio_vs_fp32_forward": (rm["forward_ms"] + rm["backward_ms"]) / r32["plain_ms"],
        "cost_vs_fp64_adjoint": (rm["forward_ms"] + rm["backward_ms"]) / (r64["forward_ms"] + r64["backward_ms"]),
        "adjoint_forward_ms": rm["forward_ms"], "adjoint_backward_ms": rm["backward_ms"],
        "J_equals_fp64": rm["J"] == res["fp64"]["J"],
        "vs_fp64_field_rel_l2": float(np.linalg.norm(dm - d64) / np.linalg.norm(d64)),
        "vs_fp64_dphi0_rel": float(abs(gm[0] - g64[0]) / abs(g64[0])),
        "vs_fp64_dc6_rel": float(abs(gm[1] - g64[1]) / abs(g64[1]))}
    # central finite differences of the FP64 forward
    rng = np.random.default_rng(99)
    errs64, errs32, errsm, errsp = [], [], [], []
    with PL.Adjoint(PL.Params(N=N, precision=0, kappa=kappa), steps, every, width) as adj:
        for _ in range(ndir):
            v = np.zeros_like(phi)
            v[sl] = rng.standard_normal(N ** 3)
            v /= np.linalg.norm(v[sl])
            fd = (adj.forward(phi + h_fd * v, pi) - adj.forward(phi - h_fd * v, pi)) / (2 * h_fd)
            errs64.append(abs(float(np.dot(d64, v[sl])) - fd) / abs(fd))
            errs32.append(abs(float(np.dot(d32, v[sl])) - fd) / abs(fd))
            errsm.append(abs(float(np.dot(dm, v[sl])) - fd) / abs(fd))
            errsp.append(abs(float(np.dot(dpp, v[sl])) - fd) / abs(fd))
        # the homogeneous shift moves every site at once: a far smaller step
        # keeps the central difference out of the sigmoid's curvature
        h_s = 1e-7
        one = np.ones_like(phi)
        fd_phi0 = (adj.forward(phi + h_s * one, pi) - adj.forward(phi - h_s * one, pi)) / (2 * h_s)
    c6 = 1.0 / (720 * kappa ** 2)
    fd_c6_by_step = {}
    for h_c in c6_steps:
        Jc = []
        for d in (+1, -1):
            c = c6 * (1 + d * h_c)
            with PL.Adjoint(PL.Params(N=N, precision=0, kappa=(1.0 / (720 * c)) ** 0.5), steps, every, width) as adj:
                Jc.append(adj.forward(phi, pi))
        fd_c6_by_step[str(h_c)] = (Jc[0] - Jc[1]) / (2 * h_c * c6)
    # the central difference in c6 converges once the step is small
    # (1e-4 and 1e-5 sit in the curvature of the sigmoid objective)
    fd_c6 = fd_c6_by_step[str(c6_steps[-1])]
    out["dc6_fd_by_relative_step"] = fd_c6_by_step
    out["fd_directions"] = ndir
    out["fd_step"] = h_fd
    out["fp64_adjoint_vs_fd_rel_max"] = float(max(errs64))
    out["fp32_adjoint_vs_fd_rel_max"] = float(max(errs32))
    out["fp32_adjoint_vs_fd_rel_median"] = float(np.median(errs32))
    out["fp32_fwd64"]["vs_fd_rel_max"] = float(max(errsm))
    out["fp32_pair"]["vs_fd_rel_max"] = float(max(errsp))
    out["dphi0"] = {"fp32": float(g32[0]), "fp64": float(g64[0]), "fd": fd_phi0}
    out["dc6"] = {"fp32": float(g32[1]), "fp64": float(g64[1]), "fd": fd_c6}
    # the configuration's units: J = J_ref / 6, phi_ref = sqrt(6) phi, c6 = g / 216
    out["config_units"] = {"J": out["J_fp32"] / 6, "dJ_dphi0": float(g32[0]) * 6 ** 0.5 / 6,
                           "dJ_dg": float(g32[1]) / 216.0 / 6}
    return out


def c1_form(N: int = 256, steps: int = 5000, seed: int = 2027, oracle_threads: int = 0):
    """The GPU drop-in configuration (C1): 256^3, 5000 steps, dtau = 0.02,
    a = 0.25, the phi^6 potential (theory 0, Kappa = sqrt(3), phi0 = sqrt(6))
    and the tilted double well (theory 1, Mass_Mode -1, Lambda_Mode 1,
    h = sqrt(6) 0.05, phi0 = -sqrt(6)), in FP64, FP32 and compensated FP32 on
    the same seeded inputs, and the reference's arithmetic on the host (the
    oracle, FP64, all threads) on the same inputs.

    Inputs: the reference's own initial conditions (SetInitialConditions,
    initialize 3, drand48 from srand48(seed), the configuration's spectrum:
    Noise 3 below |p| = 2 pi) generated on the device in FP64.  Each run is
    the reference loop with SO rows every 50 steps (TSO 1.0) and no
    false-vacuum break: the tilted well starts at <V> < 0, where the
    reference's false_vacuum_decayed() would stop at once.  At the end: the
    spectrum (reference bins), islands with the reference's mask (thres =
    2.57583 sqrt(<phi^2>) at t = 0, main.cpp:70) and with the configuration's
    energy mask (rho > 2 <rho>, z periodic), and the fields.

    Reported per potential: device time and rate of each precision; FP64
    against the oracle (fields bit for bit, rows, spectrum, island labels);
    FP32 and compensated FP32 against FP64 (energy rows, drift, field L2,
    per-bin spectrum, island counts and mask agreement)."""
    import ctypes
    from oracle import oracle as O
    from phinum_gb300 import _lib as L
    from phinum_gb300 import lattice as PL
    sq6 = 6 ** 0.5
    pots = {"phi6": (dict(theory=0, kappa=3 ** 0.5), sq6),
            "tilted_well": (dict(theory=1, mass_mode=-1, lambda_mode=1, h=sq6 * 0.05), -sq6)}
    out = {"form": "c1", "N": N, "steps": steps, "tso_steps": 50, "seed": seed,
           "workload": f"{N}^3, {steps} steps, a=0.25, dtau=0.02; phi^6 and tilted double well; "
                       "the reference's initial conditions (initialize 3, Noise 3 below |p| = 2 pi)"}
    nt = oracle_threads or O.max_threads(False)
    lib = L.load()
    for pname, (kw, phi0) in pots.items():
        gen = PL.Lattice(PL.Params(N=N, precision=0, **kw))
        gen.initial_conditions(seed=seed, noise=3.0, scale2=2 * np.pi, phi0=(phi0, 0.0))
        phi, pi = gen.download()
        avg0 = gen.volume_averages(allow_nonfinite=True)
        gen.close()
        thr = 2.57583 * float(np.sqrt(avg0[O_AVG_PHI2]))
        runs = {}
        for name, prec in (("fp64", L.FP64), ("fp32", L.FP32), ("kahan_fp32", L.FP32_KAHAN)):
            lat = PL.Lattice(PL.Params(N=N, precision=prec, **kw))
            lat.upload(phi, pi)
            kernel = tune(lib, lat) if prec != L.FP64 else "step_f64"
            t0 = time.perf_counter()
            rows = lat.run_loop(steps, 1.0, max_rows=steps // 50 + 2)
            wall = time.perf_counter() - t0
            _, ms, _ = lat.stats()
            F, K, Q, C = lat.correlation_functions()
            fphi, fpi = lat.download()
            if name == "fp64":
                rho_thr = 2.0 * float(lat.volume_averages(allow_nonfinite=True)[O_AVG_ENERGY])
            lab_r, rec_r = lat.full_analysis(thr)
            lab_e, rec_e = lat.full_analysis(rho_thr, mode=L.ISLAND_ENERGY, z_periodic=True)
            lat.close()
            runs[name] = dict(rows=rows, F=F, C=C, phi=fphi, lab_r=lab_r, rec_r=rec_r, lab_e=lab_e, rec_e=rec_e,
                              timing={"device_ms": ms, "wall_s": wall, "kernel": kernel,
                                      "site_updates_per_s": N ** 3 * steps / (ms / 1e3)})
        r64 = runs["fp64"]
        res = {"threshold_reference_mask": thr, "threshold_energy_mask": rho_thr,
               "timing": {k: v["timing"] for k, v in runs.items()},
               "islands_fp64": {"reference_mask": int(r64["rec_r"].shape[0]),
                                "energy_mask": int(r64["rec_e"].shape[0])}}
        e64 = r64["rows"][:, O_AVG_ENERGY]
        sl = slice(N * N, -N * N)
        nz = r64["F"] > 0
        for name in ("fp32", "kahan_fp32"):
            r = runs[name]
            e = r["rows"][:, O_AVG_ENERGY]
            rel = np.abs(r["F"][nz] - r64["F"][nz]) / r64["F"][nz]
            res[f"{name}_vs_fp64"] = {
                "energy_rows_rel_err_max": float(np.max(np.abs(e - e64) / np.abs(e64))),
                "energy_drift": float(abs(e[-1] - e[0]) / abs(e[0])), "energy_drift_fp64": float(abs(e64[-1] - e64[0])
                                                                                              / abs(e64[0])),
                "phi_rel_l2_end": float(np.linalg.norm(r["phi"][sl] - r64["phi"][sl]) / np.linalg.norm(r64["phi"][sl])),
                "spectrum_rel_err_max": float(rel.max()), "spectrum_rel_err_median": float(np.median(rel)),
                "spectrum_counts_equal": bool(np.array_equal(r["C"], r64["C"])),
                "islands_reference_mask": int(r["rec_r"].shape[0]),
                "islands_energy_mask": int(r["rec_e"].shape[0]),
                "energy_mask_sites_differing": int(np.count_nonzero((r["lab_e"] >= 0) != (r64["lab_e"] >= 0))),
                "energy_mask_labels_equal": bool(np.array_equal(r["lab_e"], r64["lab_e"])),
                "reference_mask_labels_equal": bool(np.array_equal(r["lab_r"], r64["lab_r"]))}
        # the reference's arithmetic on the host: the oracle on the same inputs
        p = O.Params(N=N, **kw)
        ophi, opi = phi.copy(), pi.copy()
        t0 = time.perf_counter()
        orows, clock = O.run_loop(p, ophi, opi, steps, 1.0, max_rows=steps // 50 + 2, nthreads=nt)
        t_or = time.perf_counter() - t0
        oF, oK, oQ, oC = O.spectrum(p, ophi, opi)
        olab_r, orec_r = O.islands(p, ophi, opi, thr, clock=clock)
        olab_e, orec_e = O.islands(p, ophi, opi, rho_thr, mode=1, zper=1, clock=clock)
        res["fp64_vs_oracle"] = {
            "oracle_wall_s": t_or, "oracle_threads": nt,
            "oracle_site_updates_per_s": N ** 3 * steps / t_or,
            "phi_bit_identical": bool(np.array_equal(r64["phi"], ophi)),
            "rows": int(orows.shape[0]),
            "extrema_exact": bool(np.array_equal(r64["rows"][:, 17:23], orows[:, 17:23])),
            "row_sums_rel_err_max": float(np.max(np.abs(r64["rows"][:, 9:17] - orows[:, 9:17]) /
                                                 np.maximum(np.abs(orows[:, 9:17]), 1e-300))),
            "spectrum_counts_equal": bool(np.array_equal(r64["C"], oC)),
            "spectrum_max_abs_err_over_largest_bin": float(np.max(np.abs(r64["F"] - oF)) / np.max(np.abs(oF))),
            "reference_mask_labels_equal": bool(np.array_equal(r64["lab_r"], olab_r)),
            "energy_mask_labels_equal": bool(np.array_equal(r64["lab_e"], olab_e)),
            "islands_oracle": {"reference_mask": int(orec_r.shape[0]), "energy_mask": int(orec_e.shape[0])}}
        out[pname] = res
    return out


def initial_form(N: int, n_cpu: int = 128, n_check: int = 64):
    """Initial conditions (SetInitialConditions, initialize 3, the
    configuration's spectrum: Noise 3 below |p| = 2 pi, phi0 = sqrt(6)) on the
    GPU: wall time of one phn_initial_conditions call (drand48 stream, mode
    assignment, amplitudes, two cuFFT Z2D, stores; cuFFT plan included),
    median of 3 after a warm-up call.  Agreement with the oracle at n_check^3
    and the oracle's single-thread time at n_cpu^3 (the reference generates on
    one thread per rank)."""
    from oracle import oracle as O
    from phinum_gb300 import lattice as PL
    ic = dict(seed=2026, noise=3.0, scale2=2 * np.pi, phi0=(6 ** 0.5, 0.0))
    out = {"form": "initial", "N": N, "ic": {k: v for k, v in ic.items()}}
    for name, prec in (("fp64", 0), ("fp32", 1)):
        lat = PL.Lattice(PL.Params(N=N, precision=prec))
        lat.initial_conditions(**ic)
        ts = []
        for _ in range(3):
            t0 = time.perf_counter()
            lat.initial_conditions(**ic)
            ts.append(time.perf_counter() - t0)
        lat.close()
        t = float(np.median(ts))
        out[name] = {"ms": t * 1e3, "sites_per_s": N ** 3 / t}
    lat = PL.Lattice(PL.Params(N=n_check))
    lat.initial_conditions(**ic)
    phi, pi = lat.download()
    lat.close()
    ophi, opi = O.initial_conditions(O.Params(N=n_check), **ic)
    sl = slice(n_check ** 2, -n_check ** 2)
    out["check"] = {"N": n_check, "phi_max_dev_rel": float(np.abs(phi - ophi).max() / np.abs(ophi).max()),
                    "pi_max_dev_rel": float(np.abs(pi[sl] - opi[sl]).max() / np.abs(opi[sl]).max())}
    t0 = time.perf_counter()
    O.initial_conditions(O.Params(N=n_cpu), **ic)
    t = time.perf_counter() - t0
    out["cpu_oracle"] = {"N": n_cpu, "s": t, "sites_per_s": n_cpu ** 3 / t, "cores": 1}
    out["speedup_fp64_vs_cpu_sites_per_s"] = out["fp64"]["sites_per_s"] / out["cpu_oracle"]["sites_per_s"]
    return out


def analysis_form(N: int, reps: int = 5, steps: int = 200, precisions=("fp32", "fp64")):
    """The analysis passes of the hot path on the bench's 512^3 phi^6 lattice
    after `steps` FP32 steps, wall time per call (the calls return host
    results, so each ends synchronised), median of `reps` after a warm-up:
    the reference spectrum (2 x cuFFT R2C + binning into the reference's bins,
    Calculate_CorrelationFunctions), the configuration's 64 uniform bins,
    Full_Analysis's labelling with the reference mask (thres = 2.57583
    sqrt(<phi^2>), main.cpp:70) and with the configuration's mask
    (rho > 2 <rho>, z periodic), island statistics to the host, labels kept on
    the device.  FP32 and FP64 fields."""
    from phinum_gb300 import _lib as L
    from phinum_gb300 import lattice as PL
    phi, pi = make_fields(N)
    out = {"form": "analysis", "N": N, "steps_before": steps}

    def timed(fn):
        ts = []
        for _ in range(reps):
            t0 = time.perf_counter()
            r = fn()
            ts.append(time.perf_counter() - t0)
        return float(np.median(ts)) * 1e3, r

    for name, prec in (("fp32", L.FP32), ("fp64", L.FP64)):
        if name not in precisions:
            continue
        lat = PL.Lattice(PL.Params(N=N, precision=prec))
        lat.upload(phi, pi)
        lat.evolve(steps)
        avg = lat.volume_averages()
        thr = 2.57583 * float(np.sqrt(avg[O_AVG_PHI2]))
        lat.correlation_functions()  # warm-up: cuFFT plan, key tables
        lat.spectrum_uniform(64)
        ms_spec, spec = timed(lat.correlation_functions)
        t_fft, t_bin = lat.spectrum_timing()  # device time of the last call
        ms_uni, _ = timed(lambda: lat.spectrum_uniform(64))
        rho_thr = 2.0 * avg[O_AVG_ENERGY]
        # warm-up calls size the record buffers to the island counts
        n_isl = lat.full_analysis(thr, labels=False, max_out=1 << 23)[1].shape[0]
        n_rho = lat.full_analysis(rho_thr, mode=L.ISLAND_ENERGY, z_periodic=True, labels=False,
                                  max_out=1 << 23)[1].shape[0]
        ms_isl, isl = timed(lambda: lat.full_analysis(thr, labels=False, max_out=n_isl))
        # the same with the records copied into a page-locked host buffer
        pinned = np.zeros((n_isl, len(L.ISLAND_FIELDS)))
        L.check(lat.lib.phn_pin_host(pinned.ctypes.data, pinned.nbytes))
        try:
            ms_isl_pin, isl_pin = timed(lambda: lat.full_analysis(thr, labels=False, out=pinned))
            # the same islands (index, size, volume, peak and seed positions
            # exact; the FP64 sums add block partials in arrival order, so they
            # agree to rounding from call to call)
            a, b = isl_pin[1], isl[1]
            exact = [0, 1, 2, 7, 8, 9]  # index, size, volume, peak position and value, seed
            pin_equal = bool(a.shape == b.shape and np.array_equal(a[:, exact], b[:, exact]) and
                             np.all(np.abs(a - b) <= 1e-12 * np.abs(b).max(axis=0)))
        finally:
            lat.lib.phn_unpin_host(pinned.ctypes.data)
        ms_isl_dev, _ = timed(lambda: lat.full_analysis_device(thr))
        ms_rho, rho = timed(lambda: lat.full_analysis(rho_thr, mode=L.ISLAND_ENERGY, z_periodic=True, labels=False,
                                                      max_out=n_rho))
        elem = 8 if prec == L.FP32 else 16  # complex bytes
        half = N * N * (N // 2 + 1) * elem
        # the binning pass reads both half-spectra and the key table once:
        # its roofline against the measured copy bandwidth
        bin_bytes = 2 * half + 2 * N * N * (N // 2 + 1)
        peak, peak_kind = peaks()
        out[name] = {"spectrum_ms": ms_spec, "spectrum_bins": int(spec[3].size),
                     "spectrum_transforms_device_ms": t_fft, "spectrum_binning_device_ms": t_bin,
                     "spectrum_binning_bytes": bin_bytes,
                     "spectrum_binning_gbs": bin_bytes / (t_bin * 1e-3) / 1e9 if t_bin > 0 else None,
                     "spectrum_binning_frac_of_measured_hbm":
                         (bin_bytes / (t_bin * 1e-3) / 1e9 / peak) if t_bin > 0 else None,
                     "hbm_peak_gbs": peak, "hbm_peak_kind": peak_kind,
                     "spectrum_uniform64_ms": ms_uni,
                     "spectrum_halfspectra_bytes": 2 * half,
                     "islands_reference_mask_ms": ms_isl, "islands_reference_mask_count": int(isl[1].shape[0]),
                     "islands_reference_mask_device_records_ms": ms_isl_dev,
                     "islands_reference_mask_pinned_records_ms": ms_isl_pin,
                     "islands_pinned_records_equal": pin_equal,
                     "islands_reference_mask_sites": int(isl[1][:, 1].sum()),
                     "islands_energy_mask_ms": ms_rho, "islands_energy_mask_count": int(rho[1].shape[0]),
                     "islands_energy_mask_sites": int(rho[1][:, 1].sum()),
                     "threshold": thr}
        lat.close()
    return out


O_AVG_PHI2, O_AVG_ENERGY = 9, 14  # phn_averages columns: avgphi2, avgEnergy


def io_form(N: int, directory: str):
    """Checkpoint files (SaveConfig / ExtractConfig format): phn_save_config
    and phn_load_config on an N^3 FP64 lattice with all host threads and with
    one (the reference's single fprintf loop), wall time each; the two
    outputs are compared byte for byte."""
    import hashlib
    from phinum_gb300 import lattice as PL
    phi, pi = make_fields(N)
    out = {"form": "io", "N": N, "lines": N ** 3}
    os.makedirs(directory, exist_ok=True)
    with PL.Lattice(PL.Params(N=N, precision=0)) as lat:
        lat.upload(phi, pi)
        for name, nt in (("all_threads", 0), ("one_thread", 1)):
            d = os.path.join(directory, name)
            os.makedirs(d, exist_ok=True)
            t0 = time.perf_counter()
            lat.save_config(1, d, nthreads=nt)
            ts = time.perf_counter() - t0
            t0 = time.perf_counter()
            lat.load_config(1, d, nthreads=nt)
            tl = time.perf_counter() - t0
            path = os.path.join(d, "field-1-0.out")
            with open(path, "rb") as f:
                sha = hashlib.sha256(f.read()).hexdigest()
            out[name] = {"threads": nt if nt else os.cpu_count(), "save_s": ts, "load_s": tl,
                         "bytes": os.path.getsize(path), "sha256": sha}
            os.remove(path)
    out["identical_bytes"] = out["all_threads"]["sha256"] == out["one_thread"]["sha256"]
    out["save_speedup"] = out["one_thread"]["save_s"] / out["all_threads"]["save_s"]
    out["load_speedup"] = out["one_thread"]["load_s"] / out["all_threads"]["load_s"]
    return out


def cpu_reference_rate(N: int, max_seconds: float, steps_cap: int, warmup: int = 1, precision: str = "f32"):
    """The reference loop restated in the oracle (orc_evolve: the default
    double build; orc_evolve_f32: the doubleprecision -1 float build, pinned
    bit-identical to the reference's own float build), compiled with the
    reference's -O3 -ffast-math flags, on all host threads (OpenMP over
    z-slabs, the analogue of mpirun -np K), bounded in time."""
    from oracle import oracle as O
    O.build()
    p = O.Params(N=N)
    phi, pi = make_fields(N)
    nt = O.max_threads(True)
    if precision == "f32":
        phi, pi = phi.astype(np.float32), pi.astype(np.float32)
        clock = O.Clock32(p, fast=True)
        step = lambda n: O.evolve_f32(p, phi, pi, n, clock, nthreads=nt, fast=True)  # noqa: E731
    else:
        phi, pi = phi.copy(), pi.copy()
        clock = O.Clock(p, fast=True)
        step = lambda n: O.evolve(p, phi, pi, n, clock, nthreads=nt, fast=True)  # noqa: E731
    step(max(1, warmup))  # warm-up, page-in
    t0 = time.perf_counter()
    steps = 0
    while steps < steps_cap and time.perf_counter() - t0 < max_seconds:
        step(1)
        steps += 1
    dt = time.perf_counter() - t0
    return N ** 3 * steps / dt, nt, steps, dt


def cpu_sample(N, rate, nt, steps, dt, precision):
    build = "float (doubleprecision -1)" if precision == "f32" else "double (doubleprecision 0)"
    return (f"{steps} steps of the {N}^3 lattice ({dt:.1f} s), the reference's {build} loop restated in C, "
            f"{nt} OpenMP threads over z-slabs, -O3 -ffast-math (reference flags)")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--quick", action="store_true", help="skip the slow FP64/compensated extra lines")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-extra", action="store_true", help="skip the other sizes/precisions")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer leg")
    ap.add_argument("--n", "--lattice-edge", dest="n", type=int, default=N_MAIN,
                    help="lattice edge (profiling runs use smaller cases); under torchrun spell it --lattice-edge")
    ap.add_argument("--variant", type=int, default=None, help="TMA kernel variant instead of the autotuner's pick")
    ap.add_argument("--form", default=None,
                    choices=["precision", "adjoint", "ensemble", "initial", "io", "analysis", "c1"],
                    help="report one of the extra forms (or the analysis passes) instead of the benchmark line")
    args = ap.parse_args()
    rank, local, world = env_rank()
    config = {"workload": f"phi^6 oscillon (theory 0, Kappa=sqrt(3)), {args.n}^3 periodic lattice, a=0.25, "
                          f"dtau=0.02, leapfrog kick-drift with fused volume averages + extrema every "
                          f"{TSO_STEPS} steps (TSO=1.0)",
              "N": args.n, "sites": args.n ** 3, "tso_steps": TSO_STEPS,
              "l2": "inputs larger than L2 (1.5 GB of fields vs 129 MB L2); no flush",
              "parallelism": f"replicas x{args.gpus}"}

    if args.form == "precision":
        print(json.dumps(precision_form(args.n, max(args.steps, 500))))
        return
    if args.form == "adjoint":
        kw = dict(light=True, reps_unchecked=1) if args.quick else {}
        print(json.dumps(adjoint_form(args.n, args.steps, **kw)))
        return
    if args.form == "io":
        import shutil
        import tempfile
        scratch = tempfile.mkdtemp(prefix="phn_io_")
        try:
            print(json.dumps(io_form(args.n, scratch)))
        finally:
            shutil.rmtree(scratch, ignore_errors=True)
        return
    if args.form == "initial":
        print(json.dumps(initial_form(args.n)))
        return
    if args.form == "analysis":
        print(json.dumps(analysis_form(args.n)))
        return
    if args.form == "c1":
        n = args.n if args.n != N_MAIN else 256
        print(json.dumps(c1_form(n, args.steps if args.steps != 1000 else 5000)))
        return
    if args.form == "ensemble":
        out = measure_ensemble(max(args.steps, 100), 100)
        out["workload"] = ("ensemble: 128 x 32^3 + 96 x 64^3 + 32 x 128^3 phi^6 lattices, FP32, "
                           "phi0 ~ U[0.8,1.2], g ~ U[0.05,0.2] from a fixed seed")
        print(json.dumps(out))
        return

    if args.impl == "reference":
        if rank != 0:
            return
        # the reference's single-precision build, like for like with this
        # benchmark's FP32 arm; its default double build beside it
        warm = max(3, args.warmup)
        rate, nt, steps, dt = cpu_reference_rate(args.n, 40.0, max(1, args.steps), warm, "f32")
        r64, nt64, s64, dt64 = cpu_reference_rate(args.n, 25.0, max(1, args.steps), 1, "f64")
        line = {"impl": "reference", "metric": METRIC, "value": rate, "unit": METRIC, "n_gpus": args.gpus,
                "steps": steps, "warmup": warm, "ms_per_step": dt * 1e3 / steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": config,
                "cpu_baseline": {"value": rate, "unit": METRIC, "cores": nt, "kind": "port",
                                 "sample": cpu_sample(args.n, rate, nt, steps, dt, "f32")},
                "e2e": {"value": rate, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                "also": {"f64": {"value": r64, "unit": METRIC, "cores": nt64, "kind": "port",
                                 "sample": cpu_sample(args.n, r64, nt64, s64, dt64, "f64")}}}
        print(json.dumps(line))
        return

    if world > 1:
        # one replica per GPU: this rank sees only its own device
        os.environ["CUDA_DEVICE_ORDER"] = "PCI_BUS_ID"
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    dist = Dist()
    res = measure_gpu(args, dist)
    line = {"metric": METRIC, "value": res["value"], "unit": METRIC, "n_gpus": world, "steps": args.steps,
            "warmup": max(3, args.warmup), "ms_per_step": res["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": config,
            "roofline": res["roofline"], "e2e": res["e2e"], "clocks": res["clocks"],
            "gpu_launches": res["gpu_launches"], "also": res["also"], "observed_step": res.get("observed_step"),
            "so_rows": res["rows"], "energy_drift_rel": res["energy_drift"]}
    if rank == 0 and world == 1 and not args.no_cpu:
        # like for like: the reference's float build against this FP32 line,
        # its double build against the FP64 GPU line (also.n512_fp64)
        rate, nt, steps, dt = cpu_reference_rate(args.n, 15.0, 200, 3, "f32")
        line["cpu_baseline"] = {"value": rate, "unit": METRIC, "cores": nt, "kind": "port", "dtype": "f32",
                                "sample": cpu_sample(args.n, rate, nt, steps, dt, "f32")}
        r64, nt64, s64, dt64 = cpu_reference_rate(args.n, 10.0, 200, 1, "f64")
        line["cpu_baseline_fp64"] = {"value": r64, "unit": METRIC, "cores": nt64, "kind": "port", "dtype": "f64",
                                     "sample": cpu_sample(args.n, r64, nt64, s64, dt64, "f64")}
        lfl = {"fp32_gpu_over_fp32_cpu": res["value"] / rate,
               "fp32_e2e_over_fp32_cpu": res["e2e"]["value"] / rate if res["e2e"] else None}
        g64 = res["also"].get(f"n{args.n}_fp64")
        if g64:
            lfl["fp64_gpu_over_fp64_cpu"] = g64["site_updates_per_s"] / r64
        line["like_for_like"] = lfl
    if rank == 0:
        print(json.dumps(line))
    dist.close()


if __name__ == "__main__":
    main()
