"""Checkpoint files (SaveConfig / ExtractConfig, fieldanalysis.cpp:252-312):
the library's writer produces the reference's bytes (SHA-256 of the
reference's own SaveConfig output in tests/golden/config/, made by
make_golden.py with the pinned reference), and reading gives back exactly
what was written."""
import glob
import hashlib
import json
import os

import numpy as np
import pytest

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "config")
CASES = sorted(os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(HERE, "*.npz")))


def load(name):
    with np.load(os.path.join(HERE, name + ".npz"), allow_pickle=False) as z:
        d = {k: z[k] for k in z.files}
    d["params"] = json.loads(str(d["params"]))
    return d


def lib():
    from phinum_gb300 import _lib as L
    return L, L.load()


def test_fixtures_present():
    assert len(CASES) >= 3


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("nthreads", [1, 3])
def test_writer_bytes_match_reference_save_config(name, nthreads, tmp_path):
    L, lb = lib()
    d = load(name)
    N, Nc = d["params"]["N"], d["params"]["Nc"]
    prec = L.FP64 if str(d["prec"]) == "f64" else L.FP32
    path = str(tmp_path / "field.out").encode()
    phi, pi = np.ascontiguousarray(d["phi"]), np.ascontiguousarray(d["pi"])
    L.check(lb.phn_write_config_file(path, phi.ctypes.data_as(L._PD), pi.ctypes.data_as(L._PD), N, Nc, prec,
                                     nthreads))
    raw = open(path, "rb").read()
    assert len(raw) == int(d["nbytes"])
    assert hashlib.sha256(raw).hexdigest() == str(d["sha"])


@pytest.mark.parametrize("name", CASES)
def test_read_back_is_exact(name, tmp_path):
    L, lb = lib()
    d = load(name)
    N, Nc = d["params"]["N"], d["params"]["Nc"]
    prec = L.FP64 if str(d["prec"]) == "f64" else L.FP32
    path = str(tmp_path / "field.out").encode()
    phi, pi = np.ascontiguousarray(d["phi"]), np.ascontiguousarray(d["pi"])
    L.check(lb.phn_write_config_file(path, phi.ctypes.data_as(L._PD), pi.ctypes.data_as(L._PD), N, Nc, prec, 2))
    rphi, rpi = np.zeros_like(phi), np.zeros_like(pi)
    L.check(lb.phn_read_config_file(path, rphi.ctypes.data_as(L._PD), rpi.ctypes.data_as(L._PD), N, Nc, 4))
    sl = slice(Nc * N * N, -Nc * N * N)
    if prec == L.FP64:
        assert np.array_equal(rphi[sl], phi[sl]) and np.array_equal(rpi[sl], pi[sl])
    else:  # "%.9e" identifies the float; it comes back exactly once rounded to float (as an FP32 handle does)
        assert np.array_equal(rphi[sl].astype(np.float32), phi[sl].astype(np.float32))
        assert np.array_equal(rpi[sl].astype(np.float32), pi[sl].astype(np.float32))


def test_reader_rejects_short_and_malformed_files(tmp_path):
    L, lb = lib()
    N = 4
    phi, pi = np.zeros(N * N * (N + 2)), np.zeros(N * N * (N + 2))
    short = tmp_path / "short.out"
    short.write_text("1.0 2.0\n" * 10)
    assert lb.phn_read_config_file(str(short).encode(), phi.ctypes.data_as(L._PD), pi.ctypes.data_as(L._PD), N, 1,
                                   2) == L.ERR_INVALID
    bad = tmp_path / "bad.out"
    bad.write_text("1.0 2.0\n" * 20 + "x y\n" + "1.0 2.0\n" * 43)
    assert lb.phn_read_config_file(str(bad).encode(), phi.ctypes.data_as(L._PD), pi.ctypes.data_as(L._PD), N, 1,
                                   2) == L.ERR_INVALID
    assert lb.phn_read_config_file(str(tmp_path / "none.out").encode(), phi.ctypes.data_as(L._PD),
                                   pi.ctypes.data_as(L._PD), N, 1, 2) == L.ERR_INVALID
