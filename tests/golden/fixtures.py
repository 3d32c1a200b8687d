"""Loads the golden fixtures written by make_golden.py."""
from __future__ import annotations

import glob
import hashlib
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def names():
    return sorted(os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(HERE, "*.npz")))


def load(name: str) -> dict:
    with np.load(os.path.join(HERE, name + ".npz"), allow_pickle=False) as z:
        d = {k: z[k] for k in z.files}
    d["params"] = json.loads(str(d["params"]))
    for k in ("seed", "steps"):
        d[k] = int(d[k])
    for k in ("phi0", "tso", "a", "dt", "tau_end"):
        d[k] = float(d[k])
    return d


def checkpoints(d: dict):
    return sorted(int(k.split("_")[-1]) for k in d if k.startswith("phi_sha_"))


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()


def label_digest(lab: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(lab, dtype="<i4").tobytes()).hexdigest()


def inputs_for(d: dict):
    import inputs
    p = d["params"]
    return inputs.lattice_fields(p["N"], p["Nc"], d["seed"], phi0=d["phi0"])
