"""Shared test cases: molecules, walkers and parameters (regenerated from seeds)."""
from __future__ import annotations

import functools
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests" / "golden"))

from sparse_wf_gb300 import params as P, systems  # noqa: E402

GOLDEN = ROOT / "tests" / "golden"

MOLECULES = {
    "h10": lambda: systems.hydrogen_chain(10, 1.8),
    "h10_plain": lambda: systems.hydrogen_chain(10, 1.8),
    "c2h6": lambda: systems.alkane(2),
    "c10h22": lambda: systems.alkane(10),
}


@functools.lru_cache(maxsize=None)
def golden(name):
    return dict(np.load(GOLDEN / f"{name}.npz"))


@functools.lru_cache(maxsize=None)
def case(name):
    """(mol, n_up, walkers float32, params dict (float64 values of the float32 blob), blob, offsets)."""
    from make_golden import make_params

    g = golden(name)
    mol = MOLECULES[name]()
    nu = int(g["n_up"])
    r = g["r"]
    dims, p, blob, offs = make_params(mol, nu, r[0], seed=int(g["param_seed"]), activate=bool(g["activate"]))
    return mol, nu, r, p, blob, offs


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.abs(a - b) / np.maximum(np.abs(b), 1e-300)
