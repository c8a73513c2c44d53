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


# ------------------------------------------------------------------ the oracle on all host cores
_ORACLE = {}


def _oracle_init(R, Z, n_up, params):
    from oracle import fire_oracle as O

    _ORACLE["prob"] = O.Problem(R, Z, n_up)
    _ORACLE["p"] = params


def _oracle_fl(w):
    """(log|psi|, E_kin, E_pot, |lap| + |grad|^2, grad, lap) of one walker (FP64 oracle)."""
    from oracle import fire_oracle as O

    prob, p = _ORACLE["prob"], _ORACLE["p"]
    w = np.asarray(w, np.float64)
    lp, g, lap = O.logpsi_fl(prob, p, w)
    return lp, -0.5 * (lap + g @ g), O.potential_energy(w, prob.R, prob.Z), abs(lap) + g @ g, g, lap


def oracle_batch(mol, n_up, params, walkers):
    """The oracle's forward Laplacian of every walker, one walker per process ("spawn" pool, one BLAS thread each):
    dict of log|psi|, E_kin, E_pot, E_loc, ks = (|lap| + |grad|^2) / 2, grad [B, n, 3], lap."""
    import multiprocessing as mp
    import os

    for k in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):
        os.environ[k] = "1"
    procs = max(1, min(len(walkers), os.cpu_count() or 1))
    with mp.get_context("spawn").Pool(procs, initializer=_oracle_init, initargs=(mol.R, mol.Z, n_up, params)) as pool:
        res = pool.map(_oracle_fl, list(walkers), chunksize=max(1, len(walkers) // (4 * procs)))
    lp, ekin, epot, two_ks = (np.array([x[k] for x in res]) for k in range(4))
    return dict(logpsi=lp, ekin=ekin, epot=epot, eloc=ekin + epot, ks=0.5 * two_ks,
                grad=np.array([x[4] for x in res]).reshape(len(walkers), -1, 3), lap=np.array([x[5] for x in res]))


# ------------------------------------------------------------------ the FP32 / mixed local-energy contract
ELOC_TOL = {"fp32": 1e-5, "mixed": 1e-4}


def check_eloc_contract(precision, wf, got, eloc, ks, epot, refined, lap=None, lap_ref=None, grad=None, grad_ref=None,
                        tol=None):
    """Per-walker local-energy contract of the FP32 (1e-5) and mixed (1e-4) paths against the FP64 oracle.

    E_loc = -(lap log psi + |grad log psi|^2) / 2 + V is a sum of terms that cancel: near a node of psi the two
    kinetic terms, and for a walker whose kinetic energy balances its potential energy (E_loc crosses zero) the
    kinetic and potential terms.  Its error is held relative to the magnitude of those terms,
    S = ks + |V| with ks = (|lap log psi| + |grad log psi|^2) / 2 (the reference's own float32 energy test allows 1e-2
    of |E_kin|): |dE_loc| <= tol S on every walker, and on every walker away from a node (ks <= 8 |E_loc|)
    |d lap| <= 2 tol S and |d grad| <= tol sqrt(2 S).  Every walker
    whose ks exceeds 1.05 refine_ratio |E_loc| must have gone through the
    device's FP64 refinement pass, and so must every walker whose ks exceeds 1.05 refine_ks.  Returns the fraction of
    walkers within tol |E_loc|."""
    tol = ELOC_TOL[precision] if tol is None else tol
    eloc, ks, epot = np.asarray(eloc, np.float64), np.asarray(ks, np.float64), np.asarray(epot, np.float64)
    S = ks + np.abs(epot)
    err = np.abs(np.asarray(got, np.float64) - eloc)
    must = (ks > 1.05 * wf.refine_ratio * np.abs(eloc)) | (ks > 1.05 * wf.refine_ks)
    assert np.all(refined[must]), (ks / np.abs(eloc), refined)
    assert np.all(err <= tol * S), (np.max(err / S), int(np.argmax(err / S)), int(refined.sum()))
    # the forward Laplacian's two outputs on their own, where they do not cancel: near a node lap log psi and
    # |grad log psi|^2 both grow like 1 / d^2 with the distance d to the node while their sum stays finite, and a
    # rounding of psi that moves the node moves them in opposite directions
    calm = ks <= 8 * np.abs(eloc)
    if lap is not None:
        dl = np.abs(np.asarray(lap, np.float64) - lap_ref)
        assert np.all(dl[calm] <= 2 * tol * S[calm]), np.max(dl[calm] / S[calm])
    if grad is not None:
        dg = np.linalg.norm((np.asarray(grad, np.float64) - grad_ref).reshape(len(S), -1), axis=1)
        assert np.all(dg[calm] <= tol * np.sqrt(2 * S[calm])), np.max(dg[calm] / np.sqrt(2 * S[calm]))
    return float(np.mean(err <= tol * np.abs(eloc)))
