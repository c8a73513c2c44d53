"""Generates the golden fixtures of the parity tests from the oracle (``oracle/fire_oracle.py``).

Run from the repository root:  python tests/golden/make_golden.py
Each fixture holds the molecule, float32 walkers, the parameter seed and the oracle's FP64 outputs:
neighbour lists in the reference's padded format, triplets, log|psi|, sign, kinetic/potential/local
energies and an MCMC replay block.  Parameters are not stored: ``make_params`` regenerates them from the
seed (tests/test_oracle.py checks the oracle against these vectors on the machine that made them).
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import fire_oracle as O  # noqa: E402
from sparse_wf_gb300 import params as P, systems  # noqa: E402

OUT = Path(__file__).resolve().parent


def make_params(mol, nu, r0, seed=0, activate=True):
    dims = P.ModelDims(mol.n_el, nu, mol.n_nuc)
    p = P.init_params(dims, seed)
    if activate:
        p = P.activate_jastrow(p)
    blob, offs = P.pack_params(dims, p, np.float32)
    p = P.unpack_params(dims, blob, offs)
    prob = O.Problem(mol.R, mol.Z, nu)
    hc, _ = O.embedding_value(prob, p, r0.astype(np.float64), return_pre_scale=True)
    p["scales"] = np.array([1.0 / np.std(hc), 1.0])
    _, hu = O.embedding_value(prob, p, r0.astype(np.float64), return_pre_scale=True)
    p["scales"][1] = 1.0 / np.std(hu)
    blob, offs = P.pack_params(dims, p, np.float32)
    return dims, P.unpack_params(dims, blob, offs), blob, offs


def fixture(name, mol, n_walkers, seed, activate=True, triplets=True, mcmc_steps=0):
    nu, _ = systems.spin_counts(mol)
    r = systems.init_electrons(mol, n_walkers, 1000 + seed)
    dims, p, blob, offs = make_params(mol, nu, r[0], activate=activate)
    prob = O.Problem(mol.R, mol.Z, nu)
    out = dict(R=mol.R, Z=mol.Z, n_up=nu, r=r, param_seed=0, activate=activate, cutoff=5.0, cutoff_1el=20.0,
               blob_sum=np.float64(np.sum(blob.astype(np.float64))))
    counts = np.array([O.static_counts(w, mol.R, nu, 5.0, 20.0) for w in r])
    out["counts"] = counts
    cs, cd = counts[:, 0].max() + 3, counts[:, 1].max() + 2  # padded capacities
    ne = counts[:, 3].max() + 1
    lists = {k: [] for k in ("ct_same", "nb_same", "jac_same", "ct_diff", "nb_diff", "jac_diff", "jac_ctr",
                             "jac_dep", "en_idx")}
    for w in r:
        (a, b, c), (d, e, f), (g, h) = O.pair_indices(w, nu, 5.0, cs, cd)
        for k, v in zip(("ct_same", "nb_same", "jac_same", "ct_diff", "nb_diff", "jac_diff", "jac_ctr", "jac_dep"),
                        (a, b, c, d, e, f, g, h)):
            lists[k].append(v)
        lists["en_idx"].append(O.neighbouring_nuclei(w, mol.R, 20.0, ne))
    for k, v in lists.items():
        out["nl_" + k] = np.array(v, np.int32)
    out["cap_same"], out["cap_diff"], out["cap_nuc"] = cs, cd, ne
    if triplets:
        trip = []
        for w in r:
            (_, _, _), (_, _, _), (g, h) = O.pair_indices(w, nu, 5.0)
            nt = O.static_counts(w, mol.R, nu, 5.0, 20.0)[2]
            trip.append(np.stack(O.triplet_indices(g, h, mol.n_el, nt)))
        tcap = max(t.shape[1] for t in trip)
        out["triplets"] = np.array([np.pad(t, ((0, 0), (0, tcap - t.shape[1])), constant_values=O.NO_NEIGHBOUR)
                                    for t in trip], np.int32)
    r64 = r.astype(np.float64)
    hc = np.array([O.embedding_value(prob, p, w, return_pre_scale=True)[0] for w in r64])
    out["h_contract_norm"] = np.linalg.norm(hc.reshape(n_walkers, -1), axis=1)
    lp = np.array([O.logpsi(prob, p, w) for w in r64])
    out["sign"], out["logpsi"] = lp[:, 0], lp[:, 1]
    fl = [O.logpsi_fl(prob, p, w) for w in r64]
    out["grad"] = np.array([x[1] for x in fl]).reshape(n_walkers, mol.n_el, 3)
    out["lap"] = np.array([x[2] for x in fl])
    out["ekin"] = np.array([-0.5 * (x[2] + x[1] @ x[1]) for x in fl])
    out["epot"] = np.array([O.potential_energy(w, mol.R, mol.Z) for w in r64])
    out["eloc"] = out["ekin"] + out["epot"]
    if mcmc_steps:
        rng = np.random.default_rng(77 + seed)
        noise = rng.standard_normal((mcmc_steps, n_walkers, mol.n_el, 3)).astype(np.float32)
        logu = np.log(rng.uniform(size=(mcmc_steps, n_walkers))).astype(np.float32)
        rs, margins, nacc = [], [], []
        for k in range(n_walkers):
            rr, _, na, mg = O.mcmc_block(prob, p, r64[k], noise[:, k].astype(np.float64), logu[:, k].astype(np.float64),
                                         np.float32(0.1))
            rs.append(rr)
            margins.append(mg)
            nacc.append(na)
        out.update(mcmc_noise=noise, mcmc_logu=logu, mcmc_width=0.1, mcmc_r=np.array(rs), mcmc_margin=np.array(margins),
                   mcmc_nacc=np.array(nacc))
    np.savez_compressed(OUT / f"{name}.npz", **out)
    print(name, {k: np.asarray(v).shape for k, v in out.items() if k in ("r", "eloc", "triplets")})


if __name__ == "__main__":
    fixture("h10", systems.hydrogen_chain(10, 1.8), 8, 0, mcmc_steps=5)
    fixture("h10_plain", systems.hydrogen_chain(10, 1.8), 4, 1, activate=False)
    fixture("c2h6", systems.alkane(2), 4, 2, mcmc_steps=3)
    fixture("c10h22", systems.alkane(10), 2, 3, triplets=False)
