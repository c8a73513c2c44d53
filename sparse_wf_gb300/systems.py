"""Synthetic molecules and walker initialisation.

The reference builds molecules with pyscf (``system.py``) and draws the first
walkers with ``init_electrons`` (``src/sparse_wf/mcmc.py:431-465``) after a
greedy anti-ferromagnetic spin assignment (``mcmc.py:381-428``).  pyscf is not
part of this package, so the two systems the benchmarks use are generated here:

* a linear hydrogen chain on the x axis;
* an all-trans alkane CnH2n+2 with a planar zig-zag carbon backbone
  (C-C 2.91 bohr, C-H 2.06 bohr, tetrahedral angles).

Electrons are ordered the reference's way: all spin-up electrons first, grouped
by the atom they were placed on, then all spin-down electrons.
"""
from __future__ import annotations

import dataclasses

import numpy as np

TETRA = np.arccos(-1.0 / 3.0)  # 109.47 degrees
C_C = 2.91
C_H = 2.06


@dataclasses.dataclass(frozen=True)
class Molecule:
    name: str
    R: np.ndarray  # [n_nuc, 3] float32 (the reference keeps nuclei in float32)
    Z: np.ndarray  # [n_nuc] int

    @property
    def n_nuc(self) -> int:
        return int(len(self.Z))

    @property
    def n_el(self) -> int:
        return int(np.sum(self.Z))

    @property
    def n_up(self) -> int:
        # neutral closed-shell-or-doublet convention of pyscf: n_up = ceil(n/2)
        return (self.n_el + 1) // 2


def hydrogen_chain(n: int = 10, spacing: float = 1.8) -> Molecule:
    R = np.zeros((n, 3), np.float64)
    R[:, 0] = np.arange(n) * spacing
    return Molecule(f"H{n}", R.astype(np.float32), np.ones(n, np.int64))


def alkane(n_carbon: int) -> Molecule:
    """All-trans CnH2n+2 in the xy plane (carbons), hydrogens tetrahedral."""
    if n_carbon < 1:
        raise ValueError("n_carbon must be >= 1")
    half = TETRA / 2.0
    carbons = np.zeros((n_carbon, 3))
    for k in range(n_carbon):
        carbons[k, 0] = k * C_C * np.sin(half)
        carbons[k, 1] = (k % 2) * C_C * np.cos(half)
    hydrogens = []
    z = np.array([0.0, 0.0, 1.0])
    if n_carbon == 1:
        dirs = np.array([[1, 1, 1], [1, -1, -1], [-1, 1, -1], [-1, -1, 1]], float) / np.sqrt(3.0)
        hydrogens = [carbons[0] + C_H * d for d in dirs]
    else:
        for k in range(n_carbon):
            c = carbons[k]
            if 0 < k < n_carbon - 1:
                b = (carbons[k - 1] - c) + (carbons[k + 1] - c)
                b = -b / np.linalg.norm(b)
                for s in (1.0, -1.0):
                    hydrogens.append(c + C_H * (np.cos(half) * b + s * np.sin(half) * z))
            else:
                nb = carbons[1] if k == 0 else carbons[k - 1]
                u = c - nb
                u /= np.linalg.norm(u)
                # in-plane perpendicular to u, chosen so the in-plane H continues the zig-zag (trans)
                p = np.cross(z, u)
                other = carbons[2] if (k == 0 and n_carbon > 2) else (carbons[k - 2] if n_carbon > 2 else c + p)
                if np.dot(other - nb, p) > 0:
                    p = -p
                hydrogens.append(c + C_H * (u / 3.0 + (2.0 * np.sqrt(2.0) / 3.0) * p))
                for s in (1.0, -1.0):
                    hydrogens.append(
                        c + C_H * (u / 3.0 - (np.sqrt(2.0) / 3.0) * p + s * np.sqrt(2.0 / 3.0) * z)
                    )
    R = np.concatenate([carbons, np.array(hydrogens)], axis=0)
    Z = np.concatenate([np.full(n_carbon, 6), np.ones(len(hydrogens), int)])
    return Molecule(f"C{n_carbon}H{2 * n_carbon + 2}", R.astype(np.float32), Z.astype(np.int64))


def assign_spins_to_atoms(R: np.ndarray, Z: np.ndarray) -> np.ndarray:
    """Atom index of every electron, spin-up electrons first.

    Restates ``assign_spins_to_atoms`` (``src/sparse_wf/mcmc.py:381-428``):
    Z//2 up electrons per atom, the remaining electrons of odd-Z atoms are
    assigned greedily so that spins on nearby open-shell atoms anti-align.
    """
    R = np.asarray(R, np.float64)
    Z = np.asarray(Z, np.int64)
    n_el = int(np.sum(Z))
    n_up_per_atom = Z // 2
    n_rem = n_el - 2 * int(np.sum(n_up_per_atom))
    if n_rem > 0:
        open_idx = np.where(Z % 2)[0]
        R_open = R[open_idx]
        dist = np.linalg.norm(R_open[:, None, :] - R_open[None, :, :], axis=-1)
        kernel = np.exp(-dist * 0.5)
        spins = np.zeros(n_rem)
        n_dn_left = n_rem // 2
        n_up_left = n_rem - n_dn_left
        for _ in range(n_rem):
            is_free = spins == 0
            spin_per_site = kernel[is_free, :] @ spins
            ind_atom = np.arange(n_rem)[is_free]
            loss_up = spin_per_site
            loss_dn = -spin_per_site
            if (n_up_left > 0) and (np.min(loss_up) < np.min(loss_dn)):
                spins[ind_atom[np.argmin(loss_up)]] = 1
                n_up_left -= 1
            else:
                spins[ind_atom[np.argmin(loss_dn)]] = -1
                n_dn_left -= 1
        n_up_per_atom = n_up_per_atom.copy()
        n_up_per_atom[open_idx] += (spins == 1).astype(np.int64)
    n_dn_per_atom = Z - n_up_per_atom
    ind = []
    for i, k in enumerate(n_up_per_atom):
        ind += [i] * int(k)
    for i, k in enumerate(n_dn_per_atom):
        ind += [i] * int(k)
    return np.array(ind, np.int64)


def init_electrons(mol: Molecule, n_walkers: int, seed: int, stddev: float = 1.0) -> np.ndarray:
    """Walkers [B, n_el, 3] float32: electron k ~ N(R[atom(k)], stddev^2).

    Follows ``init_electrons`` (``src/sparse_wf/mcmc.py:431-465``) for a neutral
    molecule; the Gaussian draws come from numpy's PCG64 with ``seed``.
    """
    rng = np.random.default_rng(seed)
    r = rng.standard_normal((n_walkers, mol.n_el, 3)).astype(np.float32) * np.float32(stddev)
    if mol.n_nuc > 1:
        ind = assign_spins_to_atoms(mol.R, mol.Z)
        r = r + mol.R[ind][None].astype(np.float32)
    else:
        r = r + mol.R[0][None, None].astype(np.float32)
    return r.astype(np.float32)


def spin_counts(mol: Molecule) -> tuple[int, int]:
    """(n_up, n_dn) implied by the spin assignment (equal to pyscf's for neutral molecules)."""
    n_up = int(np.sum(mol.Z // 2))
    n_rem = mol.n_el - 2 * n_up
    n_up += n_rem - n_rem // 2
    return n_up, mol.n_el - n_up
