"""Effective core potentials: the tables ``fire_ecp_energy`` consumes, built on the host.

``make_pseudopotential`` (``src/sparse_wf/pseudopotentials.py:411-457``) loads each element's ccECP from pyscf's basis
library and tabulates its channels on a radial grid (``eval_ecp_on_grid``, 149-202).  pyscf is not a dependency of
this package: the element data are an argument in pyscf's layout, {Z: (n_core, [(l, [[(exponent, coefficient), ...]
for the powers r^0, r^1, ...]), ...])} with l = -1 the local channel, e.g. ``pyscf.gto.basis.load_ecp("ccecp", "C")``
where pyscf is installed.  The molecule the wavefunction sees has the effective charges ``EcpTables.z_eff`` (its
electrons are the valence electrons); ``fire_local_energy`` called with those charges gives the kinetic and Coulomb
terms, and ``FireWaveFunction.ecp_energy`` the pseudopotential terms.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np
import torch

from . import _lib

LOG_R0, LOG_RN, N_GRID = -5.0, 10.0, 10001  # eval_ecp_on_grid's grid: logspace(-5, 10, 10001)
CUTOFF_VALUE = 1e-7                         # make_pseudopotential's cutoff_value
QUAD_SIZES = (1, 2, 4, 6, 12)               # make_spherical_grid's supported sizes


def _channel(r: np.ndarray, terms) -> np.ndarray:
    """r^-2 sum_n sum_k A_nk r^n exp(-B_nk r^2) for terms[n] = [(B, A), ...] (eval_ecp, pseudopotentials.py:140-146)."""
    val = np.zeros_like(r)
    for power, pairs in enumerate(terms):
        for b, a in pairs:
            val += a * r**power * np.exp(-b * r**2)
    return val / r**2


class EcpTables:
    """The pseudised nuclei of a molecule and their channels on the radial grid.

    Z: the nuclear charges; data: element data in pyscf's layout for the pseudised elements; n_quad: quadrature points
    per element ({Z: n}, default ``default_points``; the reference's defaults are 4 for C-Ne, 6 for Na-Ar, 12
    otherwise, ``config/default.yaml``).  Attributes: z_eff (Z - n_core), atom (indices of the pseudised nuclei),
    grid, v_loc [n_ecp, n_grid], v_nl [n_ecp, n_l, n_grid] (n_l = the largest channel count less the local one),
    cutoffs (the last grid radius where a non-local channel exceeds 1e-7 in magnitude), n_quad."""

    def __init__(self, Z, data: dict, n_quad: Optional[dict] = None, default_points: int = 12):
        Z = np.asarray(Z, np.int64)
        self.z_eff = np.array([z - data[int(z)][0] if int(z) in data else z for z in Z], np.int64)
        self.atom = np.nonzero(self.z_eff != Z)[0].astype(np.int32)
        if len(self.atom) == 0:
            raise ValueError("no nucleus of the molecule is pseudised by the given element data")
        self.grid = np.logspace(LOG_R0, LOG_RN, N_GRID)
        channels = max(len(data[int(z)][1]) for z in Z[self.atom])
        v = np.zeros((len(self.atom), channels, N_GRID))
        n_quad = n_quad or {}
        self.n_quad = np.zeros(len(self.atom), np.int32)
        for a, z in enumerate(Z[self.atom]):
            for l, terms in data[int(z)][1]:
                v[a, l] = _channel(self.grid, terms)  # l = -1: the last row
            self.n_quad[a] = n_quad.get(int(z), default_points)
        if not set(self.n_quad.tolist()) <= set(QUAD_SIZES):
            raise ValueError(f"quadrature sizes must be among {QUAD_SIZES}")
        self.v_loc = np.ascontiguousarray(v[:, -1])
        self.v_nl = np.ascontiguousarray(v[:, :-1])
        if self.v_nl.shape[1] > 4:
            raise ValueError("non-local channels beyond l = 3 are not supported (pseudopotentials.py:346)")
        above = np.abs(self.v_nl) > CUTOFF_VALUE
        last = np.max(above * np.arange(N_GRID), axis=(1, 2)) if self.v_nl.shape[1] else np.zeros(len(self.atom), int)
        self.cutoffs = self.grid[last]

    def device(self, device) -> "DeviceEcp":
        return DeviceEcp(self, device)


class DeviceEcp:
    """The tables on the device and the ``fire_ecp`` struct pointing at them."""

    def __init__(self, t: EcpTables, device):
        dev = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a)).to(device=device, dtype=dt)  # noqa: E731
        self.atom = dev(t.atom, torch.int32)
        self.grid = dev(t.grid, torch.float64)
        self.v_loc = dev(t.v_loc, torch.float64)
        self.v_nl = dev(t.v_nl if t.v_nl.size else np.zeros(1), torch.float64)
        self.cutoff = dev(t.cutoffs, torch.float64)
        self.n_quad = dev(t.n_quad, torch.int32)
        self.struct = _lib.Ecp(len(t.atom), len(t.grid), t.v_nl.shape[1], int(t.n_quad.max()),
                               C.c_void_p(self.atom.data_ptr()), C.c_void_p(self.grid.data_ptr()),
                               C.c_void_p(self.v_loc.data_ptr()), C.c_void_p(self.v_nl.data_ptr()),
                               C.c_void_p(self.cutoff.data_ptr()), C.c_void_p(self.n_quad.data_ptr()))
