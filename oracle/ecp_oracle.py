"""CPU oracle of the reference's effective-core-potential terms -- TEST INFRASTRUCTURE ONLY.

Only ``tests/`` may import this module, as the checker; the product path never calls it.

Restated from the reference project (``src/sparse_wf/pseudopotentials.py``): the radial channel values on the
logarithmic grid (``eval_ecp`` 140-146, ``eval_ecp_on_grid`` 149-202), the local term (``make_local_pseudopotential``
205-219), the spherical quadrature grids (``make_spherical_grid`` 44-133), the integration points of the non-local
term (``build_all_integration_points`` 272-334) and the non-local term itself (``make_nonlocal_pseudopotential``
337-398) with its psi ratios from the low-rank update of a cached state, and the assembly of
``make_pseudopotential`` (411-457: effective charges, channel layout, cutoffs) and ``make_local_energy``
(``hamiltonian.py:49-83``).

Parity status: **parity unpinned**.  The element data (ccECP) come from pyscf's basis library
(``pyscf.gto.basis.load_ecp``), a dependency absent here, so the functions take the element data as an argument in
pyscf's layout: {Z: (n_core, [(l, [[(exponent, coefficient), ...] for the powers r^0, r^1, ...]), ...])}, l = -1 the
local channel.  The tests pin the algorithm by its properties (quadrature exactness, low-rank ratios equal to full
evaluations, interpolation against the closed form) on synthetic element data.  Random rotations of the quadrature
grids are inputs (jax.random cannot be reproduced here).
"""
from __future__ import annotations

import numpy as np

from . import fire_oracle as O

LOG_R0, LOG_RN, N_GRID = -5.0, 10.0, 10001  # eval_ecp_on_grid defaults (pseudopotentials.py:151-153)
CUTOFF_VALUE = 1e-7                         # make_pseudopotential's cutoff_value (pseudopotentials.py:417)


def radial_grid():
    """``jnp.logspace(log_r0, log_rn, n_grid)`` (pseudopotentials.py:187)."""
    return np.logspace(LOG_R0, LOG_RN, N_GRID)


def channel_values(r, terms):
    """``eval_ecp`` (pseudopotentials.py:140-146) divided by r^2 (:197): U(r) = r^-2 sum_n sum_k A_nk r^n
    exp(-B_nk r^2), terms[n] = [(B, A), ...]."""
    val = np.zeros_like(r, dtype=np.float64)
    for n, v in enumerate(terms):
        for b, a in v:
            val += a * r**n * np.exp(-b * r**2)
    return val / r**2


class Ecp:
    """``make_pseudopotential`` (pseudopotentials.py:411-457) for nuclei (Z, R) and element data in pyscf's layout.

    z_eff: effective charges (Z - n_core, 429); mask: the pseudised nuclei (431); v [n_ecp, max_channels, n_grid]:
    per pseudised nucleus its channels on the grid, row l for l >= 0 and the local channel in the last row (the
    index -1 of eval_ecp_on_grid, :195-198); cutoffs [n_ecp]: the grid radius of the last point where any non-local
    channel exceeds CUTOFF_VALUE in magnitude (:445-447); n_quad [n_ecp]: quadrature points per pseudised nucleus."""

    def __init__(self, Z, R, data, n_quad=None, default_points=12):
        Z = np.asarray(Z, np.int64)
        self.R = np.asarray(R, np.float64)
        self.grid = radial_grid()
        self.z_eff = np.array([z - data[z][0] if z in data else z for z in Z], np.float64)
        self.mask = np.abs(Z - self.z_eff) > 2e-6
        self.R_ecp = self.R[self.mask]
        max_ch = max(len(data[z][1]) for z in data)
        self.v = np.zeros((int(self.mask.sum()), max_ch, N_GRID))
        n_quad = n_quad or {}
        self.n_quad = np.zeros(int(self.mask.sum()), np.int64)
        for a, z in enumerate(Z[self.mask]):
            for l, terms in data[int(z)][1]:
                self.v[a, l] = channel_values(self.grid, terms)  # l = -1 lands in the last row
            self.n_quad[a] = n_quad.get(int(z), default_points)
        self.v_nonloc, self.v_loc = self.v[:, :-1], self.v[:, -1]
        above = np.abs(self.v_nonloc) > CUTOFF_VALUE
        self.cutoffs = self.grid[np.max(above * np.arange(N_GRID), axis=(1, 2))]


def local_term(ecp, r):
    """``make_local_pseudopotential`` (pseudopotentials.py:205-219): sum over electrons and pseudised nuclei of the
    local channel interpolated linearly on the grid (``jnp.interp``: clamped to the end values outside it)."""
    d = np.linalg.norm(r[:, None, :] - ecp.R_ecp[None], axis=-1)  # [n, n_ecp]
    return sum(np.interp(d[:, a], ecp.grid, ecp.v_loc[a]).sum() for a in range(len(ecp.R_ecp)))


def spherical_grid(n_points):
    """Quadrature points and weights on the unit sphere (``make_spherical_grid``, pseudopotentials.py:44-133): 1 and 2
    points, the tetrahedron (4, exact to degree 2), the octahedron (6, degree 3) and the icosahedron (12, degree 5),
    equal weights 1 / n.  The icosahedron's vertices are the cyclic permutations of (0, +-1, +-phi) / sqrt(1 + phi^2),
    phi the golden ratio, in the reference's order (rows (x, 0, -y), (y, -x, 0), ... with x = phi / sqrt(1 + phi^2),
    y = 1 / sqrt(1 + phi^2))."""
    def sph(tp):
        t, p = np.asarray(tp, np.float64).T
        return np.stack([np.sin(t) * np.cos(p), np.sin(t) * np.sin(p), np.cos(t)], -1)

    if n_points == 1:
        pts = sph([[0.0, 0.0]])
    elif n_points == 2:
        pts = sph([[0.0, 0.0], [np.pi, 0.0]])
    elif n_points == 4:
        a = np.arccos(-1.0 / 3.0)
        pts = sph([[0.0, 0.0], [a, 0.0], [a, 2 * np.pi / 3], [a, 4 * np.pi / 3]])
    elif n_points == 6:
        h = np.pi / 2
        pts = sph([[0.0, 0.0], [np.pi, 0.0], [h, 0.0], [h, h], [h, np.pi], [h, 3 * h]])
    elif n_points == 12:
        phi = (1.0 + np.sqrt(5.0)) / 2.0
        x, y = phi / np.sqrt(1.0 + phi**2), 1.0 / np.sqrt(1.0 + phi**2)
        pts = np.array([[x, 0, -y], [y, -x, 0], [0, -y, x], [x, 0, y], [-y, -x, 0], [0, y, -x], [-x, 0, -y],
                        [-y, x, 0], [0, y, x], [-x, 0, y], [y, x, 0], [0, -y, -x]], np.float64)
    else:
        raise ValueError(f"unsupported number of quadrature points: {n_points}")
    return pts, np.full(n_points, 1.0 / n_points)


def rotation(u):
    """``random_rot_mat`` (pseudopotentials.py:222-228) for two given normal draws u [2, 3]: Gram-Schmidt of the two
    vectors, their cross product third, as the columns of the matrix."""
    v1 = u[0] / np.linalg.norm(u[0])
    v2 = u[1] - v1 * np.dot(v1, u[1])
    v2 = v2 / np.linalg.norm(v2)
    return np.stack([v1, v2, np.cross(v1, v2)]).T


def legendre(x, l_max):
    """P_0 .. P_l_max (l_max <= 3) at x (``eval_leg0to3``, pseudopotentials.py:231-258): [..., l_max + 1]."""
    P = [np.ones_like(x), x, 0.5 * (3 * x**2 - 1), 0.5 * (5 * x**3 - 3 * x)]
    return np.stack(P[: l_max + 1], -1)


def integration_points(ecp, r, rot):
    """``build_all_integration_points`` (pseudopotentials.py:272-334) without the padding: for every electron i
    whose closest pseudised nucleus a lies within that nucleus's cutoff, the points R_a + |r_i - R_a| (g rot_i) of
    a's quadrature grid g, rot [n, 3, 3] one rotation per electron.  Returns a list of (i, a, r', w, cos theta)
    with cos theta the angle between the rotated point's direction and r_i - R_a."""
    out = []
    for i in range(r.shape[0]):
        d = np.linalg.norm(r[i] - ecp.R_ecp, axis=-1)
        a = int(np.argmin(d))
        if not d[a] < ecp.cutoffs[a]:
            continue
        u = (r[i] - ecp.R_ecp[a]) / d[a]
        g, w = spherical_grid(int(ecp.n_quad[a]))
        gr = g @ rot[i]  # einsum("ixy,gx->igy", rot_mat, grid)
        for k in range(len(g)):
            out.append((i, a, ecp.R_ecp[a] + d[a] * gr[k], w[k], float(gr[k] @ u)))
    return out


def nonlocal_term(prob, p, ecp, r, rot, ratio="low_rank"):
    """``make_nonlocal_pseudopotential`` (pseudopotentials.py:337-398): sum over the integration points of
    sum_l v_l(|r' - R_a|) w (2l + 1) P_l(cos theta) psi(r with r_i -> r') / psi(r), the ratio from the low-rank update
    of the cached state (``log_psi_low_rank_update``) or, with ratio="full", from two full evaluations."""
    (s0, l0), st = O.logpsi_with_state(prob, p, r)
    L = ecp.v_nonloc.shape[1]
    total = 0.0
    for i, a, rp, w, cos in integration_points(ecp, r, rot):
        rn = r.copy()
        rn[i] = rp
        if ratio == "low_rank":
            (s1, l1), _ = O.logpsi_low_rank_update(prob, p, rn, np.array([i]), st)
        else:
            s1, l1 = O.logpsi(prob, p, rn)
        psi_ratio = s1 * s0 * np.exp(l1 - l0)
        dist = np.linalg.norm(rp - ecp.R_ecp[a])
        v = np.array([np.interp(dist, ecp.grid, ecp.v_nonloc[a, l]) for l in range(L)])
        total += np.sum(v * w * psi_ratio * (2 * np.arange(L) + 1) * legendre(np.array(cos), L - 1))
    return total


def local_energy(prob, p, ecp, r, rot):
    """``make_local_energy`` (hamiltonian.py:49-83) with pseudopotentials: the kinetic energy, the Coulomb potential
    with the effective charges, the local and the non-local terms."""
    return (O.kinetic_energy(prob, p, r) + O.potential_energy(r, prob.R, ecp.z_eff) + local_term(ecp, r)
            + nonlocal_term(prob, p, ecp, r, rot))
