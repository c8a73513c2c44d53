"""The oracle of the reference's effective-core-potential terms (src/sparse_wf/pseudopotentials.py) pinned by its
properties: the quadrature grids' exactness on Legendre polynomials, the integration-point geometry, the radial
interpolation against the closed form, and psi ratios from the low-rank update equal to full evaluations.  The element
data are synthetic (pyscf's ccECP tables are not available here), in pyscf's layout."""
import numpy as np
import pytest

from oracle import ecp_oracle as E
from oracle import fire_oracle as O
from sparse_wf_gb300 import params as P, systems

# carbon with 2 core electrons: a local channel (l = -1) and s / p channels, terms per power of r as (B, A)
CARBON = (2, [(-1, [[], [(14.0, 4.0)], [(8.0, 50.0)], [(13.0, -25.0)]]),
              (0, [[], [], [(7.0, 50.0)]]),
              (1, [[], [], [(6.0, -10.0)]])])


def _ecp_case(seed=0):
    mol = systems.alkane(2)
    ecp = E.Ecp(mol.Z, mol.R, {6: CARBON}, n_quad={6: 4}, default_points=12)
    val = systems.Molecule("C2H6-valence", mol.R, ecp.z_eff.astype(np.int64))
    nu, _ = systems.spin_counts(val)
    r = systems.init_electrons(val, 2, 77 + seed).astype(np.float64)
    dims = P.ModelDims(val.n_el, nu, val.n_nuc)
    p = P.init_params(dims, seed)
    p = P.activate_jastrow(p)
    blob, offs = P.pack_params(dims, p, np.float32)
    p = P.unpack_params(dims, blob, offs)
    prob = O.Problem(val.R, val.Z, nu)
    hc, _ = O.embedding_value(prob, p, r[0], return_pre_scale=True)
    p["scales"] = np.array([1.0 / np.std(hc), 1.0])
    _, hu = O.embedding_value(prob, p, r[0], return_pre_scale=True)
    p["scales"][1] = 1.0 / np.std(hu)
    return mol, val, ecp, prob, p, r


@pytest.mark.parametrize("n_points, degree", [(4, 2), (6, 3), (12, 3)])
def test_spherical_designs_integrate_legendre_polynomials(n_points, degree):
    """make_spherical_grid (pseudopotentials.py:44-133): unit vectors with weights 1 / n whose average of P_l(g . u)
    is delta_l0 for every direction u up to the design's degree (tetrahedron 2, octahedron 3, icosahedron 5; the
    non-local term uses l <= 3) -- the angular integral the non-local term needs -- whatever the rotation."""
    g, w = E.spherical_grid(n_points)
    np.testing.assert_allclose(np.linalg.norm(g, axis=1), 1.0, atol=1e-15)
    assert abs(w.sum() - 1.0) < 1e-15
    rng = np.random.default_rng(n_points)
    for _ in range(5):
        rot = E.rotation(rng.standard_normal((2, 3)))
        np.testing.assert_allclose(rot.T @ rot, np.eye(3), atol=1e-14)
        u = rng.standard_normal(3)
        u /= np.linalg.norm(u)
        avg = (w[:, None] * E.legendre((g @ rot) @ u, degree)).sum(0)
        np.testing.assert_allclose(avg, np.eye(degree + 1)[0], atol=1e-14)


def test_channels_cutoffs_and_local_term():
    """eval_ecp_on_grid / make_pseudopotential / make_local_pseudopotential: effective charges Z - n_core on the
    pseudised nuclei only, the local channel in the last row, the non-local cutoff where the channels fall below
    1e-7, and the local term within 1e-4 of the closed form (linear interpolation on the 10001-point logarithmic grid,
    points 10^(15/10000) apart: ~1e-5 on this steep local channel)."""
    mol, val, ecp, prob, p, r = _ecp_case()
    np.testing.assert_array_equal(ecp.z_eff, [4, 4, 1, 1, 1, 1, 1, 1])
    np.testing.assert_array_equal(ecp.mask, [True, True] + [False] * 6)
    assert ecp.v.shape == (2, 3, E.N_GRID)
    np.testing.assert_allclose(ecp.v_loc[0], E.channel_values(ecp.grid, CARBON[1][0][1]))
    c = ecp.cutoffs[0]
    assert 1.0 < c < 10.0 and np.all(np.abs(ecp.v_nonloc[0][:, ecp.grid > c]) <= E.CUTOFF_VALUE)
    for w in r:
        d = np.linalg.norm(w[:, None] - ecp.R_ecp[None], axis=-1)
        exact = E.channel_values(d, CARBON[1][0][1]).sum()
        assert abs(E.local_term(ecp, w) - exact) <= 1e-4 * max(1.0, abs(exact))


def test_integration_points_geometry():
    """build_all_integration_points (pseudopotentials.py:272-334): electrons within the cutoff of their closest
    pseudised nucleus get that nucleus's grid (4 points for carbon here), rotated and scaled to the electron's
    distance; cos theta is the angle to the electron's direction."""
    mol, val, ecp, prob, p, r = _ecp_case()
    rng = np.random.default_rng(3)
    w = r[0]
    rot = np.stack([E.rotation(rng.standard_normal((2, 3))) for _ in range(val.n_el)])
    pts = E.integration_points(ecp, w, rot)
    active = {i for i, *_ in pts}
    for i in range(val.n_el):
        d = np.linalg.norm(w[i] - ecp.R_ecp, axis=-1)
        assert (i in active) == (d.min() < ecp.cutoffs[int(np.argmin(d))])
    assert len(pts) == 4 * len(active) and active
    for i, a, rp, wt, cos in pts:
        d = np.linalg.norm(w[i] - ecp.R_ecp[a])
        assert abs(np.linalg.norm(rp - ecp.R_ecp[a]) - d) < 1e-12
        assert abs(cos - (rp - ecp.R_ecp[a]) @ (w[i] - ecp.R_ecp[a]) / d**2) < 1e-12
        assert wt == 0.25


def test_nonlocal_term_low_rank_ratios_equal_full_evaluations():
    """make_nonlocal_pseudopotential (pseudopotentials.py:337-398) takes psi(r_i -> r') / psi(r) from the low-rank
    update of the cached state (log_psi_low_rank_update); the same sum with two full evaluations per point agrees to
    1e-10, and the local energy with pseudopotentials is finite."""
    mol, val, ecp, prob, p, r = _ecp_case()
    rng = np.random.default_rng(5)
    w = r[1]
    rot = np.stack([E.rotation(rng.standard_normal((2, 3))) for _ in range(val.n_el)])
    a = E.nonlocal_term(prob, p, ecp, w, rot)
    b = E.nonlocal_term(prob, p, ecp, w, rot, ratio="full")
    assert a != 0.0
    assert abs(a - b) <= 1e-10 * max(1.0, abs(b))
    assert np.isfinite(E.local_energy(prob, p, ecp, w, rot))


def test_product_tables_match_the_oracle():
    """sparse_wf_gb300.ecp.EcpTables (the host tables fire_ecp_energy consumes) against the oracle's restatement of
    make_pseudopotential: effective charges, pseudised nuclei, grid, local and non-local channels, cutoffs and
    quadrature sizes."""
    from sparse_wf_gb300.ecp import EcpTables

    mol = systems.alkane(2)
    ref = E.Ecp(mol.Z, mol.R, {6: CARBON}, n_quad={6: 4})
    t = EcpTables(mol.Z, {6: CARBON}, n_quad={6: 4})
    np.testing.assert_array_equal(t.z_eff, ref.z_eff)
    np.testing.assert_array_equal(t.atom, np.nonzero(ref.mask)[0])
    np.testing.assert_array_equal(t.grid, ref.grid)
    np.testing.assert_allclose(t.v_loc, ref.v_loc, rtol=1e-15, atol=0)
    np.testing.assert_allclose(t.v_nl, ref.v_nonloc, rtol=1e-15, atol=0)
    np.testing.assert_array_equal(t.cutoffs, ref.cutoffs)
    np.testing.assert_array_equal(t.n_quad, ref.n_quad)
    with pytest.raises(ValueError):
        EcpTables(mol.Z, {6: CARBON}, n_quad={6: 5})


@pytest.mark.parametrize("n_points", [1, 2, 4, 6, 12])
def test_device_quadrature_table_matches_the_oracle(n_points):
    """The quadrature table fire_ecp_energy uses (fire_ecp_quadrature, host only) equals the oracle's grids to
    rounding, point for point."""
    import ctypes as C

    from sparse_wf_gb300 import _lib
    from sparse_wf_gb300.build import build

    build()
    lib = _lib.load()
    out = (C.c_double * (3 * n_points))()
    assert lib.fire_ecp_quadrature(n_points, out) == 0
    got = np.array(out[:]).reshape(n_points, 3)
    np.testing.assert_allclose(got, E.spherical_grid(n_points)[0], rtol=0, atol=1e-15)
    assert lib.fire_ecp_quadrature(5, out) == 1
