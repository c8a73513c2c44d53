"""The oracle (CPU restatement of the reference) against its golden vectors and against finite
differences of its own value path -- the reference's own consistency check (sparse forward
Laplacian vs dense Laplacian, tests/test_fwd_lap.py:100-118 of the reference)."""
import numpy as np
import pytest

from helpers import case, golden, rel
from oracle import fire_oracle as O


@pytest.mark.parametrize("name", ["h10", "h10_plain", "c2h6", "c10h22"])
def test_oracle_golden(name):
    g = golden(name)
    mol, nu, r, p, blob, _ = case(name)
    if abs(float(np.sum(blob.astype(np.float64))) - float(g["blob_sum"])) > 1e-6 * abs(float(g["blob_sum"])):
        pytest.skip("parameter initialiser differs on this platform (special-function rounding)")
    prob = O.Problem(mol.R, mol.Z, nu)
    for k in range(min(2, len(r))):
        w = r[k].astype(np.float64)
        s, l = O.logpsi(prob, p, w)
        assert s == g["sign"][k]
        assert abs(l - g["logpsi"][k]) <= 1e-10 * max(1.0, abs(g["logpsi"][k]))
        e = O.local_energy(prob, p, w)
        assert abs(e - g["eloc"][k]) <= 1e-9 * max(1.0, abs(g["eloc"][k]))


@pytest.mark.parametrize("name", ["h10", "c2h6", "c10h22"])
def test_neighbour_lists_golden(name):
    g = golden(name)
    mol, nu, r, *_ = case(name)
    for k, w in enumerate(r):
        (a, b, c), (d, e, f), (gg, h) = O.pair_indices(w, nu, 5.0, int(g["cap_same"]), int(g["cap_diff"]))
        for key, v in zip(("ct_same", "nb_same", "jac_same", "ct_diff", "nb_diff", "jac_diff", "jac_ctr", "jac_dep"),
                          (a, b, c, d, e, f, gg, h)):
            np.testing.assert_array_equal(v, g["nl_" + key][k])
        np.testing.assert_array_equal(O.neighbouring_nuclei(w, mol.R, 20.0, int(g["cap_nuc"])), g["nl_en_idx"][k])
        assert tuple(O.static_counts(w, mol.R, nu, 5.0, 20.0)) == tuple(g["counts"][k])


def test_pair_list_structure():
    mol, nu, r, *_ = case("c10h22")
    w = r[0]
    (cs, ns, js), (cd, nd, jd), (jc, jdp) = O.pair_indices(w, nu, 5.0)
    n = mol.n_el
    P = len(jc) - n
    keys = jc[n:] * n + jdp[n:]
    assert np.all(np.diff(keys) > 0), "combined list is row-major sorted"
    pairs = set(zip(jc[n:].tolist(), jdp[n:].tolist()))
    assert all((j, i) in pairs for i, j in pairs), "cutoff relation is symmetric"
    np.testing.assert_array_equal(jc[js], cs)
    np.testing.assert_array_equal(jdp[jd], nd)
    assert np.all((cs < nu) == (ns < nu)) and np.all((cd < nu) != (nd < nu))
    nt = O.static_counts(w, mol.R, nu, 5.0, 20.0)[2]
    t = O.triplet_indices(jc, jdp, n, nt)
    assert len(t[0]) == n + 2 * P + nt
    # every triplet row pair (in, kn) shares the dependency, centers are (i, k)
    t_in, t_k, t_kn, t_i = t
    np.testing.assert_array_equal(jdp[t_in], jdp[t_kn])
    np.testing.assert_array_equal(jc[t_in], t_i)
    np.testing.assert_array_equal(jc[t_kn], t_k)


def _fd(f, x0, h):
    y0 = f(x0)
    G = np.zeros((len(x0),) + np.shape(y0))
    L = np.zeros_like(y0)
    for k in range(len(x0)):
        e = np.zeros_like(x0)
        e[k] = h
        fp, fm, fp2, fm2 = f(x0 + e), f(x0 - e), f(x0 + 2 * e), f(x0 - 2 * e)
        G[k] = (8 * (fp - fm) - (fp2 - fm2)) / (12 * h)
        L = L + (-fp2 + 16 * fp - 30 * y0 + 16 * fm - fm2) / (12 * h * h)
    return y0, G, L


def test_sparse_fwd_lap_matches_dense_energy():
    """Sparse forward-Laplacian kinetic energy == finite-difference Laplacian of log|psi| (FP64)."""
    mol, nu, r, p, *_ = case("h10")
    prob = O.Problem(mol.R, mol.Z, nu)
    w = r[1].astype(np.float64)
    v, j, l = O.logpsi_fl(prob, p, w)
    y0, G, L = _fd(lambda x: O.logpsi(prob, p, x.reshape(-1, 3))[1], w.reshape(-1), 2e-4)
    assert abs(v - y0) < 1e-12 * abs(y0)
    np.testing.assert_allclose(j, G, rtol=1e-6, atol=1e-6 * np.abs(G).max())
    ek, ek_fd = -0.5 * (l + j @ j), -0.5 * (L + G @ G)
    assert rel(ek, ek_fd) < 1e-5


def test_sparse_fwd_lap_matches_dense_embedding():
    """Embedding value/Jacobian/Laplacian vs finite differences (reference test_embedding)."""
    mol, nu, r, p, *_ = case("c2h6")
    prob = O.Problem(mol.R, mol.Z, nu)
    w = r[0].astype(np.float64)
    h = O.embedding_fl(prob, p, w)
    y0, G, L = _fd(lambda x: O.embedding_value(prob, p, x.reshape(-1, 3)), w.reshape(-1), 1e-3)
    n = mol.n_el
    J = np.zeros((n, 3) + h.x.shape)
    for row, (c, d) in enumerate(zip(h.idx_ctr, h.idx_dep)):
        J[d, :, c] += h.jac[row]
    J = J.reshape((3 * n,) + h.x.shape)
    assert np.linalg.norm(h.x - y0) / np.linalg.norm(y0) < 1e-12
    assert np.linalg.norm(J - G) / np.linalg.norm(G) < 1e-8
    assert np.linalg.norm(h.lap - L) / np.linalg.norm(L) < 1e-6


def test_potential_energy_h2():
    R = np.array([[0.0, 0, 0], [1.4, 0, 0]])
    Z = np.array([1.0, 1.0])
    r = np.array([[0.0, 0.5, 0.0], [1.4, -0.5, 0.0]])
    d12 = np.linalg.norm(r[0] - r[1])
    ref = 1 / d12 - (1 / 0.5 + 1 / np.linalg.norm(r[0] - R[1]) + 1 / np.linalg.norm(r[1] - R[0]) + 1 / 0.5) + 1 / 1.4
    assert abs(O.potential_energy(r, R, Z) - ref) < 1e-12


def test_mcmc_block_replay_golden():
    g = golden("h10")
    mol, nu, r, p, *_ = case("h10")
    prob = O.Problem(mol.R, mol.Z, nu)
    k = 0
    rr, _, na, mg = O.mcmc_block(prob, p, r[k].astype(np.float64), g["mcmc_noise"][:, k].astype(np.float64),
                                 g["mcmc_logu"][:, k].astype(np.float64), np.float32(0.1))
    np.testing.assert_allclose(rr, g["mcmc_r"][k], atol=1e-12)
    assert na == g["mcmc_nacc"][k]


def test_single_electron_block_is_the_all_electron_block_with_one_electron_moved():
    """mcmc_single_block (proposal_single_electron, mcmc.py:100-111) equals mcmc_block fed noise that is zero on every
    electron but (offset + s) mod n at step s, decisions and positions included."""
    mol, nu, r, p, *_ = case("h10")
    prob = O.Problem(mol.R, mol.Z, nu)
    rng = np.random.default_rng(5)
    steps, n, off = 7, mol.n_el, 6
    eps = rng.standard_normal((steps, 3))
    logu = np.log(rng.uniform(size=steps))
    full = np.zeros((steps, n, 3))
    for s in range(steps):
        full[s, (off + s) % n] = eps[s]
    r0 = r[1].astype(np.float64)
    a = O.mcmc_single_block(prob, p, r0, eps, logu, 0.3, offset=off)
    b = O.mcmc_block(prob, p, r0, full, logu, 0.3)
    np.testing.assert_array_equal(a[0], b[0])
    assert a[2] == b[2] and 0 < a[2] < steps
    np.testing.assert_allclose(a[3], b[3], rtol=0, atol=0)


def test_jump_proposal_draw_mapping_and_log_ratio():
    """proposal_jump_to_atom (mcmc.py:164-193): the electron and nucleus come from the two uniforms (nucleus by
    cumulative charge), only that electron moves, to R_I + sigma eps, and the log ratio is log q(old) - log q(new)
    with q(x) = sum_J Z_J exp(-|x - R_J|^2 / (2 sigma^2)) (the reference's weights Z / sum Z cancel)."""
    R = np.array([[0.0, 0.0, 0.0], [2.0, 0.0, 0.0], [0.0, 3.0, 0.0]])
    Z = np.array([6.0, 1.0, 1.0])
    r = np.random.default_rng(3).standard_normal((5, 3))
    sigma = 2.0
    for d, e, I in (([0.0, 0.1, 0.5, -0.2, 0.3], 0, 0), ([0.99, 0.8, 0.0, 0.0, 0.0], 4, 1),
                    ([0.41, 0.95, 1.0, 1.0, -1.0], 2, 2)):
        rn, plr = O.jump_proposal(R, Z, r, np.array(d), sigma)
        moved = np.any(rn != r, axis=1)
        assert moved.sum() == 1 and moved[e]
        np.testing.assert_allclose(rn[e], R[I] + sigma * np.array(d[2:]), atol=1e-15)
        q = lambda x: np.sum(Z * np.exp(-np.sum((x - R) ** 2, axis=1) / (2 * sigma**2)))
        assert abs(plr - (np.log(q(r[e])) - np.log(q(rn[e])))) < 1e-12


def test_cluster_proposal_semantics():
    """proposal_cluster_update (mcmc.py:119-161): the k closest electrons within the radius move (noise row i to the
    i-th closest), a draw that changes the cluster around the moved center is skipped, none valid gives log 0."""
    r = np.array([[0.0, 0, 0], [0.5, 0, 0], [1.0, 0, 0], [5.0, 0, 0], [0.0, 1.5, 0]])
    idx = O.closest_k(np.linalg.norm(r - r[0], axis=-1), 1.2, 3)
    np.testing.assert_array_equal(idx, [0, 1, 2])
    idx = O.closest_k(np.linalg.norm(r - r[0], axis=-1), 0.7, 3)
    np.testing.assert_array_equal(idx, [0, 1, O.NO_NEIGHBOUR])
    k, width = 3, 1.0
    eps = np.zeros((5, k, 3))
    eps[0, 2] = [10.0, 0, 0]      # trial 0 throws the third member out of the cluster: invalid
    eps[1, 0] = [0.05, 0, 0]      # trial 1 nudges the center: valid
    d = np.concatenate([[0.0], eps.ravel()])
    rn, plr = O.cluster_proposal(r, d, k, 1.2, width, 0)
    assert plr == 0.0
    np.testing.assert_allclose(rn[0], [0.05, 0, 0])
    np.testing.assert_array_equal(rn[1:], r[1:])
    eps[:, 2] = [10.0, 0, 0]      # every trial invalid: the first is proposed with log ratio -inf
    d = np.concatenate([[0.0], eps.ravel()])
    rn, plr = O.cluster_proposal(r, d, k, 1.2, width, 0)
    assert plr == -np.inf and rn[2, 0] == 11.0


def test_woodbury_update_matches_recomputation():
    """woodburry_update (model/utils.py:216-245), the determinant part of the reference's low-rank MCMC: replacing
    k rows of A gives the slogdet and inverse of the new matrix, padded indices included (mode="fill")."""
    rng = np.random.default_rng(8)
    n = 24
    A = rng.standard_normal((n, n))
    s0, l0 = np.linalg.slogdet(A)
    Ainv = np.linalg.inv(A)
    for changed in ([3], [0, 7, 19], [5, O.NO_NEIGHBOUR, 11, O.NO_NEIGHBOUR]):
        A_new = A.copy()
        for i in changed:
            if i < n:
                A_new[i] = rng.standard_normal(n)
        (s1, l1), inv1 = O.woodbury_update(s0, l0, A, Ainv, A_new, changed)
        s_ref, l_ref = np.linalg.slogdet(A_new)
        assert s1 == s_ref and abs(l1 - l_ref) < 1e-10
        np.testing.assert_allclose(inv1, np.linalg.inv(A_new), rtol=0, atol=1e-9 * np.abs(np.linalg.inv(A_new)).max())


_STATE_FIELDS = ("ei", "h", "env", "orb", "A", "Ainv", "signs", "logdets", "one_el", "att", "vals")


def test_low_rank_update_matches_full_evaluation():
    """log_psi_low_rank_update (model/wave_function.py:249-287) against log_psi_with_state at the moved positions,
    as tests/test_low_rank.py:29-61 of the reference checks it: electron 3 moved by (2, 0, 0) twice, the updated
    state carried into the second move, every state field and log|psi| within 1e-12 (determinants and inverses
    within 1e-9)."""
    mol, nu, r, p, *_ = case("h10")
    prob = O.Problem(mol.R, mol.Z, nu)
    w = r[0].astype(np.float64)
    (s, l), st = O.logpsi_with_state(prob, p, w)
    assert (s, l) == O.logpsi(prob, p, w)
    for _ in range(2):
        wn = w.copy()
        wn[3] += [2.0, 0.0, 0.0]
        (sf, lf), full = O.logpsi_with_state(prob, p, wn)
        (su, lu), upd = O.logpsi_low_rank_update(prob, p, wn, np.array([3]), st)
        assert su == sf
        np.testing.assert_allclose(lu, lf, rtol=1e-12, atol=1e-12)
        for key in _STATE_FIELDS:
            tol = 1e-9 if key in ("A", "Ainv", "signs", "logdets") else 1e-12
            np.testing.assert_allclose(getattr(upd, key), getattr(full, key), rtol=tol, atol=tol, err_msg=key)
        w, st = wn, upd


def test_changed_counts_are_the_recomputed_rows():
    """The move statics (get_static_input, new_sparse_model.py:414-424): exactly the electrons counted in
    n_changed_hout may change embedding; the pair counts are their neighbour counts after the move, split by spin;
    a NO_NEIGHBOUR-padded index list gathers electron n - 1 like an out-of-range JAX gather (a superset)."""
    mol, nu, r, p, *_ = case("c2h6")
    prob = O.Problem(mol.R, mol.Z, nu)
    w = r[0].astype(np.float64)
    n = mol.n_el
    h0 = O.embedding_value(prob, p, w)
    rng = np.random.default_rng(11)
    for moved in ([0], [n - 1], [2, 9], [4, O.NO_NEIGHBOUR]):
        wn = w.copy()
        for i in moved:
            if i < n:
                wn[i] += 0.7 * rng.standard_normal(3)
        aff, req = O.affected_electrons(prob, w, wn, moved)
        hout, ps, pd = O.changed_counts(prob, w, wn, moved)
        assert hout == aff.sum() and ps + pd == req.sum()
        inc = O.in_cutoff_matrix(wn.astype(np.float32), prob.cutoff)
        np.testing.assert_array_equal(req.sum(1), np.where(aff, inc.sum(1), 0))
        h1 = O.embedding_value(prob, p, wn)
        np.testing.assert_allclose(h1[~aff], h0[~aff], rtol=1e-13, atol=1e-13)
        if O.NO_NEIGHBOUR in moved:
            unpadded = O.affected_electrons(prob, w, wn, [i for i in moved if i < n])[0]
            assert np.all(aff >= unpadded) and aff[n - 1]


@pytest.mark.parametrize("kind", ["single", "cluster", "cluster_random"])
def test_low_rank_blocks_match_full_evaluation_blocks(kind):
    """mcmc_steps_low_rank (mcmc.py:196-275) with the state carried between steps takes the same decisions as the
    blocks that evaluate every proposal in full: same accepted count and final positions, margins within 1e-9.
    Cluster moves of k = 4 within radius 1.2 include NO_NEIGHBOUR-padded index lists."""
    mol, nu, r, p, *_ = case("h10")
    prob = O.Problem(mol.R, mol.Z, nu)
    w = r[1].astype(np.float64)
    rng = np.random.default_rng(13)
    steps = 10
    logu = np.log(rng.uniform(size=steps))
    if kind == "single":
        noise = rng.standard_normal((steps, 3))
        a = O.mcmc_single_block(prob, p, w, noise, logu, 0.5, offset=4)
        b = O.single_electron_low_rank_block(prob, p, w, noise, logu, 0.5, offset=4)
        assert tuple(b[4]) >= (1, 0, 0)
    else:
        k, rs = 4, kind == "cluster_random"
        draws = np.concatenate([rng.uniform(size=(steps, 1)), rng.standard_normal((steps, 15 * k))], 1)
        a = O.mcmc_cluster_block(prob, p, w, draws, logu, 0.3, k, 1.2, random_sweep=rs, offset=2)
        b = O.cluster_low_rank_block(prob, p, w, draws, logu, 0.3, k, 1.2, random_sweep=rs, offset=2)
    assert a[2] == b[2] and 0 < a[2] < steps
    np.testing.assert_array_equal(a[0], b[0])
    fin = np.isfinite(a[3])
    np.testing.assert_array_equal(fin, np.isfinite(b[3]))
    np.testing.assert_allclose(b[3][fin], a[3][fin], rtol=0, atol=1e-9)


def _direction(p, seed, keys=None):
    rng = np.random.default_rng(seed)
    keys = keys or [k for k in p if k not in ("scales",)]
    return {k: rng.standard_normal(np.shape(p[k])) * (1e-2 + np.abs(p[k])) for k in keys}


def test_parameter_jvp_matches_finite_differences_and_is_linear():
    """logpsi_jvp (complex step) along a direction touching every parameter slot agrees with a fourth-order finite
    difference (1e-8 relative; the central difference's truncation error is 4e-6 at this step) and is linear in the
    direction (1e-12)."""
    mol, nu, r, p, *_ = case("h10")
    prob = O.Problem(mol.R, mol.Z, nu)
    w = r[0].astype(np.float64)
    v1, v2 = _direction(p, 1), _direction(p, 2)
    j1 = O.logpsi_jvp(prob, p, w, v1)
    eps = 1e-5

    def f(s):
        return O.logpsi(prob, {k: p[k] + s * v1[k] if k in v1 else p[k] for k in p}, w)[1]

    fd = (8 * (f(eps) - f(-eps)) - (f(2 * eps) - f(-2 * eps))) / (12 * eps)  # fourth-order stencil
    assert abs(j1 - fd) <= 1e-8 * max(1.0, abs(fd))
    j12 = O.logpsi_jvp(prob, p, w, {k: v1[k] + v2[k] for k in v1})
    assert abs(j12 - (j1 + O.logpsi_jvp(prob, p, w, v2))) <= 1e-12 * max(1.0, abs(j12))


@pytest.mark.parametrize("name", ["h10", "c2h6"])
def test_parameter_jvp_every_slot_matches_finite_differences(name):
    """logpsi_jvp along a direction on ONE slot at a time (every slot of the parameter tree) agrees with a
    fourth-order finite difference: the checker of the device's per-walker parameter gradient is exact slot by
    slot, including the slots whose complex step reaches log|psi| only through the e-e messages."""
    mol, nu, r, p, *_ = case(name)
    prob = O.Problem(mol.R, mol.Z, nu)
    w = r[0].astype(np.float64)
    rng = np.random.default_rng(11)
    eps = 1e-6  # a few directions (ElecInit's filter weights) curve enough to leave 2e-6 of truncation at 1e-5
    for slot in p:
        v = rng.standard_normal(np.shape(p[slot]))

        def f(s):
            return O.logpsi(prob, {k: p[k] + s * v if k == slot else p[k] for k in p}, w)[1]

        fd = (8 * (f(eps) - f(-eps)) - (f(2 * eps) - f(-2 * eps))) / (12 * eps)
        got = O.logpsi_jvp(prob, p, w, {slot: v})
        assert abs(got - fd) <= 1e-6 + 1e-7 * abs(fd), (slot, got, fd)


def test_parameter_jvp_closed_forms():
    """Two directions with closed-form derivatives: the spin-up orbital bias, d log|psi| = sum_d w_d tr(A_d^-1 dA_d) /
    sum_d w_d with dA_d = env_d * db on the spin-up rows and w_d the signed determinants; and the MLP Jastrow's
    log_bias, added once per electron to J1, d log|psi| = n / J1."""
    mol, nu, r, p, *_ = case("c2h6")
    prob = O.Problem(mol.R, mol.Z, nu)
    w = r[1].astype(np.float64)
    n = mol.n_el
    db = np.random.default_rng(4).standard_normal(np.shape(p["orb_up_b"]))
    (_, _), st = O.logpsi_with_state(prob, p, w)
    wd = st.signs * np.exp(st.logdets - st.logdets.max())
    env = st.env.reshape(n, O.N_DET, n)
    dl = []
    for d in range(O.N_DET):
        dA = np.zeros((n, n))
        dA[:nu] = env[:nu, d] * db.reshape(O.N_DET, n)[d]
        dl.append(np.trace(np.linalg.solve(st.A[d], dA)))
    expect = np.sum(wd * np.array(dl)) / np.sum(wd)
    got = O.logpsi_jvp(prob, p, w, {"orb_up_b": db})
    assert abs(got - expect) <= 1e-10 * max(1.0, abs(expect))
    one_el, att, vals = st.one_el, st.att, st.vals
    J1 = O._jastrow_readout(prob, p, w, one_el, att, vals)  # (sign, log J); J1 itself is rebuilt below
    nu_ = prob.n_up
    norm = np.stack([att[:nu_].sum(0), att[nu_:].sum(0)])
    vs = np.stack([vals[:nu_].sum(0), vals[nu_:].sum(0)])
    x = (vs / norm[..., None]).reshape(-1)
    x = O.silu(x @ p["att_out1_W"] + p["att_out1_b"])
    x = O.silu(x @ p["att_out2_W"] + p["att_out2_b"])
    j1 = (x @ p["att_out3_W"] + p["att_out3_b"])[1] * p["att_scale"][1] + p["att_bias"][0] + one_el[:, 1].sum()
    assert np.sign(j1) == J1[0]
    got = O.logpsi_jvp(prob, p, w, {"log_bias": np.ones_like(p["log_bias"])})
    assert abs(got - n / j1) <= 1e-10 * max(1.0, abs(n / j1))


def test_isolated_electron_empty_neighbour_list():
    """An electron without e-e neighbours (a hydrogen atom 30 bohr from an H4 chain, its electron near its nucleus):
    its pair lists are empty, its row of the sparse Jacobian holds only the self position, and the sparse forward
    Laplacian still equals the finite-difference gradient and Laplacian of log|psi| (FP64)."""
    from make_golden import make_params
    from sparse_wf_gb300 import systems

    R = np.array([[0.0, 0, 0], [1.8, 0, 0], [3.6, 0, 0], [5.4, 0, 0], [35.4, 0, 0]], np.float32)
    mol = systems.Molecule("H4+H", R, np.ones(5, np.int64))
    nu, _ = systems.spin_counts(mol)
    rng = np.random.default_rng(2)
    w = np.concatenate([R[:4] + 0.5 * rng.standard_normal((4, 3)), R[4:] + 0.3 * rng.standard_normal((1, 3))])
    w = w.astype(np.float32)
    _, p, _, _ = make_params(mol, nu, w)
    prob = O.Problem(mol.R, mol.Z, nu)
    inc = O.in_cutoff_matrix(w, prob.cutoff)
    iso = int(np.nonzero(~inc.any(1))[0][0])
    assert not inc[iso].any() and not inc[:, iso].any()
    w = w.astype(np.float64)
    v, j, l = O.logpsi_fl(prob, p, w)
    y0, G, L = _fd(lambda x: O.logpsi(prob, p, x.reshape(-1, 3))[1], w.reshape(-1), 2e-4)
    assert abs(v - y0) < 1e-12 * abs(y0)
    np.testing.assert_allclose(j, G, rtol=1e-6, atol=1e-6 * np.abs(G).max())
    assert rel(-0.5 * (l + j @ j), -0.5 * (L + G @ G)) < 1e-5


def test_philox_known_answers():
    """The numpy Philox4x32-10 (the CPU replay of the device draws) against the generator's published known-answer
    vectors (Salmon et al., SC'11, Random123 kat_vectors): zero counter and key, all-ones, and the pi digits."""
    cases = [([0, 0, 0, 0], [0, 0], [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]),
             ([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2, [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]),
             ([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0],
              [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1])]
    for ctr, key, want in cases:
        assert O.philox4x32_10(ctr, key).tolist() == want
    # vectorised over counters: each row as its own call
    ctr = np.array([[s, w, e, 3] for s in range(2) for w in range(3) for e in range(4)], np.uint64)
    key = np.broadcast_to(np.array([7, 0], np.uint64), (len(ctr), 2))
    many = O.philox4x32_10(ctr, key)
    for k in range(len(ctr)):
        assert many[k].tolist() == O.philox4x32_10(ctr[k], key[k]).tolist()
