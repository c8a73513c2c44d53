"""Parity of the CUDA path (through the C ABI) with the oracle on the same inputs.

Tolerances: neighbour lists and triplets bit-exact; FP64 build <= 1e-10 relative on log|psi|, its gradient, its
Laplacian and E_loc.  FP32 and mixed paths: log|psi| <= 3e-5 relative (test_logpsi); E_loc per walker, and the
Laplacian and the gradient of log|psi| on walkers away from a node, within 1e-5 (mixed: 1e-4) of the magnitude of
the terms E_loc is summed from,
S = (|lap log psi| + |grad log psi|^2) / 2 + |V| (helpers.check_eloc_contract).  Near a node of psi the FP32
rounding of the values that build the orbital matrices moves E_loc by up to ~2e-6 of the kinetic terms; the device
flags those walkers (kinetic terms above refine_ratio |E_loc|, or a determinant-weighted condition number above
refine_kappa) and evaluates them again with FP64 orbital-matrix values, LU and inverse; the test checks that every
walker the oracle finds ill-conditioned (with a 5 % margin) was refined."""
import ctypes as C

import numpy as np
import pytest
import torch

from helpers import case, check_eloc_contract, golden, rel
from oracle import fire_oracle as O
from sparse_wf_gb300 import _lib, systems
from sparse_wf_gb300.wavefunction import FireWaveFunction, StaticArgs

pytestmark = pytest.mark.gpu
TOL = {"fp32": 1e-5, "fp64": 1e-10, "mixed": 1e-5}


def _wf(name, precision):
    mol, nu, r, p, blob, offs = case(name)
    wf = FireWaveFunction(mol, precision=precision)
    return wf, mol, nu, r, p


def _static(wf, r, pad=1.0):
    s = wf.get_static_input(r)
    return StaticArgs(s.n_pairs_same, s.n_pairs_diff, s.n_triplets, s.n_neighbours_en)


@pytest.mark.parametrize("name", ["h10", "c2h6", "c10h22"])
@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_neighbor_lists_bit_exact(cuda_lib, name, precision):
    g = golden(name)
    wf, mol, nu, r, p = _wf(name, precision)
    rr = r.astype(np.float64) if precision == "fp64" else r
    static = StaticArgs(int(g["cap_same"]), int(g["cap_diff"]), 0, int(g["cap_nuc"]))
    out = wf.neighbor_lists(rr, static)
    assert out["status"][0] == 0
    for k in ("ct_same", "nb_same", "jac_same", "ct_diff", "nb_diff", "jac_diff", "jac_ctr", "jac_dep", "en_idx"):
        np.testing.assert_array_equal(out[k], g["nl_" + k], err_msg=k)
    np.testing.assert_array_equal(out["counts"], g["counts"])


def test_neighbor_lists_c40h82_exact(cuda_lib):
    mol = systems.alkane(40)
    nu, _ = systems.spin_counts(mol)
    r = systems.init_electrons(mol, 6, 4242)
    wf = FireWaveFunction(mol, precision="fp32")
    counts = np.array([O.static_counts(w, mol.R, nu, 5.0, 20.0) for w in r])
    static = StaticArgs(int(counts[:, 0].max()), int(counts[:, 1].max()) + 5, 0, int(counts[:, 3].max()))
    out = wf.neighbor_lists(r, static)
    np.testing.assert_array_equal(out["counts"], counts)
    for k, w in enumerate(r):
        (a, b, c), (d, e, f), (gg, h) = O.pair_indices(w, nu, 5.0, static.n_pairs_same, static.n_pairs_diff)
        for key, v in zip(("ct_same", "nb_same", "jac_same", "ct_diff", "nb_diff", "jac_diff", "jac_ctr", "jac_dep"),
                          (a, b, c, d, e, f, gg, h)):
            np.testing.assert_array_equal(out[key][k], v, err_msg=key)
        np.testing.assert_array_equal(out["en_idx"][k], O.neighbouring_nuclei(w, mol.R, 20.0, static.n_neighbours_en))


def test_neighbor_overflow_is_reported(cuda_lib):
    g = golden("c2h6")
    wf, mol, nu, r, p = _wf("c2h6", "fp32")
    out = wf.neighbor_lists(r, StaticArgs(3, 3, 0, 2))
    assert out["status"][0] & (_lib.FLAG_PAIR_OVERFLOW | _lib.FLAG_NUC_OVERFLOW)
    assert out["status"][1] == (g["counts"][:, 0] + g["counts"][:, 1]).max()


@pytest.mark.parametrize("name", ["h10", "c2h6"])
def test_triplets_exact(cuda_lib, name):
    g = golden(name)
    wf, mol, nu, r, p = _wf(name, "fp32")
    B, n = r.shape[0], mol.n_el
    cap = g["triplets"].shape[2]
    st = _static(wf, r)
    prob = wf._problem(B, StaticArgs(st.n_pairs_same, st.n_pairs_diff + 4, 0, st.n_neighbours_en))
    rt = torch.from_numpy(r).cuda()
    outs = [torch.full((B, cap), -7, dtype=torch.int32, device="cuda") for _ in range(4)]
    ws = torch.empty(64 << 20, dtype=torch.uint8, device="cuda")
    status = torch.zeros(8, dtype=torch.int32, device="cuda")
    rc = cuda_lib.fire_triplets(wf._stream(), C.byref(prob), C.c_void_p(rt.data_ptr()), cap,
                                *[C.c_void_p(o.data_ptr()) for o in outs], C.c_void_p(ws.data_ptr()),
                                C.c_size_t(ws.numel()), C.c_void_p(status.data_ptr()))
    assert rc == 0
    got = np.stack([o.cpu().numpy() for o in outs], axis=1)
    np.testing.assert_array_equal(got, g["triplets"])
    assert status[0].item() == 0


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_potential_energy(cuda_lib, precision):
    wf, mol, nu, r, p = _wf("c10h22", precision)
    rr = r.astype(np.float64) if precision == "fp64" else r
    got = wf.potential_energy(rr).double().cpu().numpy()
    ref = np.array([O.potential_energy(w.astype(np.float64), mol.R, mol.Z) for w in r])
    assert rel(got, ref).max() < (1e-6 if precision == "fp32" else 1e-12)


@pytest.mark.parametrize("name", ["h10", "c2h6", "c10h22"])
@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_embedding(cuda_lib, name, precision):
    wf, mol, nu, r, p = _wf(name, precision)
    rr = r.astype(np.float64) if precision == "fp64" else r
    static = _static(wf, rr)
    hc, hu = wf.embedding(p, rr, static)
    prob = O.Problem(mol.R, mol.Z, nu)
    for k, w in enumerate(r.astype(np.float64)):
        c_ref, u_ref = O.embedding_value(prob, p, w, return_pre_scale=True)
        c, u = hc[k].double().cpu().numpy(), hu[k].double().cpu().numpy()
        assert np.linalg.norm(c - c_ref) / np.linalg.norm(c_ref) < TOL[precision]
        assert np.linalg.norm(u - u_ref) / np.linalg.norm(u_ref) < TOL[precision]


@pytest.mark.parametrize("name", ["h10", "h10_plain", "c2h6", "c10h22"])
@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_logpsi(cuda_lib, name, precision):
    wf, mol, nu, r, p = _wf(name, precision)
    rr = r.astype(np.float64) if precision == "fp64" else r
    static = _static(wf, rr)
    sign, logpsi = wf.signed(p, rr, static)
    prob = O.Problem(mol.R, mol.Z, nu)
    ref = np.array([O.logpsi(prob, p, w) for w in r.astype(np.float64)])
    np.testing.assert_array_equal(sign.cpu().numpy(), ref[:, 0])
    err = np.abs(logpsi.double().cpu().numpy() - ref[:, 1]) / np.maximum(1.0, np.abs(ref[:, 1]))
    # FP32: the hidden planes are rounded to FP32 between layers and the orbital matrices' condition numbers (up to
    # ~1e5 on random-init H10 walkers) amplify that rounding in log det: 1.0e-5 measured on the golden H10 walkers,
    # 2.8e-5 at most on H10 x 512 (the local energy's refinement pass evaluates those walkers with FP64 values)
    assert err.max() < (3e-5 if precision == "fp32" else TOL[precision]), err.max()


@pytest.mark.parametrize("name", ["h10", "h10_plain", "c2h6", "c10h22"])
@pytest.mark.parametrize("precision", ["fp32", "fp64", "mixed"])
def test_local_energy(cuda_lib, name, precision):
    wf, mol, nu, r, p = _wf(name, precision)
    _check_local_energy(wf, mol, nu, r, p, precision)


@pytest.mark.parametrize("precision", ["fp32", "fp64", "mixed"])
def test_local_energy_odd_electron_count(cuda_lib, precision):
    """H21 chain: 21 electrons (11 up, 10 down), so the elimination's last panel is 5 columns wide, the last
    column of the matrix has no pair partner and the staged pivot rows are padded; walkers and parameters
    from seeds, the oracle evaluated here."""
    from make_golden import make_params

    mol = systems.hydrogen_chain(21, 1.8)
    nu, _ = systems.spin_counts(mol)
    r = systems.init_electrons(mol, 3, 21).astype(np.float32)
    _, p, _, _ = make_params(mol, nu, r[0], seed=5, activate=True)
    wf = FireWaveFunction(mol, precision=precision)
    _check_local_energy(wf, mol, nu, r, p, precision)


def _check_local_energy(wf, mol, nu, r, p, precision):
    rr = r.astype(np.float64) if precision == "fp64" else r
    static = _static(wf, rr)
    eloc, aux = wf.local_energy_full(p, rr, static, debug=True)
    prob = O.Problem(mol.R, mol.Z, nu)
    fl = [O.logpsi_fl(prob, p, w) for w in r.astype(np.float64)]
    ekin = np.array([-0.5 * (x[2] + x[1] @ x[1]) for x in fl])
    epot = np.array([O.potential_energy(w, mol.R, mol.Z) for w in r.astype(np.float64)])
    eref = ekin + epot
    lp = np.array([x[0] for x in fl])
    got = eloc.double().cpu().numpy()
    dbg = {k: v.double().cpu().numpy() for k, v in aux["debug"].items()}
    tol = TOL[precision]
    assert rel(dbg["potential"], epot).max() < tol
    grad_ref = np.array([x[1] for x in fl]).reshape(dbg["grad"].shape)
    lap_ref = np.array([x[2] for x in fl])
    # log|psi| in FP32 / mixed: the bound of test_logpsi (carrier rounding amplified by the orbital matrices)
    tol_lp = tol if precision == "fp64" else 3e-5
    assert np.all(np.abs(aux["logpsi"].double().cpu().numpy() - lp) / np.maximum(1, np.abs(lp)) < tol_lp)
    if precision == "fp64":
        for k in range(len(r)):
            assert np.linalg.norm(dbg["grad"][k] - grad_ref[k]) / np.linalg.norm(grad_ref[k]) < tol
        assert np.all(rel(dbg["lap"], lap_ref) < tol), (dbg["lap"], lap_ref, tol)
        assert np.all(rel(dbg["kinetic"], ekin) < tol), (dbg["kinetic"], ekin)
        assert np.all(rel(got, eref) < tol)
    else:
        ks = 0.5 * (np.abs(lap_ref) + np.sum(grad_ref.reshape(len(r), -1) ** 2, axis=1))
        check_eloc_contract(precision, wf, got, eref, ks, epot, dbg["refined"] > 0, lap=dbg["lap"], lap_ref=lap_ref,
                            grad=dbg["grad"], grad_ref=grad_ref)
    st = aux["stats"].cpu().numpy()
    assert abs(st[0] - got.mean()) < 1e-9 * max(1, abs(got.mean()))


@pytest.mark.parametrize("name", ["h10", "c2h6"])
def test_mcmc_replay(cuda_lib, name):
    g = golden(name)
    wf, mol, nu, r, p = _wf(name, "fp64")
    rr = torch.from_numpy(r.astype(np.float64)).cuda().contiguous()
    static = _static(wf, rr)
    dp = wf._params(p)
    _, logpsi = wf.signed(dp, rr, static)
    steps = g["mcmc_noise"].shape[0]
    n_acc, smax = wf.mcmc_block(dp, rr, logpsi, static, steps, float(g["mcmc_width"]),
                                replay_noise=g["mcmc_noise"].astype(np.float64),
                                replay_log_u=g["mcmc_logu"].astype(np.float64))
    sure = np.all(np.abs(g["mcmc_margin"]) > 1e-6, axis=1)
    assert sure.any()
    np.testing.assert_array_equal(n_acc.cpu().numpy()[sure], g["mcmc_nacc"][sure])
    np.testing.assert_allclose(rr.cpu().numpy()[sure], g["mcmc_r"][sure], atol=1e-12)
    assert smax.n_pairs_same + smax.n_pairs_diff > 0


@pytest.mark.parametrize("name", ["h10", "c2h6"])
def test_mcmc_single_electron_replay(cuda_lib, name):
    """Single-electron block (proposal_single_electron, mcmc.py:100-111; mcmc_steps_low_rank, 196-275) in the FP64
    build with replayed draws: the accept decisions equal the oracle's wherever the oracle's Metropolis margin is
    clear of rounding (|margin| > 1e-6), and so do the final positions (1e-12); only electron (offset + s) mod n
    moves at step s."""
    wf, mol, nu, r, p = _wf(name, "fp64")
    B, n = r.shape[0], mol.n_el
    steps, off, width = n + 3, 2, 0.4
    rng = np.random.default_rng(17)
    noise = rng.standard_normal((steps, B, 3))
    logu = np.log(rng.uniform(size=(steps, B)))
    rr = torch.from_numpy(r.astype(np.float64)).cuda().contiguous()
    static = _static(wf, rr)
    dp = wf._params(p)
    _, logpsi = wf.signed(dp, rr, static)
    n_acc, smax = wf.mcmc_single_block(dp, rr, logpsi, static, steps, width, step_offset=off, replay_noise=noise,
                                       replay_log_u=logu)
    prob = O.Problem(mol.R, mol.Z, nu)
    got_r, got_n = rr.cpu().numpy(), n_acc.cpu().numpy()
    checked = 0
    for w in range(B):
        # the C ABI takes the width as float32
        r_ref, lp_ref, na, mg = O.mcmc_single_block(prob, p, r[w].astype(np.float64), noise[:, w], logu[:, w],
                                                    float(np.float32(width)), offset=off)
        if np.all(np.abs(mg) > 1e-6):
            checked += 1
            assert got_n[w] == na, w
            np.testing.assert_allclose(got_r[w], r_ref, atol=1e-12)
            # log|psi| of the final positions: FP64 elimination of orbital matrices the chain may have made
            # ill-conditioned, so only 1e-6 here; the value path itself is pinned by test_logpsi
            np.testing.assert_allclose(logpsi[w].item(), 0.5 * lp_ref, rtol=1e-6)
    assert checked > 0
    # unmoved electrons keep their positions exactly: every electron moved at most ceil(steps / n) times
    moved = np.any(got_r != r.astype(np.float64), axis=2)
    assert moved.sum() <= B * steps
    assert smax.n_pairs_same + smax.n_pairs_diff > 0


@pytest.mark.parametrize("name", ["h10", "c2h6"])
def test_mcmc_jump_replay(cuda_lib, name):
    """Jumps to the nuclei (proposal_jump_to_atom, mcmc.py:164-193) in the FP64 build with replayed draws: accept
    decisions and final positions equal the oracle's wherever its Metropolis margin (proposal log ratio included)
    is clear of rounding."""
    wf, mol, nu, r, p = _wf(name, "fp64")
    B = r.shape[0]
    steps, sigma = 12, 2.0
    rng = np.random.default_rng(29)
    draws = np.concatenate([rng.uniform(size=(steps, B, 2)), rng.standard_normal((steps, B, 3))], axis=2)
    logu = np.log(rng.uniform(size=(steps, B)))
    rr = torch.from_numpy(r.astype(np.float64)).cuda().contiguous()
    static = _static(wf, rr)
    dp = wf._params(p)
    _, logpsi = wf.signed(dp, rr, static)
    n_acc, _ = wf.mcmc_jump_block(dp, rr, logpsi, static, steps, sigma, replay_draws=draws, replay_log_u=logu)
    prob = O.Problem(mol.R, mol.Z, nu)
    got_r, got_n = rr.cpu().numpy(), n_acc.cpu().numpy()
    checked = 0
    for w in range(B):
        r_ref, lp_ref, na, mg = O.mcmc_jump_block(prob, p, r[w].astype(np.float64), draws[:, w], logu[:, w], sigma)
        if np.all(np.abs(mg) > 1e-6):
            checked += 1
            assert got_n[w] == na, w
            np.testing.assert_allclose(got_r[w], r_ref, atol=1e-12)
            np.testing.assert_allclose(logpsi[w].item(), 0.5 * lp_ref, rtol=1e-6)
    assert checked > 0 and got_n.sum() > 0


@pytest.mark.parametrize("name,sweep", [("h10", "sequential"), ("h10", "random"), ("c2h6", "sequential")])
def test_mcmc_cluster_replay(cuda_lib, name, sweep):
    """Cluster updates (proposal_cluster_update, mcmc.py:119-161) in the FP64 build with replayed draws: accept
    decisions and final positions equal the oracle's wherever its margin is clear of rounding (invalid clusters
    give -inf)."""
    wf, mol, nu, r, p = _wf(name, "fp64")
    B, n = r.shape[0], mol.n_el
    steps, off, width, kmax, radius = n + 2, 3, 0.5, 5, 2.0
    k = min(kmax, n)
    rng = np.random.default_rng(31)
    draws = np.concatenate([rng.uniform(size=(steps, B, 1)), rng.standard_normal((steps, B, 15 * k))], axis=2)
    logu = np.log(rng.uniform(size=(steps, B)))
    rr = torch.from_numpy(r.astype(np.float64)).cuda().contiguous()
    static = _static(wf, rr)
    dp = wf._params(p)
    _, logpsi = wf.signed(dp, rr, static)
    n_acc, _ = wf.mcmc_cluster_block(dp, rr, logpsi, static, steps, width, kmax, radius, sweep, step_offset=off,
                                     replay_draws=draws, replay_log_u=logu)
    prob = O.Problem(mol.R, mol.Z, nu)
    got_r, got_n = rr.cpu().numpy(), n_acc.cpu().numpy()
    checked = 0
    for w in range(B):
        r_ref, lp_ref, na, mg = O.mcmc_cluster_block(prob, p, r[w].astype(np.float64), draws[:, w], logu[:, w],
                                                     float(np.float32(width)), k, float(np.float32(radius)),
                                                     random_sweep=sweep == "random", offset=off)
        if np.all(np.abs(mg) > 1e-6):
            checked += 1
            assert got_n[w] == na, w
            np.testing.assert_allclose(got_r[w], r_ref, atol=1e-12)
    assert checked > 0 and got_n.sum() > 0


@pytest.mark.parametrize("proposal", ["all-electron", "single-electron", "cluster-update"])
def test_make_mcmc_steps(cuda_lib, proposal):
    """make_mcmc (mcmc.py:278-346) with 4 jump steps before the proposal: walkers keep their shape and move, the
    acceptance fractions lie in [0, 1], the statics are reported for both blocks."""
    from sparse_wf_gb300.wavefunction import make_mcmc

    wf, mol, nu, r, p = _wf("h10", "fp32")
    step, width = make_mcmc(wf, steps=3, init_width=0.3, proposal=proposal, sweeps=1.0, jump_steps=4)
    rr = torch.from_numpy(r).cuda().contiguous()
    static = _static(wf, rr)
    r_new, stats = step(7, p, rr, static, width)
    assert r_new.shape == rr.shape and torch.isfinite(r_new).all()
    assert bool((r_new != rr).any())
    assert 0.0 <= stats["pmove"] <= 1.0 and 0.0 <= stats["pmove_jump"] <= 1.0
    assert stats["static_max"].n_pairs_same + stats["static_max"].n_pairs_diff > 0
    assert stats["static_max_jump"].n_pairs_same + stats["static_max_jump"].n_pairs_diff > 0


def test_mcmc_philox_draws_match_cpu_replay(cuda_lib):
    """The device's all-electron block draws (Philox4x32-10, Box-Muller) equal the oracle's numpy replay
    (philox_all_electron_noise, philox_log_u): every accepted walker moved by exactly width * eps of that replay
    (float32 positions), and the FP64 build takes the replayed Metropolis decision wherever its margin is clear
    of rounding.  This is what lets the CPU baseline run the benchmark's Metropolis block on the same walkers."""
    wf, mol, nu, r, p = _wf("c2h6", "fp32")
    rr = torch.from_numpy(r).cuda().contiguous()
    r0 = r.copy()
    static = _static(wf, rr)
    dp = wf._params(p)
    _, logpsi = wf.signed(dp, rr, static)
    width, seed = 0.02, 1234  # small moves of all 18 electrons: most proposals are accepted
    n_acc, _ = wf.mcmc_block(dp, rr, logpsi, static, 1, width, seed=seed, counter=5)
    got = rr.cpu().numpy()
    acc = n_acc.cpu().numpy()
    assert acc.sum() > 0
    for w in range(r.shape[0]):
        eps = O.philox_all_electron_noise(seed, 5, 0, w, mol.n_el)
        want = (r0[w].astype(np.float64) + np.float64(np.float32(width)) * eps.astype(np.float64)).astype(np.float32)
        if acc[w]:
            np.testing.assert_allclose(got[w], want, rtol=0, atol=4e-6)
        else:
            np.testing.assert_array_equal(got[w], r0[w])
    # decisions: FP64 build against the oracle's replayed block, 2 steps
    wf64 = FireWaveFunction(mol, precision="fp64")
    r64 = torch.from_numpy(r0.astype(np.float64)).cuda().contiguous()
    st64 = _static(wf64, r64)
    dp64 = wf64._params(p)
    _, lp64 = wf64.signed(dp64, r64, st64)
    n64, _ = wf64.mcmc_block(dp64, r64, lp64, st64, 2, width, seed=seed, counter=5)
    prob = O.Problem(mol.R, mol.Z, nu)
    checked = 0
    for w in range(r.shape[0]):
        # the oracle keeps float32 positions (the FP32 path's), the FP64 build doubles: margins within ~1e-5 of zero
        # may differ
        _, na, mg = O.mcmc_block_philox(prob, p, r0[w], 2, width, seed, 5, w)
        if np.all(np.abs(mg) > 1e-3):
            checked += 1
            assert int(n64[w]) == na
    assert checked > 0


@pytest.mark.parametrize("name", ["c2h6", "c10h22"])
@pytest.mark.parametrize("precision", ["fp32", "mixed"])
def test_mcmc_value_path_logpsi(cuda_lib, name, precision):
    """The Metropolis blocks evaluate proposals with the plain value contractions (and, in the mixed path, the
    envelope value rows on the tensor cores): one step with zero displacement that accepts every proposal leaves
    the block's own log|psi| of the walkers, which must match the oracle like fire_logpsi's (3e-5 relative)."""
    wf, mol, nu, r, p = _wf(name, precision)
    rr = torch.from_numpy(r).cuda().contiguous()
    static = _static(wf, rr)
    dp = wf._params(p)
    _, logpsi = wf.signed(dp, rr, static)
    logpsi.fill_(-1e30)  # any proposal is accepted; the block stores the proposals' log|psi|
    B = r.shape[0]
    n_acc, _ = wf.mcmc_block(dp, rr, logpsi, static, 1, 0.1, replay_noise=np.zeros((1, B, mol.n_el, 3)),
                             replay_log_u=np.zeros((1, B)))
    assert int(n_acc.sum()) == B
    prob = O.Problem(mol.R, mol.Z, nu)
    ref = np.array([O.logpsi(prob, p, w)[1] for w in r.astype(np.float64)])
    err = np.abs(logpsi.double().cpu().numpy() - ref) / np.maximum(1.0, np.abs(ref))
    assert err.max() < 3e-5, err.max()
