"""Parity of the low-rank single-electron block (fire_mcmc_low_rank_block: mcmc_steps_low_rank with the state-carrying
log_psi_low_rank_update, mcmc.py:196-275, model/wave_function.py:226-287) with the oracle's state-carrying block and
with the device's full-evaluation block, on replayed draws; and of the pseudopotential energy (fire_ecp_energy), whose
psi ratios come from the same low-rank evaluation, with the oracle's restatement."""
import numpy as np
import pytest
import torch

from helpers import case
from oracle import fire_oracle as O
from sparse_wf_gb300.wavefunction import FireWaveFunction, StaticArgs

pytestmark = pytest.mark.gpu


def _setup(name, precision):
    mol, nu, r, p, _, _ = case(name)
    wf = FireWaveFunction(mol, precision=precision)
    dt = torch.float64 if precision == "fp64" else torch.float32
    rr = torch.from_numpy(r).to("cuda", dt).contiguous()
    s = wf.get_static_input(rr)
    static = StaticArgs(s.n_pairs_same, s.n_pairs_diff, s.n_triplets, s.n_neighbours_en)
    return wf, mol, nu, r, p, rr, static


def _draws(B, steps, seed):
    rng = np.random.default_rng(seed)
    return rng.standard_normal((steps, B, 3)), np.log(rng.uniform(size=(steps, B)))


@pytest.mark.parametrize("steps", [1, 2, 3])
@pytest.mark.parametrize("name", ["h10", "c2h6"])
def test_low_rank_forced_accept_stages(cuda_lib, name, steps):
    """Stages of the low-rank step, FP64 build, every proposal accepted (log u = -inf): after 1 step log|psi| is the
    low-rank evaluation of the proposal alone (changed rows, determinant lemma, Jastrow sums); after 2 and 3 steps it
    also depends on the commit of the previous rows and the Woodbury update of the inverse.  Each is compared with a
    full evaluation of the final positions (1e-10)."""
    wf, mol, nu, r, p, rr, static = _setup(name, "fp64")
    B, n = r.shape[0], mol.n_el
    noise, _ = _draws(B, steps, 53)
    logu = np.full((steps, B), -1e300)
    dp = wf._params(p)
    logpsi = torch.zeros(B, dtype=torch.float64, device="cuda")
    n_acc, _, _ = wf.mcmc_low_rank_block(dp, rr, logpsi, static, steps, 0.4, step_offset=2, replay_noise=noise,
                                         replay_log_u=logu)
    assert n_acc.cpu().numpy().tolist() == [steps] * B
    prob = O.Problem(mol.R, mol.Z, nu)
    got = rr.cpu().numpy()
    for w in range(B):
        expect = r[w].astype(np.float64).copy()
        for s_ in range(steps):
            e = (2 + s_) % n
            expect[e] += float(np.float32(0.4)) * noise[s_, w]
        np.testing.assert_allclose(got[w], expect, atol=1e-12)
        np.testing.assert_allclose(logpsi[w].item(), O.logpsi(prob, p, expect)[1], rtol=1e-10)


@pytest.mark.parametrize("name", ["h10", "c2h6"])
def test_low_rank_block_replay_matches_oracle(cuda_lib, name):
    """FP64 build: the decisions of the oracle's state-carrying block (mcmc_low_rank_block) wherever its Metropolis
    margin is clear of rounding (|margin| > 1e-6), the final positions (1e-12), log|psi| carried by the state
    (1e-8 relative) and the move statics (n_changed_hout, n_changed_pair_same, n_changed_pair_diff) maximised over
    the walkers."""
    wf, mol, nu, r, p, rr, static = _setup(name, "fp64")
    B, n = r.shape[0], mol.n_el
    steps, off, width = n + 3, 1, 0.4
    noise, logu = _draws(B, steps, 23)
    dp = wf._params(p)
    logpsi = torch.zeros(B, dtype=torch.float64, device="cuda")
    n_acc, smax, changed = wf.mcmc_low_rank_block(dp, rr, logpsi, static, steps, width, step_offset=off,
                                                  replay_noise=noise, replay_log_u=logu)
    prob = O.Problem(mol.R, mol.Z, nu)
    got_r, got_n = rr.cpu().numpy(), n_acc.cpu().numpy()
    cmax = np.zeros(3, np.int64)
    checked = 0
    for w in range(B):
        r_ref, lp_ref, na, mg, cm = O.single_electron_low_rank_block(prob, p, r[w].astype(np.float64), noise[:, w],
                                                                     logu[:, w], float(np.float32(width)), offset=off)
        cmax = np.maximum(cmax, cm)
        if np.all(np.abs(mg) > 1e-6):
            checked += 1
            assert got_n[w] == na, w
            np.testing.assert_allclose(got_r[w], r_ref, atol=1e-12)
            np.testing.assert_allclose(logpsi[w].item(), 0.5 * lp_ref, rtol=1e-8)
    assert checked > 0
    assert tuple(changed) == tuple(int(x) for x in cmax)
    assert smax.n_pairs_same + smax.n_pairs_diff > 0


@pytest.mark.parametrize("precision", ["fp32", "mixed"])
@pytest.mark.parametrize("name", ["h10", "c10h22"])
def test_low_rank_block_matches_full_evaluation_block(cuda_lib, name, precision):
    """FP32 and mixed paths: the low-rank block and the full-evaluation block (fire_mcmc_single_block) on the same
    replayed draws take the same decisions on nearly every walker (rounding can flip a marginal one), and log|psi|
    carried by the state through n + 3 steps of Woodbury updates agrees with a fresh evaluation of the final
    positions (1e-4 relative)."""
    wf, mol, nu, r, p, rr, static = _setup(name, precision)
    B, n = r.shape[0], mol.n_el
    steps, width = n + 3, 0.4
    noise, logu = _draws(B, steps, 29)
    dp = wf._params(p)
    r_full = rr.clone()
    _, lp_full = wf.signed(dp, r_full, static)
    acc_full, _ = wf.mcmc_single_block(dp, r_full, lp_full, static, steps, width, replay_noise=noise,
                                       replay_log_u=logu)
    lp_lr = torch.zeros_like(lp_full)
    acc_lr, _, changed = wf.mcmc_low_rank_block(dp, rr, lp_lr, static, steps, width, replay_noise=noise,
                                                replay_log_u=logu)
    same = (acc_full == acc_lr).cpu().numpy()
    assert same.sum() >= B - 1
    _, lp_fresh = wf.signed(dp, rr, static)
    np.testing.assert_allclose(lp_lr.cpu().numpy(), lp_fresh.cpu().numpy(), rtol=1e-4)
    assert changed[0] >= 1


def test_low_rank_capacity_overflow_reruns(cuda_lib):
    """A changed-set capacity of 2 overflows (FIRE_FLAG_CHANGED_OVERFLOW); the wrapper reruns the block with the set
    the device saw, and the result equals a run with a generous capacity."""
    wf, mol, nu, r, p, rr, static = _setup("c2h6", "fp64")
    B, n = r.shape[0], mol.n_el
    steps, width = 6, 0.4
    noise, logu = _draws(B, steps, 31)
    dp = wf._params(p)
    ra, rb = rr.clone(), rr.clone()
    la, lb = torch.zeros(B, dtype=torch.float64, device="cuda"), torch.zeros(B, dtype=torch.float64, device="cuda")
    na, _, ca = wf.mcmc_low_rank_block(dp, ra, la, static, steps, width, replay_noise=noise, replay_log_u=logu,
                                       cap_changed=2)
    nb_, _, cb = wf.mcmc_low_rank_block(dp, rb, lb, static, steps, width, replay_noise=noise, replay_log_u=logu,
                                        cap_changed=min(n, 64))
    assert ca == cb and ca[0] > 2 and wf._lr_cap >= ca[0]
    assert torch.equal(na, nb_) and torch.equal(ra, rb)
    np.testing.assert_allclose(la.cpu().numpy(), lb.cpu().numpy(), rtol=1e-12)


def test_ecp_energy_matches_oracle(cuda_lib):
    """fire_ecp_energy in the FP64 build with replayed rotations: the local term plus the non-local quadrature with
    low-rank psi ratios against the oracle's restatement (oracle/ecp_oracle.py), 1e-7 relative, on C2H6 with a
    synthetic pseudised carbon (2 core electrons, local, s and p channels; tetrahedral quadrature).  Each ratio is
    exp(log|psi'| - log|psi|) of two FP64 evaluations that agree with the oracle to ~1e-10 relative in log|psi|
    (the forced-accept bound), i.e. a few 1e-9 in the ratio; the channel weights (up to 50 here, times 2l + 1) add
    an order of magnitude over the sum."""
    from oracle import ecp_oracle as E
    from sparse_wf_gb300 import params as P, systems
    from sparse_wf_gb300.ecp import EcpTables

    carbon = (2, [(-1, [[], [(14.0, 4.0)], [(8.0, 50.0)], [(13.0, -25.0)]]), (0, [[], [], [(7.0, 50.0)]]),
                  (1, [[], [], [(6.0, -10.0)]])])
    mol = systems.alkane(2)
    tables = EcpTables(mol.Z, {6: carbon}, n_quad={6: 4})
    val = systems.Molecule("C2H6-valence", mol.R, tables.z_eff)
    nu, _ = systems.spin_counts(val)
    r = systems.init_electrons(val, 3, 91).astype(np.float64)
    dims = P.ModelDims(val.n_el, nu, val.n_nuc)
    p = P.unpack_params(dims, *P.pack_params(dims, P.activate_jastrow(P.init_params(dims, 0)), np.float32))
    prob = O.Problem(val.R, val.Z, nu)
    hc, _ = O.embedding_value(prob, p, r[0], return_pre_scale=True)
    p["scales"] = np.array([1.0 / np.std(hc), 1.0])
    _, hu = O.embedding_value(prob, p, r[0], return_pre_scale=True)
    p["scales"][1] = 1.0 / np.std(hu)
    rng = np.random.default_rng(7)
    rot = np.stack([[E.rotation(rng.standard_normal((2, 3))) for _ in range(val.n_el)] for _ in range(len(r))])
    wf = FireWaveFunction(val, precision="fp64")
    rr = torch.from_numpy(r).cuda()
    s = wf.get_static_input(rr)
    static = StaticArgs(s.n_pairs_same, s.n_pairs_diff, s.n_triplets, s.n_neighbours_en)
    got, changed = wf.ecp_energy(wf._params(p), rr, static, tables.device("cuda"), replay_rotations=rot)
    ecp = E.Ecp(mol.Z, mol.R, {6: carbon}, n_quad={6: 4})
    for w in range(len(r)):
        ref = E.local_term(ecp, r[w]) + E.nonlocal_term(prob, p, ecp, r[w], rot[w])
        assert abs(got[w].item() - ref) <= 1e-7 * max(1.0, abs(ref)), w
    assert changed[0] >= 1


@pytest.mark.parametrize("name", ["h10", "c2h6"])
def test_low_rank_jump_block_matches_oracle(cuda_lib, name):
    """FP64 build: jumps to the nuclei evaluated from the state (fire_mcmc_low_rank_jump_block, each walker moving its
    own electron) take the oracle's decisions (mcmc_jump_block, full evaluations) wherever the margin is clear of
    rounding, with the same final positions (1e-12) and log|psi| (1e-8 relative)."""
    wf, mol, nu, r, p, rr, static = _setup(name, "fp64")
    B = r.shape[0]
    steps, sigma = 12, 2.0
    rng = np.random.default_rng(41)
    draws = np.concatenate([rng.uniform(size=(steps, B, 2)), rng.standard_normal((steps, B, 3))], axis=2)
    logu = np.log(rng.uniform(size=(steps, B)))
    dp = wf._params(p)
    logpsi = torch.zeros(B, dtype=torch.float64, device="cuda")
    n_acc, _, changed = wf.mcmc_low_rank_jump_block(dp, rr, logpsi, static, steps, sigma, replay_draws=draws,
                                                    replay_log_u=logu)
    prob = O.Problem(mol.R, mol.Z, nu)
    got_r, got_n = rr.cpu().numpy(), n_acc.cpu().numpy()
    checked = 0
    for w in range(B):
        r_ref, lp_ref, na, mg = O.mcmc_jump_block(prob, p, r[w].astype(np.float64), draws[:, w], logu[:, w],
                                                  float(np.float32(sigma)))
        if np.all(np.abs(mg[np.isfinite(mg)]) > 1e-6):
            checked += 1
            assert got_n[w] == na, w
            np.testing.assert_allclose(got_r[w], r_ref, atol=1e-12)
            np.testing.assert_allclose(logpsi[w].item(), 0.5 * lp_ref, rtol=1e-8)
    assert checked > 0 and changed[0] >= 1


def test_make_mcmc_low_rank_matches_full(cuda_lib):
    """make_mcmc(low_rank=True) with jumps and single-electron moves: the same chain as the full-evaluation blocks
    (Philox draws, FP64 build) up to walkers whose decisions sit within rounding of the threshold."""
    from sparse_wf_gb300.wavefunction import make_mcmc

    wf, mol, nu, r, p, rr, static = _setup("h10", "fp64")
    full, _ = make_mcmc(wf, proposal="single-electron", sweeps=1.0, jump_steps=4, init_width=0.3, low_rank=False)
    lowr, _ = make_mcmc(wf, proposal="single-electron", sweeps=1.0, jump_steps=4, init_width=0.3, low_rank=True)
    ra, sa = full(7, p, rr, static, 0.3)
    rb, sb = lowr(7, p, rr, static, 0.3)
    same = np.all(np.abs(ra.cpu().numpy() - rb.cpu().numpy()) < 1e-10, axis=(1, 2))
    assert same.sum() >= len(same) - 1
    assert sb["changed_max"][0] >= 1 and sb["changed_max_jump"][0] >= 1


@pytest.mark.parametrize("random_sweep", [False, True])
def test_low_rank_cluster_block_matches_oracle(cuda_lib, random_sweep):
    """FP64 build: cluster updates (k = 4 within radius 1.2 on H10, so the index lists carry padding) evaluated from the
    state take the decisions of the oracle's state-carrying block (cluster_low_rank_block) where the margin is clear of
    rounding, with its final positions (1e-12), log|psi| (1e-8) and move statics, padded entries gathering electron
    n - 1."""
    wf, mol, nu, r, p, rr, static = _setup("h10", "fp64")
    B, n = r.shape[0], mol.n_el
    steps, k, radius, width = n + 2, 4, 1.2, 0.3
    rng = np.random.default_rng(43)
    draws = np.concatenate([rng.uniform(size=(steps, B, 1)), rng.standard_normal((steps, B, 15 * k))], axis=2)
    logu = np.log(rng.uniform(size=(steps, B)))
    dp = wf._params(p)
    logpsi = torch.zeros(B, dtype=torch.float64, device="cuda")
    n_acc, _, changed = wf.mcmc_low_rank_cluster_block(
        dp, rr, logpsi, static, steps, width, k, radius, "random" if random_sweep else "sequential", step_offset=1,
        replay_draws=draws, replay_log_u=logu)
    prob = O.Problem(mol.R, mol.Z, nu)
    got_r, got_n = rr.cpu().numpy(), n_acc.cpu().numpy()
    cmax = np.zeros(3, np.int64)
    checked = 0
    for w in range(B):
        r_ref, lp_ref, na, mg, cm = O.cluster_low_rank_block(prob, p, r[w].astype(np.float64), draws[:, w],
                                                             logu[:, w], float(np.float32(width)), k,
                                                             float(np.float32(radius)), random_sweep=random_sweep,
                                                             offset=1)
        cmax = np.maximum(cmax, cm)
        if np.all(np.abs(mg[np.isfinite(mg)]) > 1e-6):
            checked += 1
            assert got_n[w] == na, w
            np.testing.assert_allclose(got_r[w], r_ref, atol=1e-12)
            np.testing.assert_allclose(logpsi[w].item(), 0.5 * lp_ref, rtol=1e-8)
    assert checked > 0
    assert tuple(changed) == tuple(int(x) for x in cmax)


def test_ecp_energy_local_channel_only(cuda_lib):
    """Stage of the pseudopotential energy: element data with only a local channel (no non-local channels, so no
    quadrature point is active); fire_ecp_energy then equals the oracle's local term (1e-10), which isolates the
    radial tables and k_ecp_local from the low-rank ratios."""
    from oracle import ecp_oracle as E
    from sparse_wf_gb300 import params as P, systems
    from sparse_wf_gb300.ecp import EcpTables

    carbon = (2, [(-1, [[], [(14.0, 4.0)], [(8.0, 50.0)], [(13.0, -25.0)]])])
    mol = systems.alkane(2)
    tables = EcpTables(mol.Z, {6: carbon}, n_quad={6: 4})
    assert tables.v_nl.shape[1] == 0
    val = systems.Molecule("C2H6-valence", mol.R, tables.z_eff)
    nu, _ = systems.spin_counts(val)
    r = systems.init_electrons(val, 3, 93).astype(np.float64)
    dims = P.ModelDims(val.n_el, nu, val.n_nuc)
    p = P.unpack_params(dims, *P.pack_params(dims, P.init_params(dims, 0), np.float32))
    wf = FireWaveFunction(val, precision="fp64")
    rr = torch.from_numpy(r).cuda()
    s = wf.get_static_input(rr)
    static = StaticArgs(s.n_pairs_same, s.n_pairs_diff, s.n_triplets, s.n_neighbours_en)
    got, _ = wf.ecp_energy(wf._params(p), rr, static, tables.device("cuda"))
    ecp = E.Ecp(mol.Z, mol.R, {6: (2, [(-1, carbon[1][0][1]), (0, [[]])])}, n_quad={6: 4})
    for w in range(len(r)):
        ref = E.local_term(ecp, r[w])
        assert abs(got[w].item() - ref) <= 1e-10 * max(1.0, abs(ref)), w
