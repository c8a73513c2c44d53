"""Host-side logic: the C-ABI library (load + exported symbols + host-only size functions), the
parameter layout shared by Python and C, static-capacity padding, synthetic systems and the
multi-process walker sharding (gloo, world size 2)."""
import ctypes as C
import os
import re
from pathlib import Path

import numpy as np
import pytest

from sparse_wf_gb300 import _lib, params as P, systems
from sparse_wf_gb300.build import build

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def lib():
    build()
    return _lib.load()


def header_symbols():
    hdr = (ROOT / "include" / "fire.h").read_text()
    return re.findall(r"^\s*(?:fire_status|int32_t)\s+(fire_\w+)\s*\(", hdr, re.M)


def test_library_exports_every_header_symbol(lib):
    syms = header_symbols()
    assert len(syms) == 27
    assert sorted(syms) == sorted(_lib.SYMBOLS)
    for s in syms:
        assert hasattr(lib, s), s
    assert lib.fire_abi_version() == 3


def test_header_slot_enum_matches_python():
    hdr = (ROOT / "include" / "fire.h").read_text()
    enum = re.search(r"enum fire_param_slot \{(.*?)\};", hdr, re.S).group(1)
    names = [x.strip() for x in enum.replace("\n", " ").split(",") if x.strip()]
    assert names[-1] == "FIRE_P_COUNT"
    assert [x.replace("FIRE_P_", "").lower() for x in names[:-1]] == [x.lower() for x in P.PARAM_SLOT_NAMES]


@pytest.mark.parametrize("mol", [systems.hydrogen_chain(10), systems.alkane(10), systems.alkane(40)])
def test_param_layout_matches(lib, mol):
    nu, _ = systems.spin_counts(mol)
    d = P.ModelDims(mol.n_el, nu, mol.n_nuc)
    prob = _lib.Problem(mol.n_el, nu, mol.n_nuc, 4, 5.0, 20.0, 100, 10, 0, 0)
    offs = (C.c_int64 * (len(P.PARAM_SLOT_NAMES) + 1))()
    assert lib.fire_param_layout(C.byref(prob), offs) == 0
    np.testing.assert_array_equal(np.array(offs[:]), P.param_offsets(d))
    p = P.init_params(d, 0)
    blob, o = P.pack_params(d, p)
    q = P.unpack_params(d, blob, o)
    for k in p:
        np.testing.assert_allclose(q[k], p[k].astype(np.float32), rtol=0, atol=0)


def test_sizes_and_invalid_arguments(lib):
    prob = _lib.Problem(82, 41, 32, 64, 5.0, 20.0, 2500, 40, 0, 0)
    a, b, c = C.c_size_t(), C.c_size_t(), C.c_size_t()
    assert lib.fire_workspace_size(C.byref(prob), 8, C.byref(a)) == 0
    assert lib.fire_workspace_size(C.byref(prob), 16, C.byref(b)) == 0
    assert b.value > a.value > 0
    assert lib.fire_prepared_size(C.byref(prob), C.byref(c)) == 0
    assert c.value >= 4 * P.param_offsets(P.ModelDims(82, 41, 32))[-1]
    bad = _lib.Problem(82, 90, 32, 64, 5.0, 20.0, 2500, 40, 0, 0)  # n_up > n_el
    assert lib.fire_workspace_size(C.byref(bad), 8, C.byref(a)) == 1
    bad = _lib.Problem(82, 41, 32, 64, 5.0, 20.0, 2500, 40, 7, 0)  # unknown precision
    assert lib.fire_prepared_size(C.byref(bad), C.byref(a)) == 1
    prob_fp64 = _lib.Problem(82, 41, 32, 64, 5.0, 20.0, 2500, 40, 2, 0)
    assert lib.fire_workspace_size(C.byref(prob_fp64), 8, C.byref(c)) == 0 and c.value > a.value


def test_local_energy_rejects_problems_beyond_the_inverse_limit(lib):
    """fire_local_energy returns FIRE_ERR_UNSUPPORTED (2) before any CUDA call for more than 798 electrons: the
    orbital-matrix inverse is eliminated in shared memory; the pointers are never dereferenced."""
    dummy = C.c_void_p(16)
    big = _lib.Problem(800, 400, 100, 4, 5.0, 20.0, 100, 10, 0, 0)
    rc = lib.fire_local_energy(None, C.byref(big), dummy, dummy, dummy, dummy, None, None, dummy, None, None, dummy,
                               C.c_size_t(1), dummy)
    assert rc == 2


def test_low_rank_block_sizes_and_argument_checks(lib):
    """fire_low_rank_workspace_size / fire_mcmc_low_rank_block: the low-rank state (with the inverses) and the
    per-step scratch grow with the changed-set capacity; capacities above 128, more than 798
    electrons, a zero capacity or half a replay are rejected before any CUDA call (pointers never dereferenced)."""
    prob = _lib.Problem(82, 41, 32, 64, 5.0, 20.0, 2500, 40, 0, 0)
    a, b = C.c_size_t(), C.c_size_t()
    assert lib.fire_low_rank_workspace_size(C.byref(prob), 8, 32, C.byref(a)) == 0
    assert lib.fire_low_rank_workspace_size(C.byref(prob), 8, 64, C.byref(b)) == 0
    # the transposed inverses alone: 8 walkers x 4 determinants x 82 x ainv_ld(82) floats
    assert b.value > a.value > 8 * 4 * 82 * 88 * 4
    assert lib.fire_low_rank_workspace_size(C.byref(prob), 8, 129, C.byref(a)) == 2
    assert lib.fire_low_rank_workspace_size(C.byref(prob), 8, 0, C.byref(a)) == 1
    dummy = C.c_void_p(16)

    def call(pr, cap, noise=None, logu=None):
        return lib.fire_mcmc_low_rank_block(None, C.byref(pr), dummy, dummy, dummy, dummy, dummy, 4, 0, 0.5, cap, 0, 0,
                                            noise, logu, None, None, dummy, C.c_size_t(1), dummy)

    assert call(prob, 129) == 2
    assert call(prob, 0) == 1
    assert call(prob, 32, noise=dummy) == 1
    big = _lib.Problem(800, 400, 100, 4, 5.0, 20.0, 100, 10, 0, 0)
    assert call(big, 32) == 2


def test_logpsi_grad_sizes_and_argument_checks(lib):
    """fire_logpsi_grad_workspace_size grows with the walkers per pass; fire_logpsi_grad rejects a workspace too small
    for the requested pass (FIRE_ERR_WORKSPACE, 3), more than 798 electrons (2) and missing outputs (1) before any CUDA
    call (the pointers are never dereferenced)."""
    prob = _lib.Problem(82, 41, 32, 64, 5.0, 20.0, 2500, 40, 0, 0)
    a, b = C.c_size_t(), C.c_size_t()
    assert lib.fire_logpsi_grad_workspace_size(C.byref(prob), 4, C.byref(a)) == 0
    assert lib.fire_logpsi_grad_workspace_size(C.byref(prob), 8, C.byref(b)) == 0
    assert b.value > a.value > 0
    dummy = C.c_void_p(16)

    def call(pr, ws_bytes, grad=dummy):
        return lib.fire_logpsi_grad(None, C.byref(pr), dummy, dummy, dummy, dummy, dummy, grad, dummy,
                                    C.c_size_t(ws_bytes), dummy)

    prob.chunk_walkers = 8
    assert call(prob, a.value) == 3  # the plan of 8 walkers per pass does not fit 4 walkers' workspace
    assert call(prob, 1) == 3
    assert call(prob, b.value, grad=None) == 1
    big = _lib.Problem(800, 400, 100, 4, 5.0, 20.0, 100, 10, 0, 0)
    assert call(big, b.value) == 2


def test_static_padding_mirrors_reference():
    from sparse_wf_gb300.wavefunction import StaticArgs

    s = StaticArgs(100, 120, 5000, 30).round_with_padding(1.1, 82, 41, 32)
    assert s.n_pairs_same >= 100 and s.n_pairs_diff >= 120 and s.n_neighbours_en == 30  # int(1.1**36)
    assert StaticArgs(7, 3, 9, 2).round_with_padding(1.0, 10, 5, 10) == StaticArgs(7, 3, 9, 2)
    big = StaticArgs(10**6, 10**6, 10**9, 10**3).round_with_padding(1.2, 10, 5, 4)
    assert big == StaticArgs(40, 50, 810, 4)


def test_alkane_geometry():
    for k in (1, 2, 5, 40):
        m = systems.alkane(k)
        assert m.n_el == 8 * k + 2 and m.n_nuc == 3 * k + 2
        assert systems.spin_counts(m) == (4 * k + 1, 4 * k + 1)
        d = np.linalg.norm(m.R[:, None] - m.R[None], axis=-1)
        np.fill_diagonal(d, np.inf)
        assert d.min() > 2.0
        if k > 1:
            assert np.isclose(d[:k, :k].min(), systems.C_C, atol=1e-5)
        ind = systems.assign_spins_to_atoms(m.R, m.Z)
        assert np.all(np.bincount(ind, minlength=m.n_nuc) == m.Z)
    h = systems.hydrogen_chain(10, 1.8)
    assert systems.spin_counts(h) == (5, 5)
    r = systems.init_electrons(h, 3, 1000)
    assert r.shape == (3, 10, 3) and r.dtype == np.float32


def _gloo_worker(rank, world, port, q):
    import torch
    import torch.distributed as dist
    from sparse_wf_gb300.distributed import energy_stats, shard

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    e = torch.from_numpy(np.random.default_rng(5).normal(-100.0, 3.0, 101))
    a, b = shard(101, rank, world)
    q.put((rank, a, b, energy_stats(e[a:b])))
    dist.destroy_process_group()


def test_walker_sharding_gloo():
    import multiprocessing as mp
    import socket

    from sparse_wf_gb300.distributed import shard

    assert [shard(10, r, 3) for r in range(3)] == [(0, 4), (4, 7), (7, 10)]
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_gloo_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
    e = np.random.default_rng(5).normal(-100.0, 3.0, 101)
    res.sort()
    assert res[0][1:3] == (0, 51) and res[1][1:3] == (51, 101)
    for _, _, _, (mean, std) in res:
        assert abs(mean - e.mean()) < 1e-12 and abs(std - e.std()) < 1e-12


def test_serving_trace_and_summary():
    """Poisson traces are reproducible and the latency summary reads the completed requests."""
    from sparse_wf_gb300.serving import poisson_trace, summarize

    a = poisson_trace(50, 20.0, seed=3)
    b = poisson_trace(50, 20.0, seed=3)
    assert [(r.kind, r.n_carbon, r.walkers, r.arrival) for r in a] == [(r.kind, r.n_carbon, r.walkers, r.arrival)
                                                                          for r in b]
    arr = [r.arrival for r in a]
    assert all(x < y for x, y in zip(arr, arr[1:]))
    assert all(4 <= r.n_carbon <= 60 and 256 <= r.walkers <= 2048 for r in a)
    for k, r in enumerate(a):
        r.done = r.arrival + 0.001 * (k + 1)
    m = summarize(a, 10.0)
    assert abs(m["p50_ms"] - np.percentile([r.latency * 1e3 for r in a], 50)) < 1e-9
    assert m["max_ms"] == pytest.approx(50.0)


def test_ragged_batch_draws():
    from sparse_wf_gb300.ragged import ragged_alkanes

    ns, ws = ragged_alkanes(64, seed=4)
    assert len(ns) == 64 and min(ns) >= 2 and max(ns) <= 40 and min(ws) >= 64 and max(ws) <= 1024
    assert ragged_alkanes(64, seed=4) == (ns, ws)


def test_make_mcmc_proposal_selection_checks():
    """make_mcmc (mcmc.py:278-346): unknown proposals are rejected, a sequential cluster sweep must cover whole
    sweeps, and the step counts follow the reference (steps, int(sweeps * n_el)); no GPU call is made."""
    from sparse_wf_gb300.wavefunction import FireWaveFunction, make_mcmc

    wf = FireWaveFunction(systems.hydrogen_chain(10), precision="fp32", device="cpu")
    with pytest.raises(ValueError):
        make_mcmc(wf, proposal="gibbs")
    with pytest.raises(ValueError):
        make_mcmc(wf, proposal="cluster-update", sweeps=1.5)
    make_mcmc(wf, proposal="cluster-update", sweeps=1.5, sweep_type="random")
    _, width = make_mcmc(wf, proposal="single-electron", init_width=0.5, jump_steps=20)
    assert width == 0.5


def test_width_scheduler_mirrors_reference():
    """make_width_scheduler (mcmc.py:349-378): every window_size updates (the first included) the width shrinks by the
    multiplier when the ring's mean acceptance, taken before the new rate is stored, is below target - error, grows
    when above target + error and stays otherwise; the first update sees the zero ring and shrinks."""
    from sparse_wf_gb300.wavefunction import make_width_scheduler

    init, update = make_width_scheduler(window_size=3, target_pmove=0.5, error=0.025, width_multiplier=2.0)
    s = init(0.8)
    widths = []
    for pm in [0.9, 0.9, 0.9, 0.9, 0.1, 0.1, 0.1, 0.5, 0.5, 0.5]:
        s = update(s, pm)
        widths.append(float(s.width))
    # update 0: zero ring -> 0.4; updates 3, 6, 9 see the means of (0.9, 0.9, 0.9), (0.9, 0.1, 0.1), (0.1, 0.5, 0.5)
    np.testing.assert_array_equal(np.float32(widths),
                                  np.float32([0.4, 0.4, 0.4, 0.8, 0.8, 0.8, 0.4, 0.4, 0.4, 0.2]))
    assert s.i == 10 and s.width.dtype == np.float32


class _FakeLowRankLib:
    """Stands in for libfire.so in the low-rank wrapper's host logic: a changed set of `need` electrons per step
    (FIRE_FLAG_CHANGED_OVERFLOW below that capacity) and, optionally, one pair-capacity overflow first."""

    def __init__(self, need, pair_overflow=False):
        self.need, self.pair_overflow, self.calls = need, pair_overflow, []

    def fire_prepared_size(self, prob, nbytes):
        nbytes._obj.value = 64
        return 0

    def fire_prepare_params(self, *args):
        return 0

    def fire_low_rank_workspace_size(self, prob, chunk, cap, nbytes):
        nbytes._obj.value = 1024 * int(cap)
        return 0

    def fire_mcmc_low_rank_block(self, stream, prob, R, Z, prepared, r, logpsi, steps, off, width, cap, seed, counter,
                                 noise, logu, n_acc, smax, ws, ws_bytes, status):
        pr = prob._obj
        n3 = pr.n_walkers * pr.n_el * 3
        rv = (C.c_float * n3).from_address(r.value)
        self.calls.append((int(cap), int(pr.cap_pairs), float(rv[0])))
        rv[0] += 1.0  # the block moves the walkers in place: a rerun must start from the original positions
        st = (C.c_int32 * _lib.STATUS_WORDS).from_address(status.value)
        if self.pair_overflow and len(self.calls) == 1:
            st[0] |= _lib.FLAG_PAIR_OVERFLOW
            st[1] = 4 * pr.cap_pairs
            return 0
        if cap < self.need:
            st[0] |= _lib.FLAG_CHANGED_OVERFLOW
            st[4] = self.need
            return 0
        sm = (C.c_int32 * 7).from_address(smax.value)
        for k, v in enumerate([1, 2, 0, 3, self.need, 20, 21]):
            sm[k] = v
        na = (C.c_int32 * pr.n_walkers).from_address(n_acc.value)
        for k in range(pr.n_walkers):
            na[k] = 5
        return 0


def _fake_wf(monkeypatch, fake):
    import torch

    from sparse_wf_gb300.wavefunction import FireWaveFunction

    monkeypatch.setattr(_lib, "load", lambda: fake)
    mol = systems.alkane(2)
    wf = FireWaveFunction(mol, precision="fp32", device="cpu")
    wf._stream = lambda: None
    r = torch.from_numpy(systems.init_electrons(mol, 2, 5)).contiguous()
    return wf, mol, r


def test_low_rank_wrapper_reruns_and_grows_capacities(monkeypatch):
    """mcmc_low_rank_block's host logic: a changed-set overflow reruns the block from the original walkers and
    log|psi| with the set the device reported (padded by 10 %, capped at the electron count), the capacity is kept
    for the next call, a pair overflow grows the neighbour capacity first, and the 7 static words come back as
    (StaticArgs, move statics)."""
    import torch

    from sparse_wf_gb300.wavefunction import StaticArgs

    fake = _FakeLowRankLib(need=14, pair_overflow=True)
    wf, mol, r = _fake_wf(monkeypatch, fake)
    params = P.init_params(wf.dims, 0)
    r0 = float(r[0, 0, 0])
    lp = torch.zeros(2)
    n_acc, smax, changed = wf.mcmc_low_rank_block(params, r, lp, StaticArgs(40, 40, 0, 8), 5, 0.5, cap_changed=4)
    caps, pairs, starts = zip(*fake.calls)
    assert caps == (4, 4, 16) and pairs[1] > pairs[0]
    assert all(x == r0 for x in starts)
    assert wf._lr_cap == 16 and changed == (14, 20, 21) and tuple(smax.__dict__.values()) == (1, 2, 0, 3)
    assert n_acc.tolist() == [5, 5]
    fake.calls.clear()
    fake.pair_overflow = False
    wf.mcmc_low_rank_block(params, r, lp, StaticArgs(40, 40, 0, 8), 5, 0.5)
    assert [c[0] for c in fake.calls] == [16]


def test_low_rank_wrapper_rejects_sets_beyond_the_limit(monkeypatch):
    """A changed set larger than the electron count allows (here all 18 electrons are the limit) raises instead of
    rerunning forever."""
    import torch

    from sparse_wf_gb300.wavefunction import StaticArgs

    fake = _FakeLowRankLib(need=30)
    wf, mol, r = _fake_wf(monkeypatch, fake)
    with pytest.raises(RuntimeError, match="limit of 18"):
        wf.mcmc_low_rank_block(P.init_params(wf.dims, 0), r, torch.zeros(2), StaticArgs(40, 40, 0, 8), 5, 0.5)


def test_low_rank_jump_and_ecp_argument_checks(lib):
    """fire_mcmc_low_rank_jump_block and fire_ecp_energy reject bad arguments before any CUDA call, through the
    declared ctypes signatures (pointers never dereferenced): a non-positive sigma, a zero or too large capacity,
    a missing or malformed fire_ecp (more than 4 non-local channels, a quadrature above 12 points, a one-point grid)."""
    prob = _lib.Problem(82, 41, 32, 4, 5.0, 20.0, 2500, 40, 0, 0)
    d = C.c_void_p(16)

    def jump(sigma, cap):
        return lib.fire_mcmc_low_rank_jump_block(None, C.byref(prob), d, d, d, d, d, 4, sigma, cap, 0, 0, None, None,
                                                 None, None, d, C.c_size_t(1), d)

    assert jump(0.0, 32) == 1 and jump(2.0, 0) == 1 and jump(2.0, 129) == 2

    def ecp(**kw):
        f = dict(n_ecp=2, n_grid=100, n_l=2, max_quad=4)
        f.update(kw)
        e = _lib.Ecp(f["n_ecp"], f["n_grid"], f["n_l"], f["max_quad"], d, d, d, d, d, d)
        return lib.fire_ecp_energy(None, C.byref(prob), d, d, d, d, C.byref(e), 32, 0, 0, None, d, None, d,
                                   C.c_size_t(1), d)

    assert lib.fire_ecp_energy(None, C.byref(prob), d, d, d, d, None, 32, 0, 0, None, d, None, d, C.c_size_t(1),
                               d) == 1
    assert ecp(n_l=5) == 1 and ecp(max_quad=13) == 1 and ecp(n_grid=1) == 1 and ecp(n_ecp=0) == 1


def test_low_rank_cluster_argument_checks(lib):
    """fire_mcmc_low_rank_cluster_block rejects, before any CUDA call and through its ctypes signature, a zero
    capacity, a negative radius, half a replay (1), and a cluster above 16 electrons or a capacity above 128 (2)."""
    prob = _lib.Problem(82, 41, 32, 4, 5.0, 20.0, 2500, 40, 0, 0)
    d = C.c_void_p(16)

    def call(k=5, radius=2.0, cap=32, draws=None, logu=None):
        return lib.fire_mcmc_low_rank_cluster_block(None, C.byref(prob), d, d, d, d, d, 4, 0, 0.2, k, radius, 0, cap,
                                                    0, 0, draws, logu, None, None, d, C.c_size_t(1), d)

    assert call(cap=0) == 1 and call(radius=-1.0) == 1 and call(draws=d) == 1
    assert call(k=17) == 2 and call(cap=129) == 2


def test_checkpoint_round_trip_and_reference_mapping(tmp_path):
    """checkpoint.save / load keep every parameter slot, the walkers, the width scheduler's state and the step;
    load_reference_params reads an expanded checkpoint (leaf paths joined by "/", loggers.py:191-208) through an
    explicit mapping, applies per-leaf transforms, checks shapes and reports unmapped leaves."""
    from sparse_wf_gb300 import checkpoint
    from sparse_wf_gb300.wavefunction import make_width_scheduler

    mol = systems.alkane(2)
    nu, _ = systems.spin_counts(mol)
    dims = P.ModelDims(mol.n_el, nu, mol.n_nuc)
    p = P.init_params(dims, 3)
    r = systems.init_electrons(mol, 4, 2)
    init, update = make_width_scheduler(window_size=3)
    ws = update(update(init(0.4), 0.6), 0.7)
    checkpoint.save(str(tmp_path / "c.npz"), p, r, ws, 17)
    back = checkpoint.load(str(tmp_path / "c.npz"), dims)
    for k in p:
        np.testing.assert_array_equal(back["params"][k], p[k])
    np.testing.assert_array_equal(back["electrons"], r)
    assert back["step"] == 17 and back["width_state"] == ws
    # an expanded reference checkpoint with made-up leaf paths; one stored transposed, one extra leaf
    leaves = {f"embedding/{k}": v for k, v in p.items()}
    leaves["embedding/orb_up_W"] = p["orb_up_W"].T
    leaves["opt/unused"] = np.zeros(3)
    (tmp_path / "ref").mkdir()
    np.savez(tmp_path / "ref" / "params.npz", **leaves)
    mapping = {k: f"embedding/{k}" for k in p}
    mapping["orb_up_W"] = ("embedding/orb_up_W", np.transpose)
    got = checkpoint.load_reference_params(str(tmp_path / "ref"), dims, mapping)
    for k in p:
        np.testing.assert_array_equal(got["params"][k], p[k])
    assert got["unused_leaves"] == ["opt/unused"]
    with pytest.raises(ValueError):
        checkpoint.load_reference_params(str(tmp_path / "ref"), dims, {**mapping, "orb_up_W": "embedding/orb_up_W"})
    with pytest.raises(KeyError):
        checkpoint.load_reference_params(str(tmp_path / "ref"), dims, {k: v for k, v in mapping.items()
                                                                         if k != "cusp"})


def _reference_tree(p):
    """The nested leaf dict of a reference MoonLikeParams built from parameter slots through REFERENCE_LEAVES
    (scalar slots split into their scalar leaves, stored with shape ())."""
    from sparse_wf_gb300.checkpoint import REFERENCE_LEAVES

    flat = {}
    for slot, src in REFERENCE_LEAVES.items():
        if isinstance(src, tuple):
            for q, v in zip(src, np.asarray(p[slot]).reshape(-1)):
                flat[q] = np.asarray(v, np.float32).reshape(())
        else:
            flat[src] = np.asarray(p[slot], np.float32)
    tree = {}
    for path, v in flat.items():
        node = tree
        *head, leaf = path.split("/")
        for h in head:
            node = node.setdefault(h, {})
        node[leaf] = v
    return flat, tree


def test_reference_checkpoint_default_mapping_npz_and_msgpack(tmp_path):
    """The default leaf mapping reads an expanded params.npz (tree_to_flat_dict paths, loggers.py:191-208) and a flax
    msgpack TrainingState (api.py:294-331) written with flax's extension types (1 = ndarray, 3 = numpy scalar) into
    the same parameter slots; extra optimizer leaves are reported, a wrong shape raises."""
    from sparse_wf_gb300 import checkpoint, params as P

    dims = P.ModelDims(6, 3, 4)
    p = P.init_params(dims, 3)
    p["scales"] = np.array([0.7, 1.3])
    flat, tree = _reference_tree(p)
    (tmp_path / "exp").mkdir()
    np.savez(tmp_path / "exp" / "params.npz", **flat)
    got = checkpoint.load_reference_params(str(tmp_path / "exp"), dims)
    for k in p:
        np.testing.assert_array_equal(got["params"][k], np.asarray(p[k], np.float32).astype(np.float64), err_msg=k)
    assert got["unused_leaves"] == []
    msgpack = pytest.importorskip("msgpack")

    def ext(o):
        if isinstance(o, np.ndarray):
            return msgpack.ExtType(1, msgpack.packb((o.shape, o.dtype.name, o.tobytes("C")), use_bin_type=True))
        if isinstance(o, np.generic):
            return msgpack.ExtType(3, msgpack.packb((o.dtype.name, o.tobytes()), use_bin_type=True))
        raise TypeError(type(o))

    r = np.random.default_rng(0).standard_normal((5, 6, 3)).astype(np.float32)
    state = {"key": np.array([0, 42], np.uint32), "params": tree, "electrons": r,
             "opt_state": {"natgrad": {"last_grad": np.zeros(7, np.float32)}}, "step": np.int64(123),
             "width_state": {"width": np.float32(0.1), "pmoves": np.zeros(20, np.float32), "i": 3}}
    (tmp_path / "chkpt000123.msgpk").write_bytes(msgpack.packb(state, default=ext, use_bin_type=True))
    got = checkpoint.load_reference_msgpack(str(tmp_path / "chkpt000123.msgpk"), dims)
    for k in p:
        np.testing.assert_array_equal(got["params"][k], np.asarray(p[k], np.float32).astype(np.float64), err_msg=k)
    np.testing.assert_array_equal(got["electrons"], r)
    assert got["step"] == 123 and got["unused_leaves"] == []
    leaves = checkpoint.read_reference_msgpack(str(tmp_path / "chkpt000123.msgpk"))
    assert leaves["width_state/i"] == 3 and leaves["opt_state/natgrad/last_grad"].shape == (7,)
    bad = dict(flat)
    bad["to_orbitals/params/to_orbitals_up/kernel"] = np.zeros((3, 3), np.float32)
    (tmp_path / "bad").mkdir()
    np.savez(tmp_path / "bad" / "params.npz", **bad)
    with pytest.raises(ValueError):
        checkpoint.load_reference_params(str(tmp_path / "bad"), dims)


def test_ragged_autotuner_selection(monkeypatch):
    """ragged.Autotuner without a GPU (RaggedBatch and the CUDA calls faked): candidates whose workspaces exceed the
    HBM budget are not built, the fastest of the rest is kept per batch signature (a second call is a cache hit),
    and no fitting candidate raises."""
    from sparse_wf_gb300 import ragged

    built, clock = [], [0.0]
    cost = {(1, 64): 3.0, (2, 64): 1.0, (4, 64): 2.0}

    class FakeBatch:
        def __init__(self, mols, walkers, precision, lanes, chunk, device):
            self.key = (lanes, chunk)
            built.append(self.key)

        def workspace_bytes(self):
            return [10e9 * self.key[0]]

        def run(self):
            pass

        def replay(self):
            clock[0] += cost[self.key]

    monkeypatch.setattr(ragged, "RaggedBatch", FakeBatch)
    monkeypatch.setattr(ragged.time, "perf_counter", lambda: clock[0])
    monkeypatch.setattr(ragged.torch.cuda, "synchronize", lambda *a: None)
    monkeypatch.setattr(ragged.torch.cuda, "empty_cache", lambda *a: None)
    tuner = ragged.Autotuner(candidates=[(1, 64), (2, 64), (4, 64), (8, 32)], budget_bytes=45e9, reps=2)
    mols = [systems.alkane(2), systems.alkane(3)]
    best = tuner.tune(mols, [64, 128])
    assert (best["lanes"], best["chunk"]) == (2, 64) and best["seconds"] == 1.0
    assert [t["lanes"] for t in best["trials"]] == [1, 2, 4]  # 8 lanes (80 GB) exceeds the budget
    n_built = len(built)
    assert tuner.tune(mols, [64, 128]) is best and len(built) == n_built
    with pytest.raises(RuntimeError):
        ragged.Autotuner(candidates=[(8, 32)], budget_bytes=45e9).tune(mols, [64, 128])


def test_serving_loop_admission_retry_and_completion():
    """ServingEngine.run's host loop without a GPU (launch, completion and workspace faked): requests are admitted in
    arrival order to free slots, a request whose state would exceed the HBM budget waits until memory is released, a
    capacity overflow sends its request back to the front of the queue with grown capacities, and every request
    completes once with its latency recorded."""
    from sparse_wf_gb300 import serving
    from sparse_wf_gb300.wavefunction import StaticArgs

    class Event:
        def __init__(self, ready):
            self.ready = ready

        def query(self):
            return self.ready()

    class FakeModel:
        static = StaticArgs(10, 10, 0, 4)

    class Engine(serving.ServingEngine):
        def __init__(self):
            self.lanes, self.budget, self.in_use, self.max_walkers, self.ws_bytes = 2, 3000.0, 0, 4096, 1 << 30
            self.log, self.overflowed, self.peak = [], set(), 0

        def model(self, n_carbon):
            return FakeModel()

        def warm(self, trace):
            pass

        def _ws_need(self, m, walkers, static):
            return 1

        def _state_bytes(self, req, m):
            return req.walkers

        def _launch(self, req, lane, static, now):
            self.log.append((req.rid, lane, static.n_pairs_same))
            self.peak = max(self.peak, self.in_use)
            t0 = serving.time.perf_counter()
            return serving._Active(req, lane, static, req.walkers, None, None, None, None, None, None, {},
                                   Event(lambda: serving.time.perf_counter() - t0 > 0.01))

        def _finish(self, a, now):
            if a.req.rid == 1 and a.req.rid not in self.overflowed:
                self.overflowed.add(a.req.rid)
                return StaticArgs(20, 20, 0, 6)
            a.req.done = now
            return None

    trace = [serving.Request(rid=i, kind="eloc", n_carbon=4, walkers=w, arrival=0.0)
             for i, w in enumerate([1000, 1500, 2000, 500])]
    eng = Engine()
    eng.run(trace, timeout=30.0)
    assert [rid for rid, _, _ in eng.log[:2]] == [0, 1]
    assert eng.peak <= 3000  # the 2000-walker request waited for memory
    retried = [x for x in eng.log if x[0] == 1]
    assert len(retried) == 2 and retried[1][2] == 20 and trace[1].retries == 1
    assert all(np.isfinite(r.done) and r.done >= r.arrival for r in trace) and len(eng.log) == 5


def test_bench_reference_arm_json_contract():
    """bench.py --impl reference (the CPU arm: the oracle port on bounded samples) prints one JSON line with the
    contract's keys, impl "reference", a cpu_baseline describing the run and an e2e object without host-device bytes."""
    import json
    import subprocess
    import sys

    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--system", "c2h6",
                          "--steps", "1", "--warmup", "0", "--cpu-sample", "1", "--walkers", "64"],
                         capture_output=True, text=True, timeout=600, cwd=str(ROOT))
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
                "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["value"] > 0 and d["steps"] == 1
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    # the same workload description as the GPU arm's line, and the Metropolis block replayed before the steps
    import argparse

    import bench
    from sparse_wf_gb300 import systems

    args = argparse.Namespace(walkers=64, gpus=1, mcmc_steps=20, mcmc_width=0.1)
    assert d["config"] == bench.workload_config(args, systems.alkane(2))
    assert "Metropolis block replayed" in d["cpu_baseline"]["sample"]
    assert abs(d["ms_per_step"] / 1e3 - d["cpu_baseline"]["cores"] / d["value"]) < 1e-9


def test_low_rank_pass_size_from_its_own_workspace(monkeypatch):
    """The low-rank blocks size their walkers per pass from their own workspace, not the local energy's pass: as many
    walkers as lr_ws_gb holds at the block's per-walker size (the fake library's workspace grows by 1000 bytes per
    walker and changed-set slot), or lr_chunk_walkers when set; the workspace is requested for that pass."""
    import torch

    from sparse_wf_gb300.wavefunction import StaticArgs

    class Fake(_FakeLowRankLib):
        def __init__(self):
            super().__init__(need=1)
            self.sizes = []

        def fire_low_rank_workspace_size(self, prob, chunk, cap, nbytes):
            self.sizes.append(int(chunk))
            nbytes._obj.value = 1000 * int(chunk) * int(cap)
            return 0

        def fire_mcmc_low_rank_block(self, stream, prob, *args):
            self.calls.append(int(prob._obj.chunk_walkers))
            return 0

    fake = Fake()
    wf, mol, _ = _fake_wf(monkeypatch, fake)
    r = torch.from_numpy(systems.init_electrons(mol, 7, 5)).contiguous()
    lp = torch.zeros(7)
    wf.chunk_walkers = 2  # the local energy's pass: not the low-rank block's
    wf.lr_ws_gb = 25e-6   # 25 kB: 6 walkers at 4 changed-set slots
    wf.mcmc_low_rank_block(P.init_params(wf.dims, 0), r, lp, StaticArgs(40, 40, 0, 8), 1, 0.3, cap_changed=4)
    assert fake.calls == [6] and fake.sizes[-1] == 6
    wf.lr_chunk_walkers = 3
    wf.mcmc_low_rank_block(P.init_params(wf.dims, 0), r, lp, StaticArgs(40, 40, 0, 8), 1, 0.3, cap_changed=4)
    assert fake.calls[-1] == 3 and fake.sizes[-1] == 3


def test_ecp_energy_wrapper_reruns(monkeypatch):
    """FireWaveFunction.ecp_energy's host loop against a fake library: a changed-set overflow reruns with the set the
    device reported, a pair overflow first grows the neighbour capacity, and the energies and move statics come back
    from the last call."""
    import torch

    from sparse_wf_gb300.ecp import EcpTables
    from sparse_wf_gb300.wavefunction import StaticArgs

    class Fake(_FakeLowRankLib):
        def fire_ecp_energy(self, stream, prob, R, Z, prepared, r, ecp, cap, seed, counter, rot, out, smax, ws, wsb,
                            status):
            pr = prob._obj
            self.calls.append((int(cap), int(pr.cap_pairs), ecp._obj.n_ecp, ecp._obj.max_quad))
            st = (C.c_int32 * _lib.STATUS_WORDS).from_address(status.value)
            if self.pair_overflow and len(self.calls) == 1:
                st[0] |= _lib.FLAG_PAIR_OVERFLOW
                st[1] = 4 * pr.cap_pairs
                return 0
            if cap < self.need:
                st[0] |= _lib.FLAG_CHANGED_OVERFLOW
                st[4] = self.need
                return 0
            o = (C.c_float * pr.n_walkers).from_address(out.value)
            for k in range(pr.n_walkers):
                o[k] = 1.5 + k
            sm = (C.c_int32 * 7).from_address(smax.value)
            for k, v in enumerate([0, 0, 0, 0, self.need, 7, 8]):
                sm[k] = v
            return 0

    fake = Fake(need=12, pair_overflow=True)
    wf, mol, r = _fake_wf(monkeypatch, fake)
    carbon = (2, [(-1, [[], [(14.0, 4.0)]]), (0, [[], [], [(7.0, 50.0)]])])
    tables = EcpTables(systems.alkane(2).Z, {6: carbon}, n_quad={6: 4})
    out, changed = wf.ecp_energy(P.init_params(wf.dims, 0), r, StaticArgs(40, 40, 0, 8), tables.device("cpu"),
                                 cap_changed=4)
    caps, pairs, n_ecp, qmax = zip(*fake.calls)
    assert caps == (4, 4, 14) and pairs[1] > pairs[0] and set(n_ecp) == {2} and set(qmax) == {4}
    assert out.tolist() == [1.5, 2.5] and changed == (12, 7, 8) and wf._lr_cap == 14


def test_bench_config_segments_with_a_fake_wavefunction(monkeypatch):
    """bench.config_segments (C1: H10 x 512, FP32 and FP64; C2: C10H22 x 4096, mixed and FP32, each against the FP64
    build) driven on the CPU by a stand-in wavefunction whose E_loc is a fixed function of the walkers plus a
    per-precision offset, and by stand-ins for the device timer and the workspace-sized pass: the segment's own
    bookkeeping (which walkers, which reference, the error and ratio entries) is what is checked."""
    import argparse

    import torch

    import bench
    from sparse_wf_gb300 import wavefunction

    offset = {"fp64": 0.0, "fp32": 2e-6, "mixed": -3e-6}
    calls = []

    class FakeStatic:
        n_pairs = 2200

        def round_with_padding(self, *a):
            return self

    class FakeWF:
        def __init__(self, mol, precision, device):
            self.mol, self.precision, self.chunk_walkers = mol, precision, 0

        def init(self, seed, r):
            assert seed == 0 and r.shape[0] == 1
            return {"seeded": True}

        def get_static_input(self, r):
            return FakeStatic()

        def _params(self, p):
            assert p == {"seeded": True}
            return p

        def local_energy_full(self, dp, r, static):
            assert r.dtype == (torch.float64 if self.precision == "fp64" else torch.float32)
            calls.append((self.mol.name, self.precision, r.shape[0], self.chunk_walkers))
            e = r.double().sum(dim=(1, 2)) + offset[self.precision]
            return e, {"static": static, "refined": 1, "stats": torch.zeros(2)}

    monkeypatch.setattr(wavefunction, "FireWaveFunction", FakeWF)
    monkeypatch.setattr(bench, "choose_chunk", lambda wf, nw, static, ws_gb: nw // 2)

    def fake_time(step, n, stream, dist, world):
        out = None
        for _ in range(n):
            out = step()
        return 2.0, out

    monkeypatch.setattr(bench, "time_steps", fake_time)
    args = argparse.Namespace(steps=2, warmup=1, ws_gb=48.0)
    out = bench.config_segments(args, torch.device("cpu"), None)
    c1, c2 = out["C1"], out["C2"]
    assert c1["walkers"] == 512 and c1["n_el"] == 10 and c1["error_walkers"] == 512
    assert set(c1) >= {"fp32", "fp64"} and "mixed" not in c1 and "mixed_over_fp32" not in c1
    assert c1["fp32"]["value"] == 512 / 2e-3 and c1["fp32"]["refined_walkers"] == 1
    assert abs(c1["fp32"]["error_vs_fp64"]["mean_energy_err_mHa"] - 2e-3) < 1e-9
    assert "error_vs_fp64" not in c1["fp64"]
    assert c2["walkers"] == 4096 and c2["n_el"] == 82 and c2["error_walkers"] == 1024
    assert abs(c2["mixed"]["error_vs_fp64"]["max_abs_mHa"] - 3e-3) < 1e-9
    assert abs(c2["mixed_over_fp32"] - 1.0) < 1e-12 and "fp64" not in c2
    # the timed paths run warm-up + timed steps on every walker in workspace-sized passes; C2's FP64 reference runs
    # once on the first 1024 walkers in passes of 64
    c2_calls = [c for c in calls if c[0] == c2["molecule"]]
    assert [c for c in c2_calls if c[1] == "fp64"] == [(c2["molecule"], "fp64", 1024, 64)]
    # C2's passes: the workspace would allow 2048 walkers, the launch grid's 65535 row tiles of 64 allow 612
    assert 65535 * 64 // (3 * (82 + 2200)) == 612
    assert sum(1 for c in c2_calls if c[1] == "mixed") == 3 and all(c[2:] == (4096, 612) for c in c2_calls
                                                                      if c[1] != "fp64")
    assert all(c[3] == 256 for c in calls if c[0] == c1["molecule"])  # C1: the workspace's 512 // 2
