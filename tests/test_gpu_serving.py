"""Ragged multi-molecule batches (one CUDA-graph launch) and the serving loop: every result is the same alone
and in the mix.

Tolerances: the value path (log|psi|, Metropolis decisions) is deterministic, so MCMC-block results must be
identical; local energies are compared statistically because the per-center sums of
squared Jacobian rows are accumulated with atomics, whose order varies from run to run: median relative
difference <= 1e-6, maximum <= 1e-3 (relative to max(1, |E|))."""
import numpy as np
import pytest
import torch

from sparse_wf_gb300 import systems
from sparse_wf_gb300.ragged import Autotuner, RaggedBatch, ragged_alkanes
from sparse_wf_gb300.serving import Request, ServingEngine
from sparse_wf_gb300.wavefunction import FireWaveFunction

pytestmark = pytest.mark.gpu


def _close(a, b):
    """Local energies of the same walkers: the run-to-run spread of the atomic accumulations (amplified on
    ill-conditioned walkers) stays far below the O(1) errors a mixed-up request would show."""
    rel = np.abs(a - b) / np.maximum(1.0, np.abs(b))
    return np.median(rel) < 1e-6 and rel.max() < 1e-3


@pytest.mark.parametrize("precision", ["fp32", "mixed"])
def test_ragged_graph_matches_per_molecule_calls(cuda_lib, precision):
    ns, ws = ragged_alkanes(5, (1, 5), (8, 40), seed=3)
    mols = [systems.alkane(n) for n in ns]
    batch = RaggedBatch(mols, ws, precision, lanes=2, chunk=16)
    batch.run_eager()
    eager = batch.results()
    batch.run()  # capture + one graph launch
    graph = batch.results()
    batch.replay()
    torch.cuda.synchronize()
    again = batch.results()
    for k, (mol, e, g, a) in enumerate(zip(mols, eager, graph, again)):
        assert np.all(np.isfinite(g))
        assert _close(g, e), k
        assert _close(a, g), k
        # the wavefunction's own entry point on the same walkers and parameters (the batch runs without the
        # refinement pass of ill-conditioned walkers, so the comparison does too)
        j = batch.jobs[k]
        j.wf.refine = False
        ref, _ = j.wf.local_energy_full(j.params, j.r, j.static)
        assert _close(g, ref.double().cpu().numpy()), k


def test_autotuner_picks_a_fitting_candidate(cuda_lib):
    ns, ws = ragged_alkanes(4, (1, 4), (8, 24), seed=9)
    mols = [systems.alkane(n) for n in ns]
    tuner = Autotuner(candidates=((1, 16), (2, 16), (2, 8)), budget_bytes=40e9, reps=1)
    best = tuner.tune(mols, ws, "fp32")
    assert (best["lanes"], best["chunk"]) in {(1, 16), (2, 16), (2, 8)}
    assert len(best["trials"]) == 3 and best["seconds"] == min(t["seconds"] for t in best["trials"])
    assert tuner.tune(mols, ws, "fp32") is best  # cached per batch signature


@pytest.mark.parametrize("precision", ["fp32", "mixed"])
def test_serving_results_same_alone_and_in_the_mix(cuda_lib, precision):
    trace = [Request(0, "eloc", 3, 40, 0.000, seed=11), Request(1, "mcmc", 2, 24, 0.001, steps=6, seed=12),
             Request(2, "eloc", 5, 32, 0.002, seed=13), Request(3, "mcmc", 4, 48, 0.002, steps=6, seed=14),
             Request(4, "eloc", 2, 16, 0.003, seed=15), Request(5, "mcmc", 5, 16, 0.004, steps=6, seed=16)]
    eng = ServingEngine(precision, lanes=3, chunk=16, max_carbon=5, max_walkers=64)
    m = eng.run(trace)
    assert m["requests"] == 6 and m["p99_ms"] >= m["p50_ms"] > 0
    # the requests really overlapped: at least one was admitted before another one finished
    assert any(b.admitted < a.done and b.rid != a.rid for a in trace for b in trace)
    for req in trace:
        solo = Request(req.rid, req.kind, req.n_carbon, req.walkers, 0.0, steps=req.steps, seed=req.seed)
        ServingEngine(precision, lanes=1, chunk=16, max_carbon=5, max_walkers=64).run([solo])
        if req.kind == "mcmc":
            np.testing.assert_array_equal(req.n_accept, solo.n_accept)
            np.testing.assert_array_equal(req.logpsi, solo.logpsi)
        else:
            assert _close(req.eloc, solo.eloc), req.rid
    # an E_loc request equals the wavefunction's own evaluation of the same walkers
    req = trace[0]
    mol = systems.alkane(req.n_carbon)
    wf = FireWaveFunction(mol, precision=precision)
    wf.refine = False  # the serving engine's evaluations run without the refinement pass
    params = wf.init(0, systems.init_electrons(mol, 64, 77)[:1])
    r = systems.init_electrons(mol, req.walkers, req.seed)
    e, _ = wf.local_energy_full(params, r, eng.models[req.n_carbon].static)
    assert _close(req.eloc, e.double().cpu().numpy())
