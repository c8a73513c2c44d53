"""Ragged multi-molecule batches: the local energies of many molecules of different sizes in one CUDA-graph
launch.

The workload: walkers of many molecules with uneven electron and neighbour counts (for example 64 alkanes
C_nH_2n+2 with n drawn from 2..40 and 64..1024 walkers each) evaluated together.  The entry points of
``libfire.so`` take device pointers and a stream and neither allocate nor synchronise, so the
``fire_local_energy`` calls of a whole batch -- one per molecule, spread over S stream lanes -- are
captured once into a CUDA graph and replayed with a single launch.  The walkers, parameters, static
capacities and outputs of every molecule stay resident; each lane owns one workspace sized for the largest
molecule placed on it (molecules of one lane run one after another and share it).

``Autotuner`` picks the launch shape of a batch -- the number of lanes and the walkers per internal chunk
-- by timing replays of the candidates that fit the HBM budget.

Capacities follow the library's rule: a replay that overflows a capacity sets the status flag; ``run``
grows the capacities from the observed maxima, re-captures and replays again (like the reference's
StaticScheduler, ``static_args.py:62-84``).
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import time
from typing import Optional, Sequence

import numpy as np
import torch

from . import _lib, systems
from .wavefunction import DeviceParams, FireWaveFunction, StaticArgs


def ragged_alkanes(n_molecules: int = 64, n_range=(2, 40), walker_range=(64, 1024), seed: int = 4):
    """Molecule sizes and walker counts of a ragged batch (numpy default_rng(seed), uniform draws)."""
    rng = np.random.default_rng(seed)
    ns = rng.integers(n_range[0], n_range[1] + 1, size=n_molecules)
    ws = rng.integers(walker_range[0], walker_range[1] + 1, size=n_molecules)
    return [int(x) for x in ns], [int(x) for x in ws]


@dataclasses.dataclass
class _Job:
    wf: FireWaveFunction
    params: DeviceParams
    r: torch.Tensor
    static: StaticArgs
    eloc: torch.Tensor
    logpsi: torch.Tensor
    sign: torch.Tensor
    stats: torch.Tensor
    status: torch.Tensor
    lane: int = 0
    cost: float = 0.0


class RaggedBatch:
    """Local energies of molecules ``mols`` with ``walkers[i]`` walkers each (initial positions drawn around the
    nuclei, seed ``1000 + i``), parameters initialised from ``params_seed`` for every molecule."""

    def __init__(self, mols: Sequence[systems.Molecule], walkers: Sequence[int], precision: str = "mixed",
                 lanes: int = 4, chunk: int = 64, params_seed: int = 0, device: str | torch.device = "cuda"):
        self.device = torch.device(device)
        self.precision = precision
        self.lanes = max(1, int(lanes))
        self.chunk = max(1, int(chunk))
        self.jobs: list[_Job] = []
        for i, (mol, B) in enumerate(zip(mols, walkers)):
            wf = FireWaveFunction(mol, precision=precision, device=self.device, chunk_walkers=self.chunk)
            r_np = systems.init_electrons(mol, int(B), 1000 + i)
            params = wf._params(wf.init(params_seed, r_np[:1]))
            wf._ws = None  # the initialiser's scratch; the batch runs in the lane workspaces
            r = wf._electrons(r_np)
            nu, _ = systems.spin_counts(mol)
            static = wf.get_static_input(r).round_with_padding(1.1, mol.n_el, nu, mol.n_nuc)
            dev = dict(dtype=wf.dtype, device=self.device)
            self.jobs.append(_Job(wf, params, r, static, torch.empty(B, **dev), torch.empty(B, **dev),
                                  torch.empty(B, **dev), torch.empty(2, dtype=torch.float64, device=self.device),
                                  torch.zeros(_lib.STATUS_WORDS, dtype=torch.int32, device=self.device),
                                  cost=float(B) * mol.n_el * mol.n_el))
        # longest-processing-time-first assignment of molecules to lanes
        load = [0.0] * self.lanes
        for j in sorted(self.jobs, key=lambda j: -j.cost):
            k = int(np.argmin(load))
            j.lane = k
            load[k] += j.cost
        self.streams = [torch.cuda.Stream(self.device) for _ in range(self.lanes)]
        self._ws: list[Optional[torch.Tensor]] = [None] * self.lanes
        self.graph: Optional[torch.cuda.CUDAGraph] = None
        self._alloc_workspaces()

    # ------------------------------------------------------------------ plumbing
    def _problem(self, j: _Job) -> _lib.Problem:
        return j.wf._problem(j.r.shape[0], j.static)

    def workspace_bytes(self) -> list[int]:
        lib = _lib.load()
        need = [0] * self.lanes
        for j in self.jobs:
            nb = C.c_size_t()
            _lib.check(lib.fire_workspace_size(C.byref(self._problem(j)), self.chunk, C.byref(nb)),
                       "fire_workspace_size")
            need[j.lane] = max(need[j.lane], int(nb.value))
        return need

    def _alloc_workspaces(self):
        for k, b in enumerate(self.workspace_bytes()):
            if self._ws[k] is None or self._ws[k].numel() < b:
                self._ws[k] = None
                self._ws[k] = torch.empty(max(b, 1), dtype=torch.uint8, device=self.device)

    def _call(self, j: _Job, stream: torch.cuda.Stream, ws: Optional[torch.Tensor] = None):
        ws = self._ws[j.lane] if ws is None else ws
        prob = self._problem(j)
        prob.chunk_walkers = 0  # smaller molecules of a lane take more walkers per pass in the same workspace
        with torch.cuda.stream(stream):
            j.status.zero_()
        _lib.check(_lib.load().fire_local_energy(
            C.c_void_p(stream.cuda_stream), C.byref(prob), C.c_void_p(j.wf.R_dev.data_ptr()),
            C.c_void_p(j.wf.Z_dev.data_ptr()), C.c_void_p(j.params.prepared.data_ptr()), C.c_void_p(j.r.data_ptr()),
            C.c_void_p(j.logpsi.data_ptr()), C.c_void_p(j.sign.data_ptr()), C.c_void_p(j.eloc.data_ptr()),
            C.c_void_p(j.stats.data_ptr()), None, C.c_void_p(ws.data_ptr()), C.c_size_t(ws.numel()),
            C.c_void_p(j.status.data_ptr())), "fire_local_energy")

    def _grow(self) -> bool:
        """Grows the capacities of every job whose status reports an overflow; True if any grew."""
        grew = False
        for j in self.jobs:
            st = j.status.cpu().numpy()
            if st[0] & (_lib.FLAG_PAIR_OVERFLOW | _lib.FLAG_NUC_OVERFLOW):
                mol = j.wf.mol
                nu, _ = systems.spin_counts(mol)
                j.static = j.wf.get_static_input(j.r).round_with_padding(1.25, mol.n_el, nu, mol.n_nuc)
                grew = True
        if grew:
            self._alloc_workspaces()
            self.graph = None
        return grew

    # ------------------------------------------------------------------ execution
    def run_eager(self):
        """One ``fire_local_energy`` call per molecule, one after another on the current stream (no graph)."""
        s = torch.cuda.current_stream(self.device)
        for _ in range(4):
            ws = max((w for w in self._ws if w is not None), key=lambda w: w.numel())
            for j in self.jobs:
                self._call(j, s, ws)
            torch.cuda.synchronize(self.device)
            if not self._grow():
                return
        raise RuntimeError("capacities did not settle")

    def capture(self):
        """Captures every molecule's call into one CUDA graph (lanes forked from and joined to one stream)."""
        torch.cuda.synchronize(self.device)
        main = torch.cuda.Stream(self.device)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=main, capture_error_mode="relaxed"):
            fork = torch.cuda.Event()
            fork.record(main)
            for s in self.streams:
                s.wait_event(fork)
            for j in self.jobs:
                self._call(j, self.streams[j.lane])
            for s in self.streams:
                e = torch.cuda.Event()
                e.record(s)
                main.wait_event(e)
        self.graph = g

    def replay(self):
        self.graph.replay()

    def run(self):
        """Captures (if needed) and replays the batch graph until no capacity overflows."""
        for _ in range(4):
            if self.graph is None:
                self.capture()
            self.replay()
            torch.cuda.synchronize(self.device)
            if not self._grow():
                return
        raise RuntimeError("capacities did not settle")

    def results(self) -> list[np.ndarray]:
        return [j.eloc.double().cpu().numpy() for j in self.jobs]

    @property
    def walker_count(self) -> int:
        return int(sum(j.r.shape[0] for j in self.jobs))


class Autotuner:
    """Picks (lanes, walkers per chunk) for a ragged batch: every candidate whose workspaces fit the HBM budget
    is built, captured and timed over ``reps`` replays; the fastest wins.  Results are kept per batch
    signature (molecule sizes and walker counts)."""

    def __init__(self, candidates=((1, 64), (2, 64), (4, 64), (4, 128), (8, 32)), budget_bytes: float = 96e9,
                 reps: int = 2):
        self.candidates = list(candidates)
        self.budget = float(budget_bytes)
        self.reps = int(reps)
        self.cache: dict = {}

    def tune(self, mols, walkers, precision="mixed", device="cuda"):
        key = (precision, tuple(m.n_el for m in mols), tuple(int(w) for w in walkers))
        if key in self.cache:
            return self.cache[key]
        trials = []
        for lanes, chunk in self.candidates:
            batch = RaggedBatch(mols, walkers, precision, lanes=lanes, chunk=chunk, device=device)
            if sum(batch.workspace_bytes()) > self.budget:
                del batch
                continue
            batch.run()  # capture and settle the capacities
            t0 = time.perf_counter()
            for _ in range(self.reps):
                batch.replay()
            torch.cuda.synchronize()
            trials.append(((time.perf_counter() - t0) / self.reps, lanes, chunk))
            del batch
            torch.cuda.empty_cache()
        if not trials:
            raise RuntimeError("no candidate fits the HBM budget")
        best = min(trials)
        self.cache[key] = dict(lanes=best[1], chunk=best[2], seconds=best[0],
                               trials=[dict(lanes=l, chunk=c, seconds=t) for t, l, c in trials])
        return self.cache[key]
