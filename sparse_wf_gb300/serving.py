"""Serving loop: local-energy and MCMC-block requests for molecules of different sizes, served as they arrive
with continuous batching on one GPU.

A request asks for either the local energy of its walkers or one all-electron Metropolis block of ``steps``
steps, for an alkane C_nH_2n+2 and a number of walkers.  The engine keeps

* one model per molecule size (wavefunction and prepared parameters, resident on the device);
* ``lanes`` execution slots, each a CUDA stream with a workspace allocated once at start-up and sized for the
  largest request the engine accepts;
* per admitted request, its walkers, outputs and status words on the device for the life of the request.

``run(trace)`` replays a trace in real time: arrived requests wait in a FIFO queue; whenever a slot is free and
the request's device state fits the HBM budget it is admitted, its host walkers are copied in and its work is
enqueued on the slot's stream, where it overlaps with the requests already on the other slots; completion is
detected by polling a CUDA event, after which the slot and the memory are released.  Latency is measured from
the request's arrival to the moment its results are in host memory; p50 and p99 are reported with the
throughput.  A request whose neighbour capacities overflow (status flag) is re-run with grown capacities, as the
library's host retry does elsewhere.

The library calls neither allocate nor synchronise, so nothing in the loop waits on the device except the
event polls.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import math
import time
from collections import deque
from typing import Optional

import numpy as np
import torch

from . import _lib, systems
from .wavefunction import DeviceParams, FireWaveFunction, StaticArgs


@dataclasses.dataclass
class Request:
    rid: int
    kind: str  # "eloc" or "mcmc"
    n_carbon: int
    walkers: int
    arrival: float  # seconds after the start of the trace
    steps: int = 10
    width: float = 0.1
    seed: int = 0
    # filled in by the engine
    admitted: float = math.nan
    done: float = math.nan
    eloc: Optional[np.ndarray] = None
    logpsi: Optional[np.ndarray] = None
    n_accept: Optional[np.ndarray] = None
    retries: int = 0

    @property
    def latency(self) -> float:
        return self.done - self.arrival


def poisson_trace(n_requests: int, rate: float, seed: int = 5, n_range=(4, 60), walker_range=(256, 2048),
                  mcmc_fraction: float = 0.5, steps: int = 10) -> list[Request]:
    """Poisson arrivals (mean ``rate`` per second) of E_loc / MCMC-block requests with uniform molecule sizes and
    walker counts (numpy default_rng(seed))."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, size=n_requests))
    out = []
    for i in range(n_requests):
        kind = "mcmc" if rng.random() < mcmc_fraction else "eloc"
        out.append(Request(i, kind, int(rng.integers(n_range[0], n_range[1] + 1)),
                           int(rng.integers(walker_range[0], walker_range[1] + 1)), float(t[i]), steps=steps,
                           seed=int(rng.integers(1 << 30))))
    return out


class _Model:
    """Wavefunction of one alkane with its prepared parameters and neighbour capacities."""

    def __init__(self, n_carbon: int, precision: str, device, chunk: int, params_seed: int):
        mol = systems.alkane(n_carbon)
        self.mol = mol
        self.wf = FireWaveFunction(mol, precision=precision, device=device, chunk_walkers=chunk)
        r = systems.init_electrons(mol, 64, 77)
        self.params: DeviceParams = self.wf._params(self.wf.init(params_seed, r[:1]))
        nu, _ = systems.spin_counts(mol)
        # capacities from 64 sample walkers, padded; a request that exceeds them is re-run with grown ones
        self.static = self.wf.get_static_input(r).round_with_padding(1.3, mol.n_el, nu, mol.n_nuc)
        self.wf._ws = None

    def problem(self, walkers: int, static: StaticArgs) -> _lib.Problem:
        return self.wf._problem(walkers, static)


@dataclasses.dataclass
class _Active:
    req: Request
    lane: int
    static: StaticArgs
    nbytes: int
    r: torch.Tensor
    out: torch.Tensor
    logpsi: torch.Tensor
    sign: torch.Tensor
    n_acc: torch.Tensor
    status: torch.Tensor
    host: dict
    event: torch.cuda.Event


class ServingEngine:
    def __init__(self, precision: str = "mixed", lanes: int = 4, chunk: int = 32, hbm_budget: float = 200e9,
                 max_carbon: int = 60, max_walkers: int = 2048, params_seed: int = 0,
                 device: str | torch.device = "cuda"):
        self.device = torch.device(device)
        self.precision = precision
        self.lanes = int(lanes)
        self.chunk = int(chunk)
        self.budget = float(hbm_budget)
        self.params_seed = params_seed
        self.max_walkers = int(max_walkers)
        self.models: dict[int, _Model] = {}
        self.streams = [torch.cuda.Stream(self.device) for _ in range(self.lanes)]
        self.dtype = torch.float64 if precision == "fp64" else torch.float32
        # lane workspaces sized for the largest accepted molecule (capacities padded once more for retries)
        big = self.model(max_carbon)
        grown = StaticArgs(*(int(1.5 * v) for v in (big.static.n_pairs_same, big.static.n_pairs_diff,
                                                    big.static.n_triplets, big.static.n_neighbours_en)))
        self.ws_bytes = self._ws_need(big, max_walkers, grown)
        self.ws = [torch.empty(self.ws_bytes, dtype=torch.uint8, device=self.device) for _ in range(self.lanes)]
        self.in_use = 0

    # ------------------------------------------------------------------ set-up
    def model(self, n_carbon: int) -> _Model:
        if n_carbon not in self.models:
            self.models[n_carbon] = _Model(n_carbon, self.precision, self.device, self.chunk, self.params_seed)
        return self.models[n_carbon]

    def _ws_need(self, m: _Model, walkers: int, static: StaticArgs) -> int:
        nb = C.c_size_t()
        _lib.check(_lib.load().fire_workspace_size(C.byref(m.problem(walkers, static)), self.chunk, C.byref(nb)),
                   "fire_workspace_size")
        return int(nb.value)

    def warm(self, trace: list[Request]):
        """Builds the models of every molecule size in the trace (outside the timed loop)."""
        for n in sorted({r.n_carbon for r in trace}):
            self.model(n)
        torch.cuda.synchronize(self.device)

    # ------------------------------------------------------------------ one request
    def _state_bytes(self, req: Request, m: _Model) -> int:
        es = 8 if self.precision == "fp64" else 4
        return req.walkers * (m.mol.n_el * 3 + 4) * es + req.walkers * 4 + 64

    def _launch(self, req: Request, lane: int, static: StaticArgs, now: float) -> _Active:
        m = self.model(req.n_carbon)
        s = self.streams[lane]
        B, n = req.walkers, m.mol.n_el
        r_host = torch.from_numpy(systems.init_electrons(m.mol, B, req.seed).astype(
            np.float64 if self.dtype == torch.float64 else np.float32)).pin_memory()
        dev = dict(dtype=self.dtype, device=self.device)
        with torch.cuda.stream(s):
            r = torch.empty((B, n, 3), **dev)
            out, logpsi, sign = torch.empty(B, **dev), torch.empty(B, **dev), torch.empty(B, **dev)
            n_acc = torch.zeros(B, dtype=torch.int32, device=self.device)
            status = torch.zeros(_lib.STATUS_WORDS, dtype=torch.int32, device=self.device)
            r.copy_(r_host, non_blocking=True)
        prob = m.problem(B, static)
        prob.chunk_walkers = 0  # as many walkers per internal pass as the slot's workspace holds
        ws = self.ws[lane]
        lib = _lib.load()
        sp = C.c_void_p(s.cuda_stream)
        R, Z, prep = (C.c_void_p(m.wf.R_dev.data_ptr()), C.c_void_p(m.wf.Z_dev.data_ptr()),
                      C.c_void_p(m.params.prepared.data_ptr()))
        wsp, wsb, stp = C.c_void_p(ws.data_ptr()), C.c_size_t(ws.numel()), C.c_void_p(status.data_ptr())
        if req.kind == "eloc":
            _lib.check(lib.fire_local_energy(sp, C.byref(prob), R, Z, prep, C.c_void_p(r.data_ptr()),
                                             C.c_void_p(logpsi.data_ptr()), C.c_void_p(sign.data_ptr()),
                                             C.c_void_p(out.data_ptr()), None, None, wsp, wsb, stp),
                       "fire_local_energy")
        else:
            _lib.check(lib.fire_logpsi(sp, C.byref(prob), R, Z, prep, C.c_void_p(r.data_ptr()),
                                       C.c_void_p(sign.data_ptr()), C.c_void_p(logpsi.data_ptr()), wsp, wsb, stp),
                       "fire_logpsi")
            _lib.check(lib.fire_mcmc_block(sp, C.byref(prob), R, Z, prep, C.c_void_p(r.data_ptr()),
                                           C.c_void_p(logpsi.data_ptr()), int(req.steps), float(req.width),
                                           C.c_uint64(req.seed), C.c_uint64(0), None, None,
                                           C.c_void_p(n_acc.data_ptr()), None, wsp, wsb, stp), "fire_mcmc_block")
        host = dict(out=torch.empty(B, dtype=self.dtype).pin_memory(),
                    logpsi=torch.empty(B, dtype=self.dtype).pin_memory(),
                    n_acc=torch.empty(B, dtype=torch.int32).pin_memory(),
                    status=torch.empty(_lib.STATUS_WORDS, dtype=torch.int32).pin_memory())
        with torch.cuda.stream(s):
            host["logpsi"].copy_(logpsi, non_blocking=True)
            host["status"].copy_(status, non_blocking=True)
            if req.kind == "eloc":
                host["out"].copy_(out, non_blocking=True)
            else:
                host["n_acc"].copy_(n_acc, non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(s)
        if math.isnan(req.admitted):
            req.admitted = now
        return _Active(req, lane, static, self._state_bytes(req, m), r, out, logpsi, sign, n_acc, status, host, ev)

    def _finish(self, a: _Active, now: float) -> Optional[StaticArgs]:
        """Stores the results; returns grown capacities if the request overflowed them."""
        st = a.host["status"].numpy()
        if st[0] & (_lib.FLAG_PAIR_OVERFLOW | _lib.FLAG_NUC_OVERFLOW):
            m = self.model(a.req.n_carbon)
            s = a.static
            return StaticArgs(max(s.n_pairs_same, int(st[1])) + 8, max(s.n_pairs_diff, int(st[1])) + 8,
                              s.n_triplets, max(s.n_neighbours_en, int(st[2])) + 2)
        a.req.done = now
        a.req.logpsi = a.host["logpsi"].numpy().copy()
        if a.req.kind == "eloc":
            a.req.eloc = a.host["out"].numpy().copy()
        else:
            a.req.n_accept = a.host["n_acc"].numpy().copy()
        return None

    # ------------------------------------------------------------------ the loop
    def run(self, trace: list[Request], time_scale: float = 1.0, timeout: float = 600.0) -> dict:
        """Serves ``trace`` in real time (arrival times multiplied by ``time_scale``); returns the metrics."""
        for r in trace:
            if r.walkers > self.max_walkers:
                raise ValueError(f"request {r.rid}: {r.walkers} walkers > {self.max_walkers}")
        self.warm(trace)
        pending = deque(sorted(trace, key=lambda r: r.arrival))
        queue: deque = deque()
        retry: dict[int, StaticArgs] = {}
        active: list[Optional[_Active]] = [None] * self.lanes
        t0 = time.perf_counter()
        done = 0
        while done < len(trace):
            now = time.perf_counter() - t0
            if now > timeout:
                raise RuntimeError("serving loop timed out")
            while pending and pending[0].arrival * time_scale <= now:
                queue.append(pending.popleft())
            # completions
            for k, a in enumerate(active):
                if a is not None and a.event.query():
                    grown = self._finish(a, time.perf_counter() - t0)
                    self.in_use -= a.nbytes
                    active[k] = None
                    if grown is not None:
                        a.req.retries += 1
                        retry[a.req.rid] = grown
                        queue.appendleft(a.req)
                    else:
                        done += 1
            # admissions (FIFO, by free slot and memory)
            for k in range(self.lanes):
                if active[k] is None and queue:
                    req = queue[0]
                    m = self.model(req.n_carbon)
                    nb = self._state_bytes(req, m)
                    if self.in_use + nb > self.budget:
                        break
                    static = retry.get(req.rid, m.static)
                    if self._ws_need(m, req.walkers, static) > self.ws_bytes:
                        raise RuntimeError(f"request {req.rid} needs more workspace than a slot holds")
                    queue.popleft()
                    self.in_use += nb
                    active[k] = self._launch(req, k, static, (time.perf_counter() - t0))
            time.sleep(0.0005)
        return summarize(trace, (time.perf_counter() - t0))


def summarize(trace: list[Request], wall: float) -> dict:
    lat = np.array([r.latency for r in trace]) * 1e3
    ev = sum(r.walkers for r in trace if r.kind == "eloc")
    st = sum(r.walkers * r.steps for r in trace if r.kind == "mcmc")
    out = dict(requests=len(trace), wall_s=wall, p50_ms=float(np.percentile(lat, 50)),
               p99_ms=float(np.percentile(lat, 99)), max_ms=float(lat.max()),
               eloc_walker_evals_per_s=ev / wall, mcmc_walker_steps_per_s=st / wall,
               retries=int(sum(r.retries for r in trace)))
    for kind in ("eloc", "mcmc"):
        lk = np.array([r.latency for r in trace if r.kind == kind]) * 1e3
        if lk.size:
            out[f"{kind}_p50_ms"] = float(np.percentile(lk, 50))
            out[f"{kind}_p99_ms"] = float(np.percentile(lk, 99))
    return out
