"""Host-side mirror of the reference's wavefunction / local-energy / MCMC interface.

``FireWaveFunction`` follows ``MoonLikeWaveFunction`` (``src/sparse_wf/model/wave_function.py:67-221``)
for the ``new_sparse`` embedding: ``init``, ``get_static_input``, ``signed``, ``__call__``,
``kinetic_energy``, the Metropolis blocks of every proposal (evaluated in full or, the ``*_low_rank_*`` ones, from
a state per walker) and the pseudopotential energy; ``make_local_energy`` follows ``hamiltonian.py:49-83``,
``make_mcmc`` ``mcmc.py:278-346`` and ``make_width_scheduler`` ``mcmc.py:349-378``.  Every numerical call goes
to ``libfire.so`` through its C ABI (``include/fire.h``) on the current CUDA stream; torch only provides device
memory and streams.

Static shapes: the reference compiles for padded ``StaticArgs`` sizes and grows them on the host
(``static_args.py:62-84``).  Here the sizes are capacities of the device buffers; the kernels report
overflow in a status word instead of truncating silently, and the host grows the capacity from the
observed maxima and re-runs the call.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import math
from typing import Optional

import numpy as np
import torch

from . import _lib
from .params import ModelDims, init_params, pack_params, param_offsets, unpack_params
from .systems import Molecule, spin_counts


@dataclasses.dataclass(frozen=True)
class StaticArgs:
    """Neighbour-count static input (``StaticArgs``, ``model/new_sparse_model.py:46-80``)."""

    n_pairs_same: int
    n_pairs_diff: int
    n_triplets: int
    n_neighbours_en: int

    @property
    def n_pairs(self) -> int:
        return self.n_pairs_same + self.n_pairs_diff

    def round_with_padding(self, padding_factor: float, n_el: int, n_up: int, n_nuc: int) -> "StaticArgs":
        """``round_with_padding`` (``static_args.py:9-14``) capped by ``StaticArgs.get_max``."""
        n_dn = n_el - n_up
        mx = (n_up * (n_up - 1) + n_dn * (n_dn - 1), 2 * n_up * n_dn, n_el * (n_el - 1) ** 2, n_nuc)

        def rnd(x, m):
            if x <= 0:
                return 0
            if padding_factor <= 1.0:
                return min(x, m)
            return int(min(padding_factor ** math.ceil(math.log(x) / math.log(padding_factor)), m))

        vals = (self.n_pairs_same, self.n_pairs_diff, self.n_triplets, self.n_neighbours_en)
        return StaticArgs(*(rnd(v, m) for v, m in zip(vals, mx)))


class DeviceParams:
    """Parameters resident on the device: the float32 blob and the prepared buffer."""

    def __init__(self, wf: "FireWaveFunction", params: dict[str, np.ndarray]):
        self.host = params
        blob, offs = pack_params(wf.dims, params, np.float32)
        self.offsets = offs
        self.blob = torch.from_numpy(blob).to(wf.device)
        lib = _lib.load()
        prob = wf._problem(1, None)
        nbytes = C.c_size_t()
        _lib.check(lib.fire_prepared_size(C.byref(prob), C.byref(nbytes)), "fire_prepared_size")
        self.prepared = torch.empty(int(nbytes.value), dtype=torch.uint8, device=wf.device)
        offs_c = (C.c_int64 * len(offs))(*[int(o) for o in offs])
        _lib.check(
            lib.fire_prepare_params(wf._stream(), C.byref(prob), C.c_void_p(self.blob.data_ptr()), offs_c,
                                    C.c_void_p(self.prepared.data_ptr()), C.c_size_t(self.prepared.numel())),
            "fire_prepare_params",
        )


class FireWaveFunction:
    """FiRE wavefunction (new_sparse embedding, isotropic envelopes, psiformer cusp + MLP/attention
    Jastrow) evaluated by the sm_103a kernels of ``libfire.so``."""

    def __init__(self, mol: Molecule, cutoff: float = 5.0, cutoff_1el: float = 20.0, precision: str = "fp32",
                 device: str | torch.device = "cuda", chunk_walkers: int = 0):
        if precision not in _lib.PREC:
            raise ValueError(f"precision must be one of {list(_lib.PREC)}")
        self.mol = mol
        self.R = np.asarray(mol.R, np.float32)
        self.Z = np.asarray(mol.Z)
        self.n_electrons = mol.n_el
        self.n_up, _ = spin_counts(mol)
        self.n_nuclei = mol.n_nuc
        self.cutoff = float(cutoff)
        self.cutoff_1el = float(cutoff_1el)
        self.precision = precision
        self.device = torch.device(device)
        self.chunk_walkers = int(chunk_walkers)
        self.dims = ModelDims(self.n_electrons, self.n_up, self.n_nuclei, self.cutoff, self.cutoff_1el)
        self.dtype = torch.float64 if precision == "fp64" else torch.float32
        self.R_dev = torch.from_numpy(self.R).to(self.device)
        self.Z_dev = torch.from_numpy(self.Z.astype(np.float32)).to(self.device)
        self._ws: Optional[torch.Tensor] = None
        self._status = torch.zeros(_lib.STATUS_WORDS, dtype=torch.int32, device=self.device)
        self._lr_cap = 0  # changed-set capacity of the last low-rank block (grown on overflow, like the statics)
        # walkers per pass of the low-rank blocks and the pseudopotential energy (0: as many as lr_ws_gb holds; the
        # per-walker state is far smaller than the local energy's planes, and one pass over the batch makes every
        # step's launches serve all walkers)
        self.lr_chunk_walkers = 0
        self.lr_ws_gb = 64.0
        # walkers per pass of the value path (log|psi| and the Metropolis blocks that evaluate every proposal in full;
        # 0: as many as the workspace holds, which, sized for the local energy's planes, holds several times the
        # local energy's pass)
        self.value_chunk_walkers = 0
        # FP32 / mixed local energy: ill-conditioned walkers ((|lap| + |grad|^2) / 2 above refine_ratio |E_loc| or
        # refine_ks Hartree, a determinant-weighted condition number of the orbital matrices above refine_kappa, or the
        # product of the two above refine_kscond) are evaluated again with FP64 orbital-matrix values; the capacity of that pass follows the counts the device
        # reports (the defaults of fire.h)
        self.refine = precision != "fp64"
        self.refine_ratio = 100.0
        self.refine_kappa = 1.0e6
        self.refine_ks = 1.0e5
        self.refine_kscond = 1.0e10
        self._refine_cap = 0
        self.last_refined = 0
        _lib.load()

    # ------------------------------------------------------------------ plumbing
    @classmethod
    def create(cls, mol: Molecule, **kw) -> "FireWaveFunction":
        return cls(mol, **kw)

    def _stream(self):
        return C.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    def _problem(self, n_walkers: int, static: Optional[StaticArgs], refine: bool = False) -> _lib.Problem:
        cap_p = static.n_pairs if static is not None else 1
        cap_n = static.n_neighbours_en if static is not None else 1
        cap_r = 0
        if refine and self.refine:
            # the last call's count padded; at least 2 % of the batch (and 2 walkers)
            cap_r = min(int(n_walkers), max(self._refine_cap, 2, -(-2 * int(n_walkers) // 100)))
        return _lib.Problem(self.n_electrons, self.n_up, self.n_nuclei, int(n_walkers), self.cutoff,
                            self.cutoff_1el, max(1, int(cap_p)), max(1, int(cap_n)), _lib.PREC[self.precision],
                            self.chunk_walkers, cap_r, float(self.refine_ratio), float(self.refine_kappa),
                            float(self.refine_ks), float(self.refine_kscond))

    def _workspace(self, prob: _lib.Problem, cap_changed: int = 0) -> torch.Tensor:
        """Workspace of the local-energy and value paths, or (cap_changed > 0) of the low-rank block."""
        lib = _lib.load()
        nbytes = C.c_size_t()
        chunk = prob.chunk_walkers if prob.chunk_walkers > 0 else prob.n_walkers
        if cap_changed > 0:
            _lib.check(lib.fire_low_rank_workspace_size(C.byref(prob), chunk, int(cap_changed), C.byref(nbytes)),
                       "fire_low_rank_workspace_size")
        else:
            _lib.check(lib.fire_workspace_size(C.byref(prob), chunk, C.byref(nbytes)), "fire_workspace_size")
        need = int(nbytes.value)
        if self._ws is None or self._ws.numel() < need:
            self._ws = None
            self._ws = torch.empty(need, dtype=torch.uint8, device=self.device)
        return self._ws

    def _lr_problem(self, n_walkers: int, static: StaticArgs, cap: int) -> _lib.Problem:
        """The problem of a low-rank call with its walkers per pass (lr_chunk_walkers, else what lr_ws_gb holds)."""
        prob = self._problem(n_walkers, static)
        c = int(self.lr_chunk_walkers)
        if c <= 0:
            nbytes = C.c_size_t()
            _lib.check(_lib.load().fire_low_rank_workspace_size(C.byref(prob), 1, int(cap), C.byref(nbytes)),
                       "fire_low_rank_workspace_size")
            c = int(self.lr_ws_gb * 1e9) // max(1, int(nbytes.value))
            # the changed rows of a pass (walkers x cap) and its electron rows stay within 65535 row tiles of 64
            c = min(c, 65535 * 64 // max(self.n_electrons, int(cap)))
        prob.chunk_walkers = max(1, min(int(n_walkers), c))
        return prob

    def _electrons(self, electrons) -> torch.Tensor:
        r = torch.as_tensor(electrons)
        if r.ndim == 2:
            r = r[None]
        return r.to(device=self.device, dtype=self.dtype).contiguous()

    def _params(self, params) -> DeviceParams:
        return params if isinstance(params, DeviceParams) else DeviceParams(self, params)

    def _read_status(self) -> np.ndarray:
        return self._status.cpu().numpy()

    def _grown(self, st: np.ndarray, static: StaticArgs) -> StaticArgs:
        """Capacities after a pair or e-n overflow: the largest counts the device saw, padded by 10 %."""
        pairs = max(int(st[1]), static.n_pairs)
        nucs = max(int(st[2]), static.n_neighbours_en)
        half = (pairs + 1) // 2
        static = StaticArgs(half, pairs - half, max(static.n_triplets, int(st[3])), nucs)
        return static.round_with_padding(1.1, self.n_electrons, self.n_up, self.n_nuclei)

    def _run(self, fn, static: StaticArgs, n_walkers: int, retries: int = 4, refine: bool = False, ws_fn=None):
        """Runs fn(problem, workspace) with overflow-driven capacity growth; returns the static used.  With refine
        (the local energy) the refinement capacity follows the device's count of ill-conditioned walkers: a call
        that found more than its capacity is repeated with the count."""
        for _ in range(retries):
            self._status.zero_()
            prob = self._problem(n_walkers, static, refine)
            fn(prob, ws_fn(prob) if ws_fn is not None else self._workspace(prob))
            st = self._read_status()
            flags = int(st[0])
            if flags & (_lib.FLAG_PAIR_OVERFLOW | _lib.FLAG_NUC_OVERFLOW):
                static = self._grown(st, static)
                continue
            if refine and prob.refine_cap > 0:
                self.last_refined = int(st[5])
                self._refine_cap = int(st[5]) + int(st[5]) // 4 + 1
                if flags & _lib.FLAG_REFINE_OVERFLOW:
                    continue
            if flags & _lib.FLAG_NONFINITE:
                pass  # NaNs propagate to the caller like the reference (train.py:263-264)
            return static
        raise RuntimeError("neighbour capacity did not converge")

    # ------------------------------------------------------------------ reference interface
    def init(self, seed: int, electrons) -> dict[str, np.ndarray]:
        """Random-init parameters; the two normalize scales are 1/std of the embedding on the first
        walker, as in ``NewSparseEmbedding.init`` (``new_sparse_model.py:354-380``)."""
        params = init_params(self.dims, seed)
        r = self._electrons(electrons)[:1]
        static = self.get_static_input(r)
        h_c, _ = self.embedding(params, r, static)
        s0 = 1.0 / float(np.std(h_c.double().cpu().numpy()))
        params["scales"] = np.array([s0 if np.isfinite(s0) else 1.0, 1.0])
        _, h_u = self.embedding(params, r, static)
        s1 = 1.0 / float(np.std(h_u.double().cpu().numpy()))
        params["scales"][1] = s1 if np.isfinite(s1) else 1.0
        return params

    def get_static_input(self, electrons) -> StaticArgs:
        """``get_static_input`` (``model/new_sparse_model.py:399-437``): counts maximised over walkers."""
        r = self._electrons(electrons)
        B = r.shape[0]
        counts = torch.zeros((B, 4), dtype=torch.int32, device=self.device)
        out = _lib.NeighborOut()
        out.counts = counts.data_ptr()
        prob = self._problem(B, StaticArgs(1, 0, 0, self.n_nuclei))
        lib = _lib.load()
        self._status.zero_()
        _lib.check(lib.fire_neighbors(self._stream(), C.byref(prob), C.c_void_p(r.data_ptr()),
                                      C.c_void_p(self.R_dev.data_ptr()), C.byref(out),
                                      C.c_void_p(self._status.data_ptr())), "fire_neighbors")
        c = counts.max(dim=0).values.cpu().numpy()
        return StaticArgs(int(c[0]), int(c[1]), int(c[2]), int(c[3]))

    def neighbor_lists(self, electrons, static: StaticArgs) -> dict[str, np.ndarray]:
        """``get_pair_indices`` + ``get_neighbouring_nuclei`` in the reference's padded format."""
        r = self._electrons(electrons)
        B, n = r.shape[0], self.n_electrons
        cs, cd = static.n_pairs_same, static.n_pairs_diff
        dev = dict(dtype=torch.int32, device=self.device)
        t = {k: torch.empty((B, cs), **dev) for k in ("ct_same", "nb_same", "jac_same")}
        t.update({k: torch.empty((B, cd), **dev) for k in ("ct_diff", "nb_diff", "jac_diff")})
        t.update({k: torch.empty((B, n + cs + cd), **dev) for k in ("jac_ctr", "jac_dep")})
        t["en_idx"] = torch.empty((B, n, max(1, static.n_neighbours_en)), **dev)
        t["counts"] = torch.empty((B, 4), **dev)
        out = _lib.NeighborOut()
        for k, v in t.items():
            setattr(out, k, v.data_ptr())
        out.cap_same, out.cap_diff = cs, cd
        prob = self._problem(B, static)
        self._status.zero_()
        _lib.check(_lib.load().fire_neighbors(self._stream(), C.byref(prob), C.c_void_p(r.data_ptr()),
                                              C.c_void_p(self.R_dev.data_ptr()), C.byref(out),
                                              C.c_void_p(self._status.data_ptr())), "fire_neighbors")
        res = {k: v.cpu().numpy() for k, v in t.items()}
        res["status"] = self._read_status()
        return res

    def embedding(self, params, electrons, static: StaticArgs):
        """Value-path embedding: (h after message passing, h after the update MLP before scales[1])."""
        p = self._params(params)
        r = self._electrons(electrons)
        B = r.shape[0]
        hc = torch.empty((B, self.n_electrons, 256), dtype=self.dtype, device=self.device)
        hu = torch.empty_like(hc)

        def fn(prob, ws):
            _lib.check(_lib.load().fire_embedding(
                self._stream(), C.byref(prob), C.c_void_p(self.R_dev.data_ptr()), C.c_void_p(p.prepared.data_ptr()),
                C.c_void_p(r.data_ptr()), C.c_void_p(hc.data_ptr()), C.c_void_p(hu.data_ptr()),
                C.c_void_p(ws.data_ptr()), C.c_size_t(ws.numel()), C.c_void_p(self._status.data_ptr())),
                "fire_embedding")

        self._run(fn, static, B)
        return hc, hu

    def signed(self, params, electrons, static: StaticArgs):
        """(sign, log|psi|) per walker (``wave_function.py:183-190``)."""
        p = self._params(params)
        r = self._electrons(electrons)
        B = r.shape[0]
        sign = torch.empty(B, dtype=self.dtype, device=self.device)
        logpsi = torch.empty(B, dtype=self.dtype, device=self.device)

        def fn(prob, ws):
            prob.chunk_walkers = int(self.value_chunk_walkers)
            _lib.check(_lib.load().fire_logpsi(
                self._stream(), C.byref(prob), C.c_void_p(self.R_dev.data_ptr()), C.c_void_p(self.Z_dev.data_ptr()),
                C.c_void_p(p.prepared.data_ptr()), C.c_void_p(r.data_ptr()), C.c_void_p(sign.data_ptr()),
                C.c_void_p(logpsi.data_ptr()), C.c_void_p(ws.data_ptr()), C.c_size_t(ws.numel()),
                C.c_void_p(self._status.data_ptr())), "fire_logpsi")

        self._run(fn, static, B)
        return sign, logpsi

    def __call__(self, params, electrons, static: StaticArgs):
        return self.signed(params, electrons, static)[1]

    def logpsi_grad(self, params, electrons, static: StaticArgs, chunk: int = 0, ws_gb: float = 8.0):
        """Per-walker gradient of log|psi| with respect to every parameter (the rows of the Jacobian that SPRING
        contracts: ``jax.grad`` of ``log_p`` vmapped over the walkers, ``preconditioner.py:185-191``).

        Returns (grad [B, L] in the blob layout of ``fire_param_layout``, sign [B], log|psi| [B]); ``unflatten_grad``
        splits a row into the parameter slots.  chunk: walkers per internal pass (0: as many as a workspace of
        ws_gb gigabytes holds)."""
        p = self._params(params)
        r = self._electrons(electrons)
        B = r.shape[0]
        L = int(p.offsets[-1])
        grad = torch.empty((B, L), dtype=self.dtype, device=self.device)
        sign = torch.empty(B, dtype=self.dtype, device=self.device)
        logpsi = torch.empty(B, dtype=self.dtype, device=self.device)
        lib = _lib.load()

        def ws_fn(prob):
            nbytes = C.c_size_t()
            c = int(chunk)
            if c <= 0:
                _lib.check(lib.fire_logpsi_grad_workspace_size(C.byref(prob), 1, C.byref(nbytes)),
                           "fire_logpsi_grad_workspace_size")
                c = max(1, min(B, int(ws_gb * 1e9) // max(1, int(nbytes.value))))
            prob.chunk_walkers = c
            _lib.check(lib.fire_logpsi_grad_workspace_size(C.byref(prob), c, C.byref(nbytes)),
                       "fire_logpsi_grad_workspace_size")
            need = int(nbytes.value)
            if self._ws is None or self._ws.numel() < need:
                self._ws = None
                self._ws = torch.empty(need, dtype=torch.uint8, device=self.device)
            return self._ws

        def fn(prob, ws):
            _lib.check(lib.fire_logpsi_grad(
                self._stream(), C.byref(prob), C.c_void_p(self.R_dev.data_ptr()), C.c_void_p(p.prepared.data_ptr()),
                C.c_void_p(r.data_ptr()), C.c_void_p(sign.data_ptr()), C.c_void_p(logpsi.data_ptr()),
                C.c_void_p(grad.data_ptr()), C.c_void_p(ws.data_ptr()), C.c_size_t(ws.numel()),
                C.c_void_p(self._status.data_ptr())), "fire_logpsi_grad")

        self._run(fn, static, B, ws_fn=ws_fn)
        return grad, sign, logpsi

    def unflatten_grad(self, row) -> dict[str, np.ndarray]:
        """One gradient row (blob layout) as {slot: array shaped like the parameter}."""
        row = np.asarray(row.cpu() if isinstance(row, torch.Tensor) else row)
        return unpack_params(self.dims, row, param_offsets(self.dims))

    def local_energy_full(self, params, electrons, static: StaticArgs, debug: bool = False):
        """E_loc per walker plus (log|psi|, sign, (mean, std) in FP64, debug dict, static used)."""
        p = self._params(params)
        r = self._electrons(electrons)
        B = r.shape[0]
        dev = dict(dtype=self.dtype, device=self.device)
        eloc = torch.empty(B, **dev)
        logpsi = torch.empty(B, **dev)
        sign = torch.empty(B, **dev)
        stats = torch.empty(2, dtype=torch.float64, device=self.device)
        dbg = _lib.ElocDebug()
        dbg_t = {}
        if debug:
            dbg_t = dict(kinetic=torch.empty(B, **dev), potential=torch.empty(B, **dev),
                         logdet=torch.empty((B, 4), dtype=torch.float64, device=self.device),
                         sign_det=torch.empty((B, 4), dtype=torch.float64, device=self.device),
                         jastrow=torch.empty(B, **dev), grad=torch.empty((B, self.n_electrons, 3), **dev),
                         lap=torch.empty(B, **dev), refined=torch.zeros(B, dtype=torch.int32, device=self.device),
                         cond=torch.zeros(B, dtype=torch.float64, device=self.device))
            for k, v in dbg_t.items():
                setattr(dbg, k, v.data_ptr())

        def fn(prob, ws):
            _lib.check(_lib.load().fire_local_energy(
                self._stream(), C.byref(prob), C.c_void_p(self.R_dev.data_ptr()), C.c_void_p(self.Z_dev.data_ptr()),
                C.c_void_p(p.prepared.data_ptr()), C.c_void_p(r.data_ptr()), C.c_void_p(logpsi.data_ptr()),
                C.c_void_p(sign.data_ptr()), C.c_void_p(eloc.data_ptr()), C.c_void_p(stats.data_ptr()),
                C.byref(dbg) if debug else None, C.c_void_p(ws.data_ptr()), C.c_size_t(ws.numel()),
                C.c_void_p(self._status.data_ptr())), "fire_local_energy")

        self.last_refined = 0
        used = self._run(fn, static, B, refine=True)
        return eloc, dict(logpsi=logpsi, sign=sign, stats=stats, debug=dbg_t, static=used, refined=self.last_refined)

    def kinetic_energy(self, params, electrons, static: StaticArgs):
        """``kinetic_energy`` (``wave_function.py:215-221``) through the sparse forward Laplacian."""
        _, aux = self.local_energy_full(params, electrons, static, debug=True)
        return aux["debug"]["kinetic"]

    def potential_energy(self, electrons):
        r = self._electrons(electrons)
        out = torch.empty(r.shape[0], dtype=self.dtype, device=self.device)
        prob = self._problem(r.shape[0], None)
        _lib.check(_lib.load().fire_potential_energy(self._stream(), C.byref(prob), C.c_void_p(r.data_ptr()),
                                                     C.c_void_p(self.R_dev.data_ptr()),
                                                     C.c_void_p(self.Z_dev.data_ptr()), C.c_void_p(out.data_ptr())),
                   "fire_potential_energy")
        return out

    def mcmc_block(self, params, electrons: torch.Tensor, logpsi: torch.Tensor, static: StaticArgs, steps: int,
                   width: float, seed: int = 0, counter: int = 0, replay_noise=None, replay_log_u=None):
        """In-place all-electron Metropolis block; returns (n_accept per walker, static_max)."""
        p = self._params(params)
        r = electrons
        assert r.is_contiguous() and r.dtype == self.dtype
        B = r.shape[0]
        n_acc = torch.zeros(B, dtype=torch.int32, device=self.device)
        smax = torch.zeros(4, dtype=torch.int32, device=self.device)
        noise = None if replay_noise is None else self._electrons(replay_noise).reshape(steps, B, -1, 3).contiguous()
        logu = None if replay_log_u is None else torch.as_tensor(replay_log_u).to(self.device, self.dtype).contiguous()
        r0 = r.clone()
        lp0 = logpsi.clone()

        def fn(prob, ws):
            prob.chunk_walkers = int(self.value_chunk_walkers)
            r.copy_(r0)
            logpsi.copy_(lp0)
            n_acc.zero_()
            smax.zero_()
            _lib.check(_lib.load().fire_mcmc_block(
                self._stream(), C.byref(prob), C.c_void_p(self.R_dev.data_ptr()), C.c_void_p(self.Z_dev.data_ptr()),
                C.c_void_p(p.prepared.data_ptr()), C.c_void_p(r.data_ptr()), C.c_void_p(logpsi.data_ptr()),
                int(steps), float(width), C.c_uint64(seed), C.c_uint64(counter),
                C.c_void_p(noise.data_ptr()) if noise is not None else None,
                C.c_void_p(logu.data_ptr()) if logu is not None else None, C.c_void_p(n_acc.data_ptr()),
                C.c_void_p(smax.data_ptr()), C.c_void_p(ws.data_ptr()), C.c_size_t(ws.numel()),
                C.c_void_p(self._status.data_ptr())), "fire_mcmc_block")

        self._run(fn, static, B)
        sm = smax.cpu().numpy()
        return n_acc, StaticArgs(int(sm[0]), int(sm[1]), 0, int(sm[3]))


    def mcmc_single_block(self, params, electrons: torch.Tensor, logpsi: torch.Tensor, static: StaticArgs,
                          steps: int, width: float, step_offset: int = 0, seed: int = 0, counter: int = 0,
                          replay_noise=None, replay_log_u=None):
        """In-place single-electron Metropolis block (``mcmc_steps_low_rank`` with ``proposal_single_electron``,
        ``mcmc.py:100-111, 196-275``): step s moves electron (step_offset + s) mod n.  Every proposal is evaluated in
        full (no low-rank state).  replay_noise [steps, B, 3], replay_log_u [steps, B].  Returns (n_accept per walker,
        static_max)."""
        p = self._params(params)
        r = electrons
        assert r.is_contiguous() and r.dtype == self.dtype
        B = r.shape[0]
        n_acc = torch.zeros(B, dtype=torch.int32, device=self.device)
        smax = torch.zeros(4, dtype=torch.int32, device=self.device)
        noise = None
        if replay_noise is not None:
            noise = torch.as_tensor(np.asarray(replay_noise)).to(self.device, self.dtype).reshape(steps, B, 3).contiguous()
        logu = None if replay_log_u is None else torch.as_tensor(replay_log_u).to(self.device, self.dtype).contiguous()
        r0 = r.clone()
        lp0 = logpsi.clone()

        def fn(prob, ws):
            prob.chunk_walkers = int(self.value_chunk_walkers)
            r.copy_(r0)
            logpsi.copy_(lp0)
            n_acc.zero_()
            smax.zero_()
            _lib.check(_lib.load().fire_mcmc_single_block(
                self._stream(), C.byref(prob), C.c_void_p(self.R_dev.data_ptr()), C.c_void_p(self.Z_dev.data_ptr()),
                C.c_void_p(p.prepared.data_ptr()), C.c_void_p(r.data_ptr()), C.c_void_p(logpsi.data_ptr()),
                int(steps), int(step_offset), float(width), C.c_uint64(seed), C.c_uint64(counter),
                C.c_void_p(noise.data_ptr()) if noise is not None else None,
                C.c_void_p(logu.data_ptr()) if logu is not None else None, C.c_void_p(n_acc.data_ptr()),
                C.c_void_p(smax.data_ptr()), C.c_void_p(ws.data_ptr()), C.c_size_t(ws.numel()),
                C.c_void_p(self._status.data_ptr())), "fire_mcmc_single_block")

        self._run(fn, static, B)
        sm = smax.cpu().numpy()
        return n_acc, StaticArgs(int(sm[0]), int(sm[1]), 0, int(sm[3]))

    def _low_rank(self, fn_name, r, logpsi, static: StaticArgs, cap_changed, launch):
        """Runs a low-rank block, launch(lib_fn, prob, ws, cap, n_acc, smax), with the reruns it needs: from the
        original walkers and log|psi| after a pair / e-n overflow (grown neighbour capacities) or a changed-set
        overflow (the set the device saw, padded by 10 %; above the limit an error).  Keeps the capacity for the
        next call.  Returns (n_accept per walker, static_max, move statics)."""
        assert r.is_contiguous() and r.dtype == self.dtype
        B, n = r.shape[0], self.n_electrons
        n_acc = torch.zeros(B, dtype=torch.int32, device=self.device)
        smax = torch.zeros(7, dtype=torch.int32, device=self.device)
        r0 = r.clone()
        lp0 = logpsi.clone()
        limit = min(n, _lib.LOW_RANK_MAX_CHANGED)
        if cap_changed is None:
            # the moved electron and its neighbours before and after the move: about twice the mean degree, >= 16
            cap_changed = self._lr_cap or max(16, 2 * static.n_pairs // max(1, n) + 1)
        cap = min(int(cap_changed), limit)
        fn = getattr(_lib.load(), fn_name)
        for _ in range(6):
            self._status.zero_()
            r.copy_(r0)
            logpsi.copy_(lp0)
            n_acc.zero_()
            smax.zero_()
            prob = self._lr_problem(B, static, cap)
            _lib.check(launch(fn, prob, self._workspace(prob, cap), cap, n_acc, smax), fn_name)
            st = self._read_status()
            flags = int(st[0])
            if flags & (_lib.FLAG_PAIR_OVERFLOW | _lib.FLAG_NUC_OVERFLOW):
                static = self._grown(st, static)
                continue
            if flags & _lib.FLAG_CHANGED_OVERFLOW:
                need = int(st[4])
                if need > limit:
                    raise RuntimeError(f"a changed set of {need} electrons exceeds the low-rank block's limit of "
                                       f"{limit}; use the full-evaluation block")
                cap = min(limit, max(need, int(need * 1.1) + 1))
                continue
            break
        else:
            raise RuntimeError("low-rank capacities did not converge")
        self._lr_cap = cap
        sm = smax.cpu().numpy()
        return n_acc, StaticArgs(int(sm[0]), int(sm[1]), 0, int(sm[3])), (int(sm[4]), int(sm[5]), int(sm[6]))

    def _replay(self, arr, shape):
        if arr is None:
            return None
        return torch.as_tensor(np.asarray(arr)).to(self.device, self.dtype).reshape(shape).contiguous()

    def mcmc_low_rank_block(self, params, electrons: torch.Tensor, logpsi: torch.Tensor, static: StaticArgs,
                            steps: int, width: float, step_offset: int = 0, seed: int = 0, counter: int = 0,
                            replay_noise=None, replay_log_u=None, cap_changed: Optional[int] = None):
        """In-place single-electron Metropolis block evaluated by the low-rank update of a cached state
        (``mcmc_steps_low_rank`` with ``proposal_single_electron`` and ``log_psi_with_state`` /
        ``log_psi_low_rank_update``, ``mcmc.py:100-111, 196-275``, ``wave_function.py:226-287``): the proposals,
        draws and acceptance of ``mcmc_single_block``, with log|psi'| from the walker's state (changed rows, the
        determinant lemma and a Woodbury update of the inverses) instead of a full evaluation.  logpsi receives
        log|psi| of the walkers at the start (from their state) and follows the accepted moves.  cap_changed bounds
        the changed set of a step (at most 128); an overflow reruns the block with the set the device saw, and the
        capacity is kept for the next call.  Returns (n_accept per walker, static_max, (n_changed_hout,
        n_changed_pair_same, n_changed_pair_diff)) with the maxima over steps and walkers."""
        p = self._params(params)
        B = electrons.shape[0]
        noise = self._replay(replay_noise, (steps, B, 3))
        logu = self._replay(replay_log_u, (steps, B))

        def launch(fn, prob, ws, cap, n_acc, smax):
            return fn(self._stream(), C.byref(prob), C.c_void_p(self.R_dev.data_ptr()),
                      C.c_void_p(self.Z_dev.data_ptr()), C.c_void_p(p.prepared.data_ptr()),
                      C.c_void_p(electrons.data_ptr()), C.c_void_p(logpsi.data_ptr()), int(steps), int(step_offset),
                      float(width), int(cap), C.c_uint64(seed), C.c_uint64(counter),
                      C.c_void_p(noise.data_ptr()) if noise is not None else None,
                      C.c_void_p(logu.data_ptr()) if logu is not None else None, C.c_void_p(n_acc.data_ptr()),
                      C.c_void_p(smax.data_ptr()), C.c_void_p(ws.data_ptr()), C.c_size_t(ws.numel()),
                      C.c_void_p(self._status.data_ptr()))

        return self._low_rank("fire_mcmc_low_rank_block", electrons, logpsi, static, cap_changed, launch)

    def mcmc_low_rank_cluster_block(self, params, electrons: torch.Tensor, logpsi: torch.Tensor, static: StaticArgs,
                                    steps: int, width: float, max_cluster_size: int = 5,
                                    max_cluster_radius: float = 2.0, sweep_type: str = "sequential",
                                    step_offset: int = 0, seed: int = 0, counter: int = 0, replay_draws=None,
                                    replay_log_u=None, cap_changed: Optional[int] = None):
        """In-place Metropolis block of cluster updates (``proposal_cluster_update``, ``mcmc.py:119-161``) evaluated by
        the low-rank update of a cached state: the proposals, draws (replay_draws [steps, B, 1 + 15 k]) and acceptance
        of ``mcmc_cluster_block``, the cluster's electrons moved together.  Outputs and capacities as
        ``mcmc_low_rank_block``."""
        if sweep_type not in ("sequential", "random"):
            raise ValueError(f"Invalid sweep_type: {sweep_type}")
        p = self._params(params)
        B = electrons.shape[0]
        k = min(int(max_cluster_size), self.n_electrons)
        draws = self._replay(replay_draws, (steps, B, 1 + 15 * k))
        logu = self._replay(replay_log_u, (steps, B))

        def launch(fn, prob, ws, cap, n_acc, smax):
            return fn(self._stream(), C.byref(prob), C.c_void_p(self.R_dev.data_ptr()),
                      C.c_void_p(self.Z_dev.data_ptr()), C.c_void_p(p.prepared.data_ptr()),
                      C.c_void_p(electrons.data_ptr()), C.c_void_p(logpsi.data_ptr()), int(steps), int(step_offset),
                      float(width), int(max_cluster_size), float(max_cluster_radius),
                      int(sweep_type == "random"), int(cap), C.c_uint64(seed), C.c_uint64(counter),
                      C.c_void_p(draws.data_ptr()) if draws is not None else None,
                      C.c_void_p(logu.data_ptr()) if logu is not None else None, C.c_void_p(n_acc.data_ptr()),
                      C.c_void_p(smax.data_ptr()), C.c_void_p(ws.data_ptr()), C.c_size_t(ws.numel()),
                      C.c_void_p(self._status.data_ptr()))

        return self._low_rank("fire_mcmc_low_rank_cluster_block", electrons, logpsi, static, cap_changed, launch)

    def mcmc_low_rank_jump_block(self, params, electrons: torch.Tensor, logpsi: torch.Tensor, static: StaticArgs,
                                 steps: int, sigma: float = 2.0, seed: int = 0, counter: int = 0, replay_draws=None,
                                 replay_log_u=None, cap_changed: Optional[int] = None):
        """In-place Metropolis block of jumps to the nuclei (``proposal_jump_to_atom``, ``mcmc.py:164-193``) evaluated
        by the low-rank update of a cached state: the proposals, draws (replay_draws [steps, B, 5]) and acceptance of
        ``mcmc_jump_block``, each walker moving its own electron.  Outputs and capacities as
        ``mcmc_low_rank_block``."""
        p = self._params(params)
        B = electrons.shape[0]
        draws = self._replay(replay_draws, (steps, B, 5))
        logu = self._replay(replay_log_u, (steps, B))

        def launch(fn, prob, ws, cap, n_acc, smax):
            return fn(self._stream(), C.byref(prob), C.c_void_p(self.R_dev.data_ptr()),
                      C.c_void_p(self.Z_dev.data_ptr()), C.c_void_p(p.prepared.data_ptr()),
                      C.c_void_p(electrons.data_ptr()), C.c_void_p(logpsi.data_ptr()), int(steps), float(sigma),
                      int(cap), C.c_uint64(seed), C.c_uint64(counter),
                      C.c_void_p(draws.data_ptr()) if draws is not None else None,
                      C.c_void_p(logu.data_ptr()) if logu is not None else None, C.c_void_p(n_acc.data_ptr()),
                      C.c_void_p(smax.data_ptr()), C.c_void_p(ws.data_ptr()), C.c_size_t(ws.numel()),
                      C.c_void_p(self._status.data_ptr()))

        return self._low_rank("fire_mcmc_low_rank_jump_block", electrons, logpsi, static, cap_changed, launch)

    def ecp_energy(self, params, electrons, static: StaticArgs, ecp, seed: int = 0, counter: int = 0,
                   replay_rotations=None, cap_changed: Optional[int] = None):
        """Pseudopotential energy of every walker (``fire_ecp_energy``): the local term and the non-local quadrature
        with psi ratios from the low-rank update of a cached state (``make_pseudopotential``,
        ``pseudopotentials.py:205-219, 272-398``).  The wavefunction's molecule carries the effective charges
        (``EcpTables.z_eff``); ecp is the ``DeviceEcp`` of its tables.  replay_rotations [B, n, 3, 3] replaces the
        random rotations.  Returns (e_ecp [B], move statics maximised over the ratios)."""
        p = self._params(params)
        r = self._electrons(electrons)
        B, n = r.shape[0], self.n_electrons
        out = torch.zeros(B, dtype=self.dtype, device=self.device)
        smax = torch.zeros(7, dtype=torch.int32, device=self.device)
        rot = None
        if replay_rotations is not None:
            rot = torch.as_tensor(np.asarray(replay_rotations)).to(self.device, self.dtype).reshape(B, n, 3, 3)
            rot = rot.contiguous()
        limit = min(n, _lib.LOW_RANK_MAX_CHANGED)
        cap = min(int(cap_changed or self._lr_cap or max(16, 2 * static.n_pairs // max(1, n) + 1)), limit)
        lib = _lib.load()
        for _ in range(6):
            self._status.zero_()
            smax.zero_()
            prob = self._lr_problem(B, static, cap)
            ws = self._workspace(prob, cap)
            _lib.check(lib.fire_ecp_energy(
                self._stream(), C.byref(prob), C.c_void_p(self.R_dev.data_ptr()), C.c_void_p(self.Z_dev.data_ptr()),
                C.c_void_p(p.prepared.data_ptr()), C.c_void_p(r.data_ptr()), C.byref(ecp.struct), int(cap),
                C.c_uint64(seed), C.c_uint64(counter), C.c_void_p(rot.data_ptr()) if rot is not None else None,
                C.c_void_p(out.data_ptr()), C.c_void_p(smax.data_ptr()), C.c_void_p(ws.data_ptr()),
                C.c_size_t(ws.numel()), C.c_void_p(self._status.data_ptr())), "fire_ecp_energy")
            st = self._read_status()
            flags = int(st[0])
            if flags & (_lib.FLAG_PAIR_OVERFLOW | _lib.FLAG_NUC_OVERFLOW):
                static = self._grown(st, static)
                continue
            if flags & _lib.FLAG_CHANGED_OVERFLOW:
                need = int(st[4])
                if need > limit:
                    raise RuntimeError(f"a changed set of {need} electrons exceeds the low-rank limit of {limit}")
                cap = min(limit, max(need, int(need * 1.1) + 1))
                continue
            break
        else:
            raise RuntimeError("low-rank capacities did not converge")
        self._lr_cap = cap
        sm = smax.cpu().numpy()
        return out, (int(sm[4]), int(sm[5]), int(sm[6]))

    def mcmc_jump_block(self, params, electrons: torch.Tensor, logpsi: torch.Tensor, static: StaticArgs,
                        steps: int, sigma: float = 2.0, seed: int = 0, counter: int = 0, replay_draws=None,
                        replay_log_u=None):
        """In-place Metropolis block of jumps to the nuclei (``proposal_jump_to_atom``, ``mcmc.py:164-193``, run for
        ``make_mcmc``'s ``jump_steps``): one random electron per step moves to R_I + sigma * eps, nucleus I drawn with
        probability Z_I / sum Z, the proposal's log ratio in the test.  Every proposal is evaluated in full.
        replay_draws [steps, B, 5] = (u_electron, u_nucleus, eps[3]), replay_log_u [steps, B].  Returns (n_accept
        per walker, static_max)."""
        p = self._params(params)
        r = electrons
        assert r.is_contiguous() and r.dtype == self.dtype
        B = r.shape[0]
        n_acc = torch.zeros(B, dtype=torch.int32, device=self.device)
        smax = torch.zeros(4, dtype=torch.int32, device=self.device)
        draws = None
        if replay_draws is not None:
            draws = torch.as_tensor(np.asarray(replay_draws)).to(self.device, self.dtype).reshape(steps, B, 5)
            draws = draws.contiguous()
        logu = None if replay_log_u is None else torch.as_tensor(replay_log_u).to(self.device, self.dtype).contiguous()
        r0 = r.clone()
        lp0 = logpsi.clone()

        def fn(prob, ws):
            prob.chunk_walkers = int(self.value_chunk_walkers)
            r.copy_(r0)
            logpsi.copy_(lp0)
            n_acc.zero_()
            smax.zero_()
            _lib.check(_lib.load().fire_mcmc_jump_block(
                self._stream(), C.byref(prob), C.c_void_p(self.R_dev.data_ptr()), C.c_void_p(self.Z_dev.data_ptr()),
                C.c_void_p(p.prepared.data_ptr()), C.c_void_p(r.data_ptr()), C.c_void_p(logpsi.data_ptr()),
                int(steps), float(sigma), C.c_uint64(seed), C.c_uint64(counter),
                C.c_void_p(draws.data_ptr()) if draws is not None else None,
                C.c_void_p(logu.data_ptr()) if logu is not None else None, C.c_void_p(n_acc.data_ptr()),
                C.c_void_p(smax.data_ptr()), C.c_void_p(ws.data_ptr()), C.c_size_t(ws.numel()),
                C.c_void_p(self._status.data_ptr())), "fire_mcmc_jump_block")

        self._run(fn, static, B)
        sm = smax.cpu().numpy()
        return n_acc, StaticArgs(int(sm[0]), int(sm[1]), 0, int(sm[3]))

    def mcmc_cluster_block(self, params, electrons: torch.Tensor, logpsi: torch.Tensor, static: StaticArgs,
                           steps: int, width: float, max_cluster_size: int = 5, max_cluster_radius: float = 2.0,
                           sweep_type: str = "sequential", step_offset: int = 0, seed: int = 0, counter: int = 0,
                           replay_draws=None, replay_log_u=None):
        """In-place Metropolis block of cluster updates (``proposal_cluster_update``, ``mcmc.py:119-161``): each step
        moves the electrons closest to a center (sequential or random) that lie within ``max_cluster_radius`` and
        keeps the first of 5 draws whose cluster is unchanged around the moved center (none: rejected).  Every
        proposal is evaluated in full.  replay_draws [steps, B, 1 + 15 k] = (u_center, eps [5][k][3]) with
        k = min(max_cluster_size, n_el), replay_log_u [steps, B].  Returns (n_accept per walker, static_max)."""
        if sweep_type not in ("sequential", "random"):
            raise ValueError(f"Invalid sweep_type: {sweep_type}")
        p = self._params(params)
        r = electrons
        assert r.is_contiguous() and r.dtype == self.dtype
        B = r.shape[0]
        k = min(int(max_cluster_size), self.mol.n_el)
        n_acc = torch.zeros(B, dtype=torch.int32, device=self.device)
        smax = torch.zeros(4, dtype=torch.int32, device=self.device)
        draws = None
        if replay_draws is not None:
            draws = torch.as_tensor(np.asarray(replay_draws)).to(self.device, self.dtype).reshape(steps, B, 1 + 15 * k)
            draws = draws.contiguous()
        logu = None if replay_log_u is None else torch.as_tensor(replay_log_u).to(self.device, self.dtype).contiguous()
        r0 = r.clone()
        lp0 = logpsi.clone()

        def fn(prob, ws):
            prob.chunk_walkers = int(self.value_chunk_walkers)
            r.copy_(r0)
            logpsi.copy_(lp0)
            n_acc.zero_()
            smax.zero_()
            _lib.check(_lib.load().fire_mcmc_cluster_block(
                self._stream(), C.byref(prob), C.c_void_p(self.R_dev.data_ptr()), C.c_void_p(self.Z_dev.data_ptr()),
                C.c_void_p(p.prepared.data_ptr()), C.c_void_p(r.data_ptr()), C.c_void_p(logpsi.data_ptr()),
                int(steps), int(step_offset), float(width), int(max_cluster_size), float(max_cluster_radius),
                1 if sweep_type == "random" else 0, C.c_uint64(seed), C.c_uint64(counter),
                C.c_void_p(draws.data_ptr()) if draws is not None else None,
                C.c_void_p(logu.data_ptr()) if logu is not None else None, C.c_void_p(n_acc.data_ptr()),
                C.c_void_p(smax.data_ptr()), C.c_void_p(ws.data_ptr()), C.c_size_t(ws.numel()),
                C.c_void_p(self._status.data_ptr())), "fire_mcmc_cluster_block")

        self._run(fn, static, B)
        sm = smax.cpu().numpy()
        return n_acc, StaticArgs(int(sm[0]), int(sm[1]), 0, int(sm[3]))

def make_local_energy(wf: FireWaveFunction, pseudopotentials=None):
    """``make_local_energy`` (``hamiltonian.py:49-83``): ``local_energy(key, params, electrons, static) -> (E_loc,
    new_static)``.  With pseudopotentials (the ``DeviceEcp`` of the molecule's ``EcpTables``; the wavefunction's
    molecule then carries the effective charges) the local and non-local pseudopotential terms are added, the
    quadrature rotations keyed by key (an integer seed)."""

    def local_energy(key, params, electrons, static: StaticArgs):
        eloc, aux = wf.local_energy_full(params, electrons, static)
        if pseudopotentials is not None:
            e_pp, _ = wf.ecp_energy(params, electrons, aux["static"], pseudopotentials, seed=int(key))
            eloc = eloc + e_pp
        return eloc, aux["static"]

    return local_energy


@dataclasses.dataclass(frozen=True)
class WidthSchedulerState:
    """``WidthSchedulerState`` (``mcmc.py:349-378``): the proposal width, the ring of the last window_size
    acceptance rates and the number of updates so far (float32 values, as in the reference)."""

    width: np.float32
    pmoves: tuple
    i: int


def make_width_scheduler(window_size: int = 20, target_pmove: float = 0.5, error: float = 0.025,
                         width_multiplier: float = 1.1):
    """``make_width_scheduler`` (``mcmc.py:349-378``): returns (init, update).  update(state, pmove) stores pmove in
    the ring and, on the calls whose count so far is a multiple of window_size (the first call included), divides the
    width by width_multiplier if the ring's mean is below target_pmove - error and multiplies it if above
    target_pmove + error.  As in the reference the mean is that of the ring before pmove is stored, so the first call
    sees the zero-initialised ring and narrows the width."""
    mult = np.float32(width_multiplier)

    def init(init_width: float) -> WidthSchedulerState:
        return WidthSchedulerState(np.float32(init_width), (np.float32(0.0),) * window_size, 0)

    def update(state: WidthSchedulerState, pmove: float) -> WidthSchedulerState:
        ring = list(state.pmoves)
        ring[state.i % window_size] = np.float32(pmove)
        pm_mean = np.mean(np.asarray(state.pmoves, np.float32), dtype=np.float32)
        width = state.width
        if state.i % window_size == 0:
            if pm_mean < np.float32(target_pmove - error):
                width = np.float32(width / mult)
            if pm_mean > np.float32(target_pmove + error):
                width = np.float32(width * mult)
        return WidthSchedulerState(width, tuple(ring), state.i + 1)

    return init, update


def make_mcmc(wf: FireWaveFunction, steps: int = 20, init_width: float = 0.1, proposal: str = "all-electron",
              sweeps: float = 2.0, jump_steps: int = 0, max_cluster_size: int = 5, max_cluster_radius: float = 2.0,
              sweep_type: str = "sequential", low_rank: bool = True):
    """``make_mcmc`` (``mcmc.py:278-346``) for the "all-electron" proposal (``steps`` moves of every electron) and
    the "single-electron" proposal (``int(sweeps * n_el)`` one-electron moves in sequential order, the reference's
    default; ``init_width`` 0.5 there, ``config/default.yaml``), preceded by ``jump_steps`` jumps to the nuclei
    (sigma 2, ``mcmc.py:320-326, 332-335``; 20 in the reference's defaults); "cluster-update" runs
    ``int(sweeps * n_el)`` cluster moves (``mcmc.py:305-316``; sequential sweeps must be whole):
    ``mcmc_step(key, params, electrons, static, width) -> (electrons, stats)`` with key an integer seed.  low_rank
    (the default, as the reference's ``mcmc_steps_low_rank``) evaluates the single-electron moves, the cluster updates
    and the jumps from a state per walker (``mcmc_low_rank_block``, ``mcmc_low_rank_cluster_block``,
    ``mcmc_low_rank_jump_block``); low_rank=False evaluates every proposal in full.  stats then also hold the move
    statics."""
    proposal = proposal.lower()
    if proposal not in ("all-electron", "single-electron", "cluster-update"):
        raise ValueError(f"Invalid proposal: {proposal}")
    n_steps = steps if proposal == "all-electron" else int(sweeps * wf.mol.n_el)
    if proposal == "cluster-update":
        if sweep_type == "sequential" and n_steps % wf.mol.n_el != 0:
            raise ValueError("Number of sweeps must be integer for sequential sweep")
        if n_steps <= 0:
            raise ValueError("Number of steps (sweeps * n_el) must be greater than 0")

    def mcmc_step(key, params, electrons, static: StaticArgs, width):
        p = wf._params(params)
        r = wf._electrons(electrons).clone()
        _, logpsi = wf.signed(p, r, static)
        stats = {}
        if jump_steps > 0:  # the reference keeps the jump block's statics apart (static_max["mcmc_jump"])
            if low_rank:
                n_jump, smax_jump, stats["changed_max_jump"] = wf.mcmc_low_rank_jump_block(
                    p, r, logpsi, static, jump_steps, 2.0, seed=int(key), counter=1)
            else:
                n_jump, smax_jump = wf.mcmc_jump_block(p, r, logpsi, static, jump_steps, 2.0, seed=int(key),
                                                       counter=1)
            stats["pmove_jump"] = float(n_jump.float().mean().item()) / jump_steps
            stats["static_max_jump"] = smax_jump
        if proposal == "all-electron":
            n_acc, smax = wf.mcmc_block(p, r, logpsi, static, n_steps, float(width), seed=int(key))
        elif proposal == "cluster-update" and low_rank:
            n_acc, smax, stats["changed_max"] = wf.mcmc_low_rank_cluster_block(
                p, r, logpsi, static, n_steps, float(width), max_cluster_size, max_cluster_radius, sweep_type,
                seed=int(key))
        elif proposal == "cluster-update":
            n_acc, smax = wf.mcmc_cluster_block(p, r, logpsi, static, n_steps, float(width), max_cluster_size,
                                                max_cluster_radius, sweep_type, seed=int(key))
        elif low_rank:
            n_acc, smax, stats["changed_max"] = wf.mcmc_low_rank_block(p, r, logpsi, static, n_steps, float(width),
                                                                       seed=int(key))
        else:
            n_acc, smax = wf.mcmc_single_block(p, r, logpsi, static, n_steps, float(width), seed=int(key))
        stats.update(pmove=float(n_acc.float().mean().item()) / max(n_steps, 1), static_max=smax, stepsize=width)
        return r, stats

    return mcmc_step, init_width
