#!/usr/bin/env python
"""Benchmark of the FiRE local-energy hot path: walker E_loc evaluations per second.

Workload (default): all-trans C40H82 (322 electrons, 122 nuclei), 2048 walkers drawn around the nuclei
(sigma = 1 bohr), random-init default-architecture parameters (seed 0), e-e cutoff 5 bohr.  The walkers
first go through one 20-step all-electron Metropolis block (Gaussian proposals, width 0.1 bohr, Philox draws
of seed 1000; a warm-up block runs on a copy); then one step = one local-energy evaluation (sparse forward
Laplacian + Coulomb potential) of every walker.  Synthetic data: there is no dataset; molecules, walkers and
parameters are generated here.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--precision mixed|fp32] [--impl reference]

Prints one JSON line (rank 0).  `value` is the headline path's device-resident throughput (inputs
already in HBM; default the mixed path), `e2e` the same metric through the public API with the walkers
copied from pinned host memory and E_loc copied back inside the timed region.  `fp32_path` times the
plain FP32 path on the same walkers the same way; `accuracy` compares both with the FP64 build on a
sample of the walkers.  `--impl reference` times the CPU oracle (the numpy FP64 restatement of the reference
algorithm) on a sample of the same workload: the same parameters, the same Metropolis block replayed from the
same Philox draws, one walker per host core.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "walker E_loc evals/s"
UNIT = "walker-evals/s"
SYSTEMS = {"c40h82": 40, "c10h22": 10, "c2h6": 2}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["fp32", "mixed"], help="the timed (headline) path")
    ap.add_argument("--system", default="c40h82", choices=list(SYSTEMS))
    ap.add_argument("--walkers", type=int, default=2048)
    ap.add_argument("--chunk", type=int, default=0, help="walkers per internal pass (0: from --ws-gb)")
    ap.add_argument("--ws-gb", type=float, default=48.0, help="workspace budget in GB")
    ap.add_argument("--mcmc-steps", type=int, default=20, help="Metropolis steps before the E_loc evaluation")
    ap.add_argument("--mcmc-width", type=float, default=0.1)
    ap.add_argument("--mcmc-single-steps", type=int, default=32,
                    help="single-electron Metropolis steps timed on a copy of the walkers (0: skip)")
    ap.add_argument("--mcmc-single-width", type=float, default=0.5)
    ap.add_argument("--mcmc-low-rank-steps", type=int, default=32,
                    help="single-electron steps of the low-rank block, timed on a copy of the walkers (0: skip)")
    ap.add_argument("--acc-walkers", type=int, default=1024,
                    help="walkers checked against the FP64 build (0: no comparison with the FP64 build, and so no "
                         "smaller configurations either)")
    ap.add_argument("--no-compare", action="store_true", help="skip timing the FP32 path beside the mixed one")
    ap.add_argument("--grad-walkers", type=int, default=256,
                    help="walkers of the per-walker parameter-gradient segment (0: skip)")
    ap.add_argument("--serving-requests", type=int, default=20, help="requests of the serving segment (0: skip)")
    ap.add_argument("--serving-rate", type=float, default=200.0, help="offered load, requests per second")
    ap.add_argument("--serving-carbons", default="4,60", help="alkane sizes C_n of the serving requests (min,max)")
    ap.add_argument("--serving-walkers", default="256,2048", help="walkers per serving request (min,max)")
    ap.add_argument("--no-ragged", action="store_true",
                    help="skip the 64-alkane ragged batch (one CUDA-graph launch vs one call per molecule)")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the smaller configurations (H10 x 512: FP32 and FP64; C10H22 x 4096: mixed and FP32)")
    ap.add_argument("--cpu-sample", type=int, default=0,
                    help="walkers in the CPU samples (0: one per host core, at most 16)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    return ap.parse_args()


def config_segments(args, dev, stream):
    """The benchmark's smaller configurations beside the headline one (world size 1), on walkers drawn around the
    nuclei (sigma 1 bohr, seed 1000; no Metropolis block) with random-init parameters (seed 0, normalize scales
    from walker 0):
      C1: H10 chain (1.8 bohr spacing), 512 walkers: the FP32 path and the FP64 build;
      C2: C10H22, 4096 walkers: the mixed and the plain FP32 path.
    Each path is timed like the headline step (warm-up steps, then timed steps) and its per-walker and mean-energy
    error stated against the FP64 build of the same kernels on the same walkers and parameters (all 512 walkers of
    C1, the first 1024 of C2)."""
    import numpy as np
    import torch

    from sparse_wf_gb300 import systems
    from sparse_wf_gb300.wavefunction import FireWaveFunction

    out = {}
    for key, mol, walkers, paths, K in (("C1", systems.hydrogen_chain(10, 1.8), 512, ("fp32", "fp64"), 512),
                                        ("C2", systems.alkane(10), 4096, ("mixed", "fp32"), 1024)):
        n_up, _ = systems.spin_counts(mol)
        r_np = systems.init_electrons(mol, walkers, 1000)
        seg = {"molecule": mol.name, "n_el": mol.n_el, "walkers": walkers, "error_walkers": K}
        params, e = None, {}
        # the timed paths, then (C2) the FP64 build once on the first K walkers as the reference
        runs = [(p, walkers, True) for p in paths] + ([("fp64", K, False)] if "fp64" not in paths else [])
        for prec, nw, timed in runs:
            wf = FireWaveFunction(mol, precision=prec, device=dev)
            if params is None:
                params = wf.init(0, r_np[:1])
            rr = r_np[:nw].astype(np.float64) if prec == "fp64" else r_np[:nw]
            r = torch.from_numpy(rr).to(dev)
            static = wf.get_static_input(r).round_with_padding(1.1, mol.n_el, n_up, mol.n_nuc)
            # walkers per pass: the workspace budget, and (as the library's own choice does) at most 65535 row
            # tiles of 64 for the pass's Jacobian planes
            grid_cap = max(1, 65535 * 64 // (3 * (mol.n_el + static.n_pairs)))
            wf.chunk_walkers = min(choose_chunk(wf, nw, static, args.ws_gb), grid_cap) if timed else min(nw, 64)
            dp = wf._params(params)
            st = {"static": static}

            def step():
                return wf.local_energy_full(dp, r, st["static"])

            if timed:
                for _ in range(args.warmup):
                    eloc, aux = step()
                    st["static"] = aux["static"]
                ms, (eloc, aux) = time_steps(step, args.steps, stream, None, 1)
                seg[prec] = {"value": nw / (ms / 1e3), "unit": UNIT, "ms_per_step": ms,
                             "chunk_walkers": wf.chunk_walkers, "refined_walkers": int(aux.get("refined", 0))}
            else:
                eloc, aux = step()
            e[prec] = eloc.double().cpu().numpy()
            del wf, dp, r, step
            torch.cuda.empty_cache()
        for prec in paths:
            if prec != "fp64":
                seg[prec]["error_vs_fp64"] = energy_error(e[prec][:K], e["fp64"][:K])
        if "mixed" in seg and "fp32" in seg:
            seg["mixed_over_fp32"] = seg["mixed"]["value"] / seg["fp32"]["value"]
        out[key] = seg
    return out


def molecule(name):
    from sparse_wf_gb300 import systems

    return systems.alkane(SYSTEMS[name])


def workload_config(args, mol):
    """The workload both arms report (identical in the reference arm's line and in this one)."""
    return {"workload": f"{mol.name} all-trans, {args.walkers} walkers per GPU after a {args.mcmc_steps}-step "
                        f"all-electron Metropolis block (width {args.mcmc_width} bohr, Philox draws of seed 1000); "
                        f"step = local energy (sparse forward Laplacian + Coulomb) of every walker",
            "n_el": mol.n_el, "n_nuc": mol.n_nuc, "walkers_per_gpu": args.walkers, "mcmc_steps": args.mcmc_steps,
            "mcmc_width_bohr": args.mcmc_width, "params": "random init, seed 0; normalize scales from walker 0",
            "l2": "inputs larger than L2: every step streams GB-scale planes",
            "parallelism": f"walker shards x{args.gpus}"}


# ------------------------------------------------------------------------ CPU oracle pool
# The CPU baseline and the reference arm time the oracle (numpy FP64, one walker per process, one BLAS thread
# each).  The pool is started with "spawn": a process forked from one that holds a CUDA context can hang.
_POOL = {}


def _pool_init(R, Z, n_up, params):
    from oracle import fire_oracle as O

    _POOL["prob"] = O.Problem(R, Z, n_up)
    _POOL["p"] = params


def _pool_eloc(r):
    import numpy as np
    from oracle import fire_oracle as O

    return float(O.local_energy(_POOL["prob"], _POOL["p"], np.asarray(r, np.float64)))


def _pool_mcmc(job):
    from oracle import fire_oracle as O

    walker, r, steps, width, seed, counter = job
    r_new, n_acc, margins = O.mcmc_block_philox(_POOL["prob"], _POOL["p"], r, steps, width, seed, counter, walker)
    return r_new, n_acc, float(min(abs(m) for m in margins)) if len(margins) else float("inf")


def oracle_pool(mol, n_up, params, procs):
    import multiprocessing as mp

    for k in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):
        os.environ[k] = "1"
    return mp.get_context("spawn").Pool(procs, initializer=_pool_init, initargs=(mol.R, mol.Z, n_up, params))


def cpu_sample_size(args):
    return args.cpu_sample if args.cpu_sample > 0 else max(1, min(os.cpu_count() or 1, 16))


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum, ncu) of the tensor-core contractions of one mixed-path
# C40H82 local energy, per walker: 6.615 GB over the 25 k_gemm_tca / k_env_tc launches of a 16-walker step.  Every
# launch's rows, and so its traffic, grow in proportion to the walkers.
TC_TRAFFIC_PER_WALKER = {("c40h82", "mixed"): 6.615e9 / 16}


def gemm_flops(n, N, pairs, value_rows=True, derivative_rows=True):
    """Algorithmic FLOPs (2 per multiply-add) of the dense contractions of one walker's E_loc: of the value rows
    (one per node), of the derivative rows (Jacobian and Laplacian rows; the mixed path's tensor-core share), or
    both."""
    F, D = 256, 4
    rows = (n if value_rows else 0) + ((n + 3 * (n + pairs)) if derivative_rows else 0)  # rows of a sparse node
    e5 = (1 if value_rows else 0) + (4 if derivative_rows else 0)  # ElecInit / envelope rows per electron
    f = e5 * n * 2 * F * (2 * F + F + 5 * F)  # ElecInit GLU / Dense / Dense on [x, jac(3), lap]
    f += 2 * rows * 2 * F * F  # update MLP
    f += e5 * n * 2 * (8 * N) * n * D  # envelope contraction
    f += rows * 2 * F * D * n  # orbitals (needed spin only)
    f += rows * 2 * F * F  # attention values
    f += 2 * rows * 2 * F * F  # MLP Jastrow hidden layers
    if value_rows and derivative_rows:
        f += (3 * n + 2) * 2 * (2 * F * F + F * F + 2 * F)  # attention readout MLP (dense tangents)
    return float(f)


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.p is not None:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.p.kill()
        self.f.flush()

    def summary(self):
        rows = []
        try:
            for line in Path(self.f.name).read_text().splitlines():
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        except OSError:
            pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def cpu_baseline(pool, walkers):
    """Oracle E_loc of `walkers` (one per process of `pool`), timed: (walker-evals/s, energies, seconds)."""
    import numpy as np

    t0 = time.perf_counter()
    e = pool.map(_pool_eloc, [w for w in walkers], chunksize=1)
    dt = time.perf_counter() - t0
    return len(walkers) / dt, np.array(e), dt


def run_reference(args):
    """CPU reference arm: the oracle (numpy FP64 restatement of the reference algorithm) on a sample of the same
    workload: the reference's own initialisation of the parameters (normalize scales from walker 0, computed by the
    oracle in FP64), the first S walkers of the same initial set, the benchmark's Metropolis block replayed from the
    device's Philox draws (float32 positions, as on the device), then W + K steps of E_loc of the S walkers, one per
    host core."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import numpy as np

    sys.path.insert(0, str(ROOT / "tests" / "golden"))
    from make_golden import make_params
    from sparse_wf_gb300 import systems

    mol = molecule(args.system)
    n_up, _ = systems.spin_counts(mol)
    S = cpu_sample_size(args)
    r = systems.init_electrons(mol, args.walkers * args.gpus, 1000)[:max(S, 1)]
    _, p, _, _ = make_params(mol, n_up, r[0], seed=0, activate=False)
    t_setup = time.perf_counter()
    acc, closest = 0.0, float("inf")
    with oracle_pool(mol, n_up, p, S) as pool:
        if args.mcmc_steps > 0:
            res = pool.map(_pool_mcmc, [(w, r[w], args.mcmc_steps, args.mcmc_width, 1000, 0) for w in range(S)],
                           chunksize=1)
            r = np.stack([x[0] for x in res])
            acc = float(np.mean([x[1] for x in res])) / args.mcmc_steps
            closest = min(x[2] for x in res)
        t_setup = time.perf_counter() - t_setup
        for _ in range(args.warmup):
            cpu_baseline(pool, r)
        times = []
        for _ in range(args.steps):
            _, _, dt = cpu_baseline(pool, r)
            times.append(dt)
    ms = 1e3 * statistics.mean(times)
    v = S / (ms / 1e3)
    sample = (f"{S} of the {args.walkers} {mol.name} walkers per step (one per host core), after the same "
              f"{args.mcmc_steps}-step Metropolis block replayed from the device's Philox draws "
              f"(acceptance {acc:.3f}, smallest |margin| {closest:.2e}; set-up {t_setup:.0f} s); numpy FP64 oracle"
              if args.mcmc_steps > 0 else f"{S} of the {args.walkers} {mol.name} walkers per step")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": workload_config(args, mol),
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": S, "kind": "port", "sample": sample},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def energy_error(e_path, e_ref):
    """Per-walker and mean-energy differences (mHa) of two E_loc arrays of the same walkers; the clipped
    mean is the one the reference's optimizer uses (median +- 5 mean-absolute-deviations,
    update.py:45-62, 158-160; clip_local_energy 5.0, default.yaml:137-139)."""
    import numpy as np

    def clipped_mean(e):
        c = np.median(e)
        mad = np.mean(np.abs(e - c))
        return float(np.clip(e, c - 5 * mad, c + 5 * mad).mean())

    d = np.abs(e_path - e_ref) * 1e3
    return {"max_abs_mHa": float(d.max()), "median_abs_mHa": float(np.median(d)),
            "mean_energy_err_mHa": float(abs(e_path.mean() - e_ref.mean()) * 1e3),
            "clipped_mean_energy_err_mHa": float(abs(clipped_mean(e_path) - clipped_mean(e_ref)) * 1e3)}


def choose_chunk(wf, B, static, ws_gb):
    """The largest walker chunk whose workspace fits the budget."""
    import ctypes as C

    from sparse_wf_gb300 import _lib

    lo, hi = 1, B
    while lo < hi:
        mid = (lo + hi + 1) // 2
        prob = wf._problem(B, static)
        nb = C.c_size_t()
        _lib.check(_lib.load().fire_workspace_size(C.byref(prob), mid, C.byref(nb)), "fire_workspace_size")
        if nb.value <= ws_gb * 1e9:
            lo = mid
        else:
            hi = mid - 1
    return lo


def time_steps(step, n, stream, dist, world):
    """Device time (ms) of one step averaged over n steps, bracketed by barriers and synchronizes; max over
    ranks."""
    import torch

    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    e0.record(stream)
    out = None
    for _ in range(n):
        out = step()
    e1.record(stream)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    ms = e0.elapsed_time(e1) / n
    if world > 1:
        t = torch.tensor([ms], device=stream.device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    return ms, out


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    import numpy as np
    import torch
    import torch.distributed as dist

    from sparse_wf_gb300 import _lib, systems
    from sparse_wf_gb300.build import build
    from sparse_wf_gb300.distributed import shard
    from sparse_wf_gb300.wavefunction import FireWaveFunction

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        dist.init_process_group("nccl", device_id=dev)
    if rank == 0:
        build()
    if world > 1:
        dist.barrier()

    mol = molecule(args.system)
    n_up, _ = systems.spin_counts(mol)
    r_all = systems.init_electrons(mol, args.walkers * world, 1000)  # weak scaling: walkers per GPU fixed
    a, b = shard(len(r_all), rank, world)
    B = b - a
    wf = FireWaveFunction(mol, precision=args.precision, device=dev)
    params = wf.init(0, r_all[:1])
    dp = wf._params(params)
    r_dev = torch.from_numpy(r_all[a:b]).to(dev)
    static = wf.get_static_input(r_dev).round_with_padding(1.1, mol.n_el, n_up, mol.n_nuc)
    wf.chunk_walkers = args.chunk if args.chunk > 0 else choose_chunk(wf, B, static, args.ws_gb)
    stream = torch.cuda.current_stream(dev)

    # Metropolis block (all-electron Gaussian proposals, Philox draws of seed 1000 + rank, counter 0) that moves the
    # walkers before the E_loc steps; an untimed warm-up block (counter 1) runs on a copy first
    mcmc = None
    if args.mcmc_steps > 0:
        _, logpsi = wf.signed(dp, r_dev, static)
        r_w, lp_w = r_dev.clone(), logpsi.clone()
        wf.mcmc_block(dp, r_w, lp_w, static, args.mcmc_steps, args.mcmc_width, seed=1000 + rank, counter=1)
        del r_w, lp_w
        blk = {}

        def block():
            blk["acc"], blk["smax"] = wf.mcmc_block(dp, r_dev, logpsi, static, args.mcmc_steps, args.mcmc_width,
                                                    seed=1000 + rank, counter=0)

        ms_block, _ = time_steps(block, 1, stream, dist, world)
        acc = float(blk["acc"].float().mean().item()) / args.mcmc_steps
        mcmc = {"steps": args.mcmc_steps, "width_bohr": args.mcmc_width, "ms_per_block": ms_block,
                "walker_steps_per_s": B * world * args.mcmc_steps / (ms_block / 1e3), "acceptance": acc,
                "precision": args.precision}
        if args.mcmc_single_steps > 0:
            # single-electron proposals (the reference's default, sequential sweep) on a copy of the walkers, so
            # the E_loc workload below is unchanged
            r1, lp1 = r_dev.clone(), logpsi.clone()
            blk1 = {}

            def block1():
                blk1["acc"], _ = wf.mcmc_single_block(dp, r1, lp1, static, args.mcmc_single_steps,
                                                      args.mcmc_single_width, seed=2000 + rank, counter=0)

            ms1, _ = time_steps(block1, 1, stream, dist, world)
            mcmc["single_electron"] = {
                "steps": args.mcmc_single_steps, "width_bohr": args.mcmc_single_width, "ms_per_block": ms1,
                "walker_steps_per_s": B * world * args.mcmc_single_steps / (ms1 / 1e3),
                "acceptance": float(blk1["acc"].float().mean().item()) / args.mcmc_single_steps,
                "evaluation": "every proposal by the full value path (no low-rank update)"}
            del r1, lp1
        if args.mcmc_low_rank_steps > 0:
            # the same proposals evaluated from a state per walker (fire_mcmc_low_rank_block): one untimed block
            # (it settles the changed-set capacity), then one timed block
            r2, lp2 = r_dev.clone(), logpsi.clone()
            blk2 = {}

            def block2():
                blk2["acc"], _, blk2["changed"] = wf.mcmc_low_rank_block(
                    dp, r2, lp2, static, args.mcmc_low_rank_steps, args.mcmc_single_width, seed=3000 + rank,
                    counter=0)

            block2()
            ms2, _ = time_steps(block2, 1, stream, dist, world)
            mcmc["single_electron_low_rank"] = {
                "steps": args.mcmc_low_rank_steps, "width_bohr": args.mcmc_single_width, "ms_per_block": ms2,
                "walker_steps_per_s": B * world * args.mcmc_low_rank_steps / (ms2 / 1e3),
                "acceptance": float(blk2["acc"].float().mean().item()) / args.mcmc_low_rank_steps,
                "changed_max": list(blk2["changed"]), "cap_changed": wf._lr_cap,
                "evaluation": "low-rank update of a state per walker (state built once per block)"}
            del r2, lp2
        static = wf.get_static_input(r_dev).round_with_padding(1.1, mol.n_el, n_up, mol.n_nuc)
    r_np = r_dev.cpu().numpy()

    def step():
        return wf.local_energy_full(dp, r_dev, static)

    for _ in range(args.warmup):
        eloc, aux = step()
        static = aux["static"]
    with ClockSampler(local) as clk:
        ms, (eloc, aux) = time_steps(step, args.steps, stream, dist, world)
    total_walkers = args.walkers * world
    value = total_walkers / (ms / 1e3)
    e_stats = aux["stats"].cpu().numpy()
    refined = {args.precision: int(aux.get("refined", 0))}  # ill-conditioned walkers of the last timed step

    # per-stage device times (CUDA events around every stage / contraction launch) for the roofline
    _lib.profile_enable(True)
    step()
    torch.cuda.synchronize()
    prof = _lib.profile_report()
    _lib.profile_enable(False)
    counts = wf.neighbor_lists(r_dev[: min(B, 64)], static)["counts"]
    pairs = float(np.mean(counts[:, 0] + counts[:, 1]))
    peaks, peak_kind = measured_peaks()
    # the contractions run inside a seconds-long step: the sustained bf16 figure is their ceiling
    peak = peaks["bf16_tflops_sustained"]
    if args.precision == "mixed":
        # the tensor-core contractions (the Jacobian and Laplacian rows): their FLOPs over their launches' time
        flops = gemm_flops(mol.n_el, mol.n_nuc, pairs, value_rows=False) * B
        g_launches, g_ms = prof.get("gemm_tc", (0, float("nan")))
        kernel = "tensor-core contractions of one step (k_gemm_tca, k_env_tc: the Jacobian and Laplacian rows)"
    else:
        flops = gemm_flops(mol.n_el, mol.n_nuc, pairs) * B
        g_launches = prof.get("gemm", (0, 0.0))[0] + prof.get("gemm_comp", (0, 0.0))[0]
        g_ms = prof.get("gemm", (0, 0.0))[1] + prof.get("gemm_comp", (0, 0.0))[1]
        kernel = "all dense contractions of one step (CUDA cores: k_gemm, k_gemm_comp)"
    achieved = flops / (g_ms / 1e3) / 1e12
    tpw = TC_TRAFFIC_PER_WALKER.get((args.system, args.precision))
    traffic = tpw * B / max(g_launches, 1) if tpw else None  # bytes per launch, like achieved
    roofline = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                "frac": achieved / peak, "traffic": traffic, "kernel": kernel, "launches": g_launches,
                "avg_launch_ms": g_ms / max(g_launches, 1), "peak_source": f"bf16 dense sustained, {peak_kind}",
                "flops_per_step": flops}
    # the CUDA-core value-row contractions beside it (compensated; their FLOPs over their launches' time)
    vc_launches, vc_ms = prof.get("gemm_comp", (0, float("nan")))
    vflops = gemm_flops(mol.n_el, mol.n_nuc, pairs, derivative_rows=False) * B
    roofline["value_rows"] = {"kernel": "k_gemm_comp (compensated value rows)", "launches": vc_launches, "ms": vc_ms,
                              "flops_per_step": vflops, "tflops": vflops / (vc_ms / 1e3) / 1e12}
    stages = {k: {"launches": v[0], "ms": v[1]} for k, v in prof.items() if k != "kernels_launched"}

    # end to end through the public API: pinned host walkers in, E_loc out, every step
    e2e = None
    if not args.no_e2e:
        r_host = torch.from_numpy(r_np).pin_memory()
        e_host = torch.empty(B, dtype=torch.float32).pin_memory()

        def e2e_step():
            r_dev.copy_(r_host, non_blocking=True)
            e, _ = step()
            e_host.copy_(e, non_blocking=True)

        t0 = time.perf_counter()
        ms_e2e, _ = time_steps(e2e_step, args.steps, stream, dist, world)
        ms_e2e = max(ms_e2e, (time.perf_counter() - t0) * 1e3 / args.steps)
        e2e = {"value": total_walkers / (ms_e2e / 1e3), "unit": UNIT, "h2d_bytes_per_step": int(r_host.numel() * 4),
               "d2h_bytes_per_step": int(e_host.numel() * 4)}

    # accuracy against the FP64 build of the same kernels (which matches the oracle to 1e-10) on the
    # same walkers and parameters
    accuracy = None
    e_path = {args.precision: eloc.double().cpu().numpy()}
    K = min(args.acc_walkers, B)
    e64 = None
    if K > 0:
        wf._ws = None
        torch.cuda.empty_cache()
        wf64 = FireWaveFunction(mol, precision="fp64", device=dev)
        wf64.chunk_walkers = min(K, 64)
        r64 = r_dev[:K].double()
        st64 = wf64.get_static_input(r64).round_with_padding(1.1, mol.n_el, n_up, mol.n_nuc)
        e64 = wf64.local_energy_full(params, r64, st64)[0].cpu().numpy()
        del wf64
        torch.cuda.empty_cache()

    # the plain FP32 path on the same walkers, timed the same way
    fp32 = None
    if args.precision == "mixed" and not args.no_compare:
        wf._ws = None
        torch.cuda.empty_cache()
        wf32 = FireWaveFunction(mol, precision="fp32", device=dev)
        wf32.chunk_walkers = wf.chunk_walkers
        dp32 = wf32._params(params)
        st32 = static

        def step32():
            return wf32.local_energy_full(dp32, r_dev, st32)

        for _ in range(args.warmup):
            e32, aux32 = step32()
            st32 = aux32["static"]
        ms32, (e32, aux32) = time_steps(step32, args.steps, stream, dist, world)
        refined["fp32"] = int(aux32.get("refined", 0))
        e_path["fp32"] = e32.double().cpu().numpy()
        fp32 = {"value": total_walkers / (ms32 / 1e3), "unit": UNIT, "ms_per_step": ms32,
                "chunk_walkers": wf32.chunk_walkers}
        del wf32
        torch.cuda.empty_cache()
    if e64 is not None:
        accuracy = {"walkers": K, "reference": "FP64 build of the same kernels (FP64 oracle to <= 1e-10)"}
        accuracy.update({k: energy_error(v[:K], e64) for k, v in e_path.items()})
        for k in e_path:  # walkers of the whole batch that went through the FP64 refinement pass
            accuracy[k]["refined_fraction"] = refined.get(k, 0) / B

    # per-walker gradient of log|psi| with respect to every parameter (the SPRING Jacobian rows) on the first
    # post-Metropolis walkers: one untimed call, one timed call; rows checked against the FP64 build on 4 walkers
    param_grad = None
    Bg = min(args.grad_walkers, B)
    if Bg > 0:
        wf._ws = None
        torch.cuda.empty_cache()
        rg = r_dev[:Bg].contiguous()
        out = {}

        def grad_step():
            out["g"], _, _ = wf.logpsi_grad(dp, rg, static)

        grad_step()
        ms_g, _ = time_steps(grad_step, 1, stream, dist, world)
        Kg = min(4, Bg)
        g32 = out["g"][:Kg].double().cpu().numpy()
        L = int(out["g"].shape[1])
        del out["g"]
        wf._ws = None
        torch.cuda.empty_cache()
        wf64g = FireWaveFunction(mol, precision="fp64", device=dev)
        r64g = r_dev[:Kg].double()
        g64 = wf64g.logpsi_grad(params, r64g, wf64g.get_static_input(r64g))[0].cpu().numpy()
        del wf64g
        torch.cuda.empty_cache()
        rel_row = np.linalg.norm(g32 - g64, axis=1) / np.linalg.norm(g64, axis=1)
        param_grad = {"walkers": Bg * world, "ms": ms_g, "walker_grads_per_s": Bg * world / (ms_g / 1e3),
                      "params_per_walker": L, "output_gb": Bg * L * 4 / 1e9,
                      "precision": "fp32 (reverse mode on the CUDA cores)",
                      "fp32_vs_fp64_row_rel_err_max": float(rel_row.max()), "checked_walkers": Kg}

    # serving segment: Poisson-arriving E_loc / 10-step MCMC requests of mixed molecule sizes (rank 0)
    serving = None
    if rank == 0 and args.serving_requests > 0:
        from sparse_wf_gb300.serving import ServingEngine, poisson_trace

        wf._ws = None
        torch.cuda.empty_cache()
        nr = tuple(int(x) for x in args.serving_carbons.split(","))
        wr = tuple(int(x) for x in args.serving_walkers.split(","))
        serving = {"offered_rate_per_s": args.serving_rate, "carbons": list(nr), "walkers": list(wr),
                   "mcmc_steps": 10, "slots": 4}
        for prec in ([args.precision, "fp32"] if args.precision == "mixed" and not args.no_compare
                     else [args.precision]):
            trace = poisson_trace(args.serving_requests, args.serving_rate, seed=5, n_range=nr, walker_range=wr)
            eng = ServingEngine(prec, lanes=4, chunk=32, max_carbon=nr[1], max_walkers=wr[1], device=dev)
            serving[prec] = eng.run(trace)
            del eng
            torch.cuda.empty_cache()

    ragged = None
    if rank == 0 and not args.no_ragged:
        from sparse_wf_gb300.ragged import RaggedBatch, ragged_alkanes

        wf._ws = None
        torch.cuda.empty_cache()
        ns, ws = ragged_alkanes(64, seed=4)
        rb = RaggedBatch([systems.alkane(k) for k in ns], ws, args.precision, lanes=4, chunk=64, device=dev)
        rb.run_eager()
        t0 = time.perf_counter()
        rb.run_eager()
        te = time.perf_counter() - t0
        rb.run()
        t0 = time.perf_counter()
        rb.replay()
        torch.cuda.synchronize()
        tg = time.perf_counter() - t0
        ragged = {"molecules": 64, "walkers": int(sum(ws)), "one_graph_launch_s": tg, "per_molecule_calls_s": te,
                  "walker_evals_per_s": sum(ws) / tg, "lanes": 4, "chunk_walkers": 64}
        del rb
        torch.cuda.empty_cache()

    # the smaller configurations (C1, C2), after every segment of the headline workload and only with the
    # comparisons against the FP64 build; a failure there is recorded in the line instead of ending the run
    configs = None
    if world == 1 and not args.no_configs and args.acc_walkers > 0:
        wf._ws = None
        torch.cuda.empty_cache()
        try:
            configs = config_segments(args, dev, stream)
        except Exception as exc:
            configs = {"error": f"{type(exc).__name__}: {exc}"[:400]}
        torch.cuda.empty_cache()

    # CPU baseline + oracle check on the same post-Metropolis walkers (rank 0): the oracle, one walker per core
    cpu = None
    check = None
    if rank == 0 and not args.no_cpu_baseline:
        S = min(cpu_sample_size(args), B)
        with oracle_pool(mol, n_up, params, S) as pool:
            rate, e_ref, dt = cpu_baseline(pool, r_np[:S])
        cpu = {"value": rate, "unit": UNIT, "cores": S, "kind": "port",
               "sample": f"{S} of the {B} post-Metropolis {mol.name} walkers (one per host core), numpy FP64 "
                         f"oracle, {dt:.1f} s"}
        check = {"walkers": S, "reference": "FP64 oracle"}
        for k, v in e_path.items():
            d = np.abs(v[:S] - e_ref)
            check[k] = {"max_abs_err_mHa": float(d.max() * 1e3), "max_rel_err": float((d / np.abs(e_ref)).max())}

    if rank == 0:
        st = e_stats
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            # mixed: FP16 hi + lo operands on the tensor cores with FP32 accumulation, FP32 on the CUDA cores
            "vs_baseline": None, "dtype": "f32" if args.precision == "fp32" else "f16/f32",
            "data": "synthetic",
            "config": workload_config(args, mol),
            "run": {"precision": args.precision, "chunk_walkers": wf.chunk_walkers, "mean_pairs_per_walker": pairs,
                    "cap_pairs": static.n_pairs, "E_mean": float(st[0]), "E_std": float(st[1]),
                    "refined_walkers": refined},
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "clocks": clk.summary(),
            "gpu_launches": int(prof.get("kernels_launched", (0, 0))[0]) * args.steps,
            "fp32_path": fp32, "mixed_over_fp32": (value / fp32["value"]) if fp32 else None,
            "accuracy": accuracy, "mcmc": mcmc, "serving": serving, "ragged": ragged, "stages_ms": stages,
            "oracle_check": check, "param_grad": param_grad, "configs": configs,
        }
        print(json.dumps(line))
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
