#!/usr/bin/env python
"""Benchmark of the FiRE local-energy hot path: walker E_loc evaluations per second.

Workload (default): all-trans C40H82 (322 electrons, 122 nuclei), 2048 walkers drawn around the nuclei
(sigma = 1 bohr), random-init default-architecture parameters (seed 0), e-e cutoff 5 bohr.  One step
= one local-energy evaluation (sparse forward Laplacian + Coulomb potential) of every walker.
Synthetic data: there is no dataset; molecules, walkers and parameters are generated here.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--precision fp32|mixed] [--impl reference]

Prints one JSON line (rank 0).  `value` is device-resident throughput (inputs already in HBM), `e2e`
the same metric through the public API with the walkers copied from pinned host memory and E_loc
copied back inside the timed region.  `--impl reference` times the CPU oracle port of the reference
algorithm (numpy, FP64, all host threads) on a bounded sample of the same workload.
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
    ap.add_argument("--precision", default="fp32", choices=["fp32", "mixed"])
    ap.add_argument("--system", default="c40h82", choices=list(SYSTEMS))
    ap.add_argument("--walkers", type=int, default=2048)
    ap.add_argument("--chunk", type=int, default=0, help="walkers per internal pass (0: from --ws-gb)")
    ap.add_argument("--ws-gb", type=float, default=48.0, help="workspace budget in GB")
    ap.add_argument("--cpu-sample", type=int, default=2, help="walkers in the CPU baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    return ap.parse_args()


def molecule(name):
    from sparse_wf_gb300 import systems

    return systems.alkane(SYSTEMS[name])


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def gemm_flops(n, N, pairs):
    """Algorithmic FLOPs (2 per multiply-add) of the dense contractions of one walker's E_loc."""
    F, D = 256, 4
    rows = 2 * n + 3 * (n + pairs)  # value + Laplacian rows + Jacobian rows of a sparse node
    f = 5 * n * 2 * F * (2 * F + F + 5 * F)  # ElecInit GLU / Dense / Dense on [x, jac(3), lap]
    f += 2 * rows * 2 * F * F  # update MLP
    f += 5 * n * 2 * (8 * N) * n * D  # envelope contraction
    f += rows * 2 * F * D * n  # orbitals (needed spin only)
    f += rows * 2 * F * F  # attention values
    f += 2 * rows * 2 * F * F  # MLP Jastrow hidden layers
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


def cpu_baseline(mol, r, params, n_up, sample):
    """The oracle (numpy FP64 port of the reference algorithm) on `sample` walkers, all host threads."""
    from oracle import fire_oracle as O
    import numpy as np

    prob = O.Problem(mol.R, mol.Z, n_up)
    t0 = time.perf_counter()
    e = [O.local_energy(prob, params, r[k].astype(np.float64)) for k in range(sample)]
    dt = time.perf_counter() - t0
    return sample / dt, np.array(e), dt


def run_reference(args):
    """CPU reference arm: the oracle port timed on bounded samples of the workload."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import numpy as np

    sys.path.insert(0, str(ROOT / "tests" / "golden"))
    from make_golden import make_params
    from sparse_wf_gb300 import systems

    mol = molecule(args.system)
    n_up, _ = systems.spin_counts(mol)
    r = systems.init_electrons(mol, max(args.cpu_sample, 1), 1000)
    _, p, _, _ = make_params(mol, n_up, r[0])
    for _ in range(min(args.warmup, 1)):
        cpu_baseline(mol, r, p, n_up, 1)
    rates = []
    for _ in range(args.steps):
        rate, _, _ = cpu_baseline(mol, r, p, n_up, args.cpu_sample)
        rates.append(rate)
    v = statistics.median(rates)
    cores = os.cpu_count()
    sample = f"{args.cpu_sample} of {args.walkers} {mol.name} walkers per step, numpy FP64 oracle port"
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * args.walkers / v, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"{mol.name} all-trans, {args.walkers} walkers, local energy", "n_el": mol.n_el},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


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
    from sparse_wf_gb300.wavefunction import FireWaveFunction, StaticArgs

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
    r_np = r_all[a:b]
    B = len(r_np)
    wf = FireWaveFunction(mol, precision=args.precision, device=dev)
    params = wf.init(0, r_all[:1])
    dp = wf._params(params)
    r_dev = torch.from_numpy(r_np).to(dev)
    static = wf.get_static_input(r_dev).round_with_padding(1.1, mol.n_el, n_up, mol.n_nuc)
    # workspace: the largest chunk within the budget
    if args.chunk > 0:
        wf.chunk_walkers = args.chunk
    else:
        import ctypes as C

        lo, hi = 1, B
        while lo < hi:
            mid = (lo + hi + 1) // 2
            prob = wf._problem(B, static)
            nb = C.c_size_t()
            _lib.load().fire_workspace_size(C.byref(prob), mid, C.byref(nb))
            if nb.value <= args.ws_gb * 1e9:
                lo = mid
            else:
                hi = mid - 1
        wf.chunk_walkers = lo

    def step():
        return wf.local_energy_full(dp, r_dev, static)

    for _ in range(args.warmup):
        eloc, aux = step()
        static = aux["static"]
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(args.steps):
            eloc, aux = step()
        e1.record(stream)
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
    ms = e0.elapsed_time(e1) / args.steps
    if world > 1:
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    total_walkers = args.walkers * world
    value = total_walkers / (ms / 1e3)

    # per-stage device times (CUDA events around every stage / contraction launch) for the roofline
    _lib.profile_enable(True)
    step()
    torch.cuda.synchronize()
    prof = _lib.profile_report()
    _lib.profile_enable(False)
    counts = wf.neighbor_lists(r_dev[: min(B, 64)], static)["counts"]
    pairs = float(np.mean(counts[:, 0] + counts[:, 1]))
    flops = gemm_flops(mol.n_el, mol.n_nuc, pairs) * B
    peaks, peak_kind = measured_peaks()
    g_launches, g_ms = prof.get("gemm", (0, float("nan")))
    achieved = flops / (g_ms / 1e3) / 1e12
    roofline = {"bound": "tensor", "achieved": achieved, "peak": peaks["bf16_tflops"], "unit": "TFLOP/s",
                "frac": achieved / peaks["bf16_tflops"], "traffic": None,
                "kernel": "k_gemm (all dense contractions of one step)", "launches": g_launches,
                "avg_launch_ms": g_ms / max(g_launches, 1), "peak_source": f"bf16 dense, {peak_kind}",
                "flops_per_step": flops}
    stages = {k: {"launches": v[0], "ms": v[1]} for k, v in prof.items() if k != "kernels_launched"}

    # end to end through the public API: pinned host walkers in, E_loc out, every step
    e2e = None
    if not args.no_e2e:
        r_host = torch.from_numpy(r_np).pin_memory()
        e_host = torch.empty(B, dtype=torch.float32).pin_memory()
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        t0 = time.perf_counter()
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        for _ in range(args.steps):
            r_dev.copy_(r_host, non_blocking=True)
            eloc, aux = step()
            e_host.copy_(eloc, non_blocking=True)
        f1.record(stream)
        torch.cuda.synchronize()
        ms_e2e = max(f0.elapsed_time(f1), (time.perf_counter() - t0) * 1e3) / args.steps
        if world > 1:
            t = torch.tensor([ms_e2e], device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms_e2e = float(t.item())
        e2e = {"value": total_walkers / (ms_e2e / 1e3), "unit": UNIT, "h2d_bytes_per_step": int(r_host.numel() * 4),
               "d2h_bytes_per_step": int(e_host.numel() * 4)}

    # CPU baseline + oracle check on the same walkers (rank 0)
    cpu = None
    check = None
    if rank == 0 and not args.no_cpu_baseline:
        rate, e_ref, dt = cpu_baseline(mol, r_np, params, n_up, args.cpu_sample)
        cpu = {"value": rate, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
               "sample": f"{args.cpu_sample} of {B} {mol.name} walkers, numpy FP64 oracle, {dt:.1f} s"}
        got = eloc[: args.cpu_sample].double().cpu().numpy()
        check = {"walkers": args.cpu_sample, "max_abs_err_mHa": float(np.abs(got - e_ref).max() * 1e3),
                 "mean_err_mHa": float(abs(got.mean() - e_ref.mean()) * 1e3), "reference": "FP64 oracle"}

    if rank == 0:
        st = aux["stats"].cpu().numpy()
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32" if args.precision == "fp32" else "bf16/f32",
            "data": "synthetic",
            "config": {"workload": f"{mol.name} all-trans, {args.walkers} walkers per GPU, local energy "
                                   f"(sparse forward Laplacian + Coulomb)", "n_el": mol.n_el, "n_nuc": mol.n_nuc,
                       "walkers_per_gpu": args.walkers, "precision": args.precision,
                       "chunk_walkers": wf.chunk_walkers, "mean_pairs_per_walker": pairs,
                       "cap_pairs": static.n_pairs, "l2": "working set of every step >> L2 (GB-scale planes)",
                       "parallelism": f"walker shards x{world}", "E_mean": float(st[0]), "E_std": float(st[1])},
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "clocks": clk.summary(),
            "gpu_launches": int(prof.get("kernels_launched", (0, 0))[0]) * args.steps,
            "stages_ms": stages, "oracle_check": check,
        }
        print(json.dumps(line))
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
