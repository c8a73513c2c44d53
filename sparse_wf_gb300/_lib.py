"""ctypes binding of ``libfire.so`` (declarations in ``include/fire.h``).

The library is the product path; there is no CPU fallback.  ``load()`` raises when
the shared library is missing or cannot be loaded.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libfire.so"

FIRE_OK = 0
STATUS_WORDS = 8
NO_NEIGHBOUR = 1_000_000
PREC = {"fp32": 0, "mixed": 1, "fp64": 2}
FLAG_PAIR_OVERFLOW = 1
FLAG_NUC_OVERFLOW = 2
FLAG_NONFINITE = 4
FLAG_TRIPLET_OVERFLOW = 8
FLAG_SINGULAR = 16
FLAG_TIMEOUT = 32
FLAG_CHANGED_OVERFLOW = 64
FLAG_REFINE_OVERFLOW = 128
LOW_RANK_MAX_CHANGED = 128  # LR_KMAX: capacity limit of a low-rank step's changed set
TRIPLETS_STATIC_MAX_WORDS = 4 * 1024 * 1024  # FIRE_TRIPLETS_STATIC_MAX_WORDS
ERRORS = {1: "invalid argument", 2: "unsupported size", 3: "workspace too small", 4: "CUDA launch failed"}

# exported entry points, in header order
SYMBOLS = [
    "fire_abi_version", "fire_param_layout", "fire_prepared_size", "fire_workspace_size",
    "fire_prepare_params", "fire_neighbors", "fire_triplets", "fire_logpsi", "fire_local_energy",
    "fire_embedding", "fire_mcmc_block", "fire_potential_energy", "fire_profile_enable", "fire_profile_report",
    "fire_gemm_mixed", "fire_triplets_static", "fire_mcmc_single_block", "fire_mcmc_jump_block",
    "fire_mcmc_cluster_block", "fire_low_rank_workspace_size", "fire_mcmc_low_rank_block", "fire_mcmc_low_rank_jump_block",
    "fire_mcmc_low_rank_cluster_block",
    "fire_ecp_quadrature",
    "fire_ecp_energy",
    "fire_logpsi_grad_workspace_size", "fire_logpsi_grad",
]


class Problem(C.Structure):
    _fields_ = [
        ("n_el", C.c_int32), ("n_up", C.c_int32), ("n_nuc", C.c_int32), ("n_walkers", C.c_int32),
        ("cutoff", C.c_float), ("cutoff_1el", C.c_float), ("cap_pairs", C.c_int32), ("cap_nuc", C.c_int32),
        ("precision", C.c_int32), ("chunk_walkers", C.c_int32), ("refine_cap", C.c_int32),
        ("refine_ratio", C.c_float), ("refine_kappa", C.c_float), ("refine_ks", C.c_float),
        ("refine_kscond", C.c_float),
    ]


class NeighborOut(C.Structure):
    _fields_ = [(name, C.c_void_p) for name in (
        "ct_same", "nb_same", "jac_same", "ct_diff", "nb_diff", "jac_diff", "jac_ctr", "jac_dep", "en_idx",
        "counts")] + [("cap_same", C.c_int32), ("cap_diff", C.c_int32)]


class Ecp(C.Structure):
    _fields_ = [("n_ecp", C.c_int32), ("n_grid", C.c_int32), ("n_l", C.c_int32), ("max_quad", C.c_int32)] + [
        (name, C.c_void_p) for name in ("atom", "grid", "v_loc", "v_nl", "cutoff", "n_quad")]


class ElocDebug(C.Structure):
    _fields_ = [(name, C.c_void_p) for name in
                ("kinetic", "potential", "logdet", "sign_det", "jastrow", "grad", "lap", "refined", "cond")]


_lib = None


def load() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(f"{LIB_PATH.name} is not built; run sparse_wf_gb300.build.build()")
    lib = C.CDLL(str(LIB_PATH))
    P = C.POINTER(Problem)
    vp, i32, u64, f32, sz = C.c_void_p, C.c_int32, C.c_uint64, C.c_float, C.c_size_t
    sig = {
        "fire_abi_version": ([], i32),
        "fire_param_layout": ([P, C.POINTER(C.c_int64)], i32),
        "fire_prepared_size": ([P, C.POINTER(sz)], i32),
        "fire_workspace_size": ([P, i32, C.POINTER(sz)], i32),
        "fire_prepare_params": ([vp, P, vp, C.POINTER(C.c_int64), vp, sz], i32),
        "fire_neighbors": ([vp, P, vp, vp, C.POINTER(NeighborOut), vp], i32),
        "fire_triplets": ([vp, P, vp, i32, vp, vp, vp, vp, vp, sz, vp], i32),
        "fire_logpsi": ([vp, P, vp, vp, vp, vp, vp, vp, vp, sz, vp], i32),
        "fire_local_energy": ([vp, P, vp, vp, vp, vp, vp, vp, vp, vp, C.POINTER(ElocDebug), vp, sz, vp], i32),
        "fire_embedding": ([vp, P, vp, vp, vp, vp, vp, vp, sz, vp], i32),
        "fire_mcmc_block": ([vp, P, vp, vp, vp, vp, vp, i32, f32, u64, u64, vp, vp, vp, vp, vp, sz, vp], i32),
        "fire_mcmc_single_block": ([vp, P, vp, vp, vp, vp, vp, i32, i32, f32, u64, u64, vp, vp, vp, vp, vp, sz, vp],
                                   i32),
        "fire_mcmc_jump_block": ([vp, P, vp, vp, vp, vp, vp, i32, f32, u64, u64, vp, vp, vp, vp, vp, sz, vp], i32),
        "fire_mcmc_cluster_block": ([vp, P, vp, vp, vp, vp, vp, i32, i32, f32, i32, f32, i32, u64, u64, vp, vp, vp, vp,
                                     vp, sz, vp], i32),
        "fire_low_rank_workspace_size": ([P, i32, i32, C.POINTER(sz)], i32),
        "fire_mcmc_low_rank_block": ([vp, P, vp, vp, vp, vp, vp, i32, i32, f32, i32, u64, u64, vp, vp, vp, vp, vp, sz,
                                      vp], i32),
        "fire_mcmc_low_rank_jump_block": ([vp, P, vp, vp, vp, vp, vp, i32, f32, i32, u64, u64, vp, vp, vp, vp, vp,
                                           sz, vp], i32),
        "fire_mcmc_low_rank_cluster_block": ([vp, P, vp, vp, vp, vp, vp, i32, i32, f32, i32, f32, i32, i32, u64, u64,
                                              vp, vp, vp, vp, vp, sz, vp], i32),
        "fire_ecp_quadrature": ([i32, C.POINTER(C.c_double)], i32),
        "fire_ecp_energy": ([vp, P, vp, vp, vp, vp, C.POINTER(Ecp), i32, u64, u64, vp, vp, vp, vp, sz, vp], i32),
        "fire_potential_energy": ([vp, P, vp, vp, vp, vp], i32),
        "fire_profile_enable": ([i32], i32),
        "fire_profile_report": ([C.c_char_p, sz], i32),
        "fire_gemm_mixed": ([vp, i32, i32, i32, vp, vp, vp, vp, sz, vp], i32),
        "fire_triplets_static": ([vp, P, vp, i32, vp, vp, vp, vp, vp], i32),
        "fire_logpsi_grad_workspace_size": ([P, i32, C.POINTER(sz)], i32),
        "fire_logpsi_grad": ([vp, P, vp, vp, vp, vp, vp, vp, vp, sz, vp], i32),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


def check(rc: int, what: str) -> None:
    if rc != FIRE_OK:
        raise RuntimeError(f"{what}: {ERRORS.get(rc, rc)}")


def profile_enable(on: bool) -> None:
    check(load().fire_profile_enable(1 if on else 0), "fire_profile_enable")


def profile_report() -> dict[str, tuple[int, float]]:
    """{stage: (launches, total_ms)} of the calls made while profiling was enabled (waits for them)."""
    buf = C.create_string_buffer(1 << 16)
    check(load().fire_profile_report(buf, len(buf)), "fire_profile_report")
    out = {}
    for line in buf.value.decode().splitlines():
        name, k, ms = line.split()
        out[name] = (int(k), float(ms))
    return out
