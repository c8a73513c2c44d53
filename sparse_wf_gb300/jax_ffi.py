"""jax.ffi binding of the hot path: the reference's jitted local-energy and Metropolis calls as XLA custom calls.

The reference evaluates ``local_energy(key, params, electrons, static)`` per walker under ``jax.vmap``, chunked by
``batched_energy_fn`` (``update.py:95-100``) inside ``jax.pmap`` (``update.py:221-222``), and its Metropolis step
``MCStep`` (``mcmc.py:329-344``) the same way.  ``local_energy`` and ``mcmc_block`` below are one XLA custom call
each over the whole walker batch, served by the handlers of ``xla/fire_xla.cc`` (``FireLocalEnergy``,
``FireMcmcBlock``) on top of ``libfire.so``; ``logpsi_grad`` (``FireLogpsiGrad``) gives the per-walker parameter
gradient that the dense SPRING preconditioner contracts (``preconditioner.py:190-191``); the library's workspace comes from XLA's scratch allocator.

Parameters go in as the prepared buffer of ``fire_prepare_params`` (``DeviceParams.prepared`` as a uint8 array).
The status words come back as an output: a set flag in ``status[0]`` means the capacities in ``static`` were too
small; grow them from ``status[1:4]`` and repeat the call, as the reference's StaticScheduler grows its static sizes
(``static_args.py:62-84``).

jax is imported on first use; ``available()`` says whether jax and the compiled handler library are present.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

XLA_LIB = Path(__file__).resolve().parent / "libfire_xla.so"
_registered = False


def available() -> bool:
    """True when jax imports and the handler library has been built (``build.build_xla``)."""
    try:
        import jax  # noqa: F401
    except ImportError:
        return False
    return XLA_LIB.exists()


def _register():
    global _registered
    if _registered:
        return
    import jax

    if not XLA_LIB.exists():
        raise RuntimeError(f"{XLA_LIB.name} is not built; run sparse_wf_gb300.build.build_xla() where jax is installed")
    lib = ctypes.cdll.LoadLibrary(str(XLA_LIB))
    jax.ffi.register_ffi_target("fire_local_energy", jax.ffi.pycapsule(lib.FireLocalEnergy), platform="CUDA")
    jax.ffi.register_ffi_target("fire_mcmc_block", jax.ffi.pycapsule(lib.FireMcmcBlock), platform="CUDA")
    jax.ffi.register_ffi_target("fire_logpsi_grad", jax.ffi.pycapsule(lib.FireLogpsiGrad), platform="CUDA")
    _registered = True


def _attrs(static, n_up, precision, cutoff, cutoff_1el, chunk):
    return dict(n_up=np.int32(n_up), cutoff=np.float32(cutoff), cutoff_1el=np.float32(cutoff_1el),
                cap_pairs=np.int32(static.n_pairs_same + static.n_pairs_diff),
                cap_nuc=np.int32(max(1, static.n_neighbours_en)), precision=np.int32(precision),
                chunk=np.int32(chunk))


def local_energy(prepared, R, Z, electrons, static, n_up, precision=1, cutoff=5.0, cutoff_1el=20.0, chunk=0):
    """Batch local energy (``hamiltonian.py:69-81`` over ``update.py:95-100``): electrons [B, n, 3] float32 ->
    (e_loc [B], logpsi [B], sign [B], (mean, std) float64 [2], status [8] int32).  The float64 statistics need
    ``jax_enable_x64``."""
    import jax
    import jax.numpy as jnp

    _register()
    B = electrons.shape[0]
    out = (jax.ShapeDtypeStruct((B,), jnp.float32),) * 3 + (
        jax.ShapeDtypeStruct((2,), jnp.float64), jax.ShapeDtypeStruct((8,), jnp.int32))
    logpsi, sign, e_loc, stats, status = jax.ffi.ffi_call("fire_local_energy", out)(
        R, Z, prepared, electrons, **_attrs(static, n_up, precision, cutoff, cutoff_1el, chunk))
    return e_loc, logpsi, sign, stats, status


def mcmc_block(prepared, R, Z, electrons, logpsi, static, n_up, steps, width, seed, counter=0, precision=1,
               cutoff=5.0, cutoff_1el=20.0, chunk=0):
    """All-electron Metropolis block (``mcmc.py:38-97``): (electrons, logpsi) -> (electrons', logpsi',
    n_accept [B], static_max [4], status [8])."""
    import jax
    import jax.numpy as jnp

    _register()
    B = electrons.shape[0]
    out = (jax.ShapeDtypeStruct(electrons.shape, jnp.float32), jax.ShapeDtypeStruct((B,), jnp.float32),
           jax.ShapeDtypeStruct((B,), jnp.int32), jax.ShapeDtypeStruct((4,), jnp.int32),
           jax.ShapeDtypeStruct((8,), jnp.int32))
    return jax.ffi.ffi_call("fire_mcmc_block", out)(
        R, Z, prepared, electrons, logpsi, steps=np.int32(steps), width=np.float32(width), seed=np.int64(seed),
        counter=np.int64(counter), **_attrs(static, n_up, precision, cutoff, cutoff_1el, chunk))


def logpsi_grad(prepared, R, electrons, static, n_up, n_params, cutoff=5.0, cutoff_1el=20.0, chunk=0):
    """Per-walker gradient of log|psi| with respect to every parameter (``jac_fn`` of the dense SPRING
    preconditioner, ``preconditioner.py:190-191``, as rows): electrons [B, n, 3] float32 -> (grad [B, n_params] in
    the blob layout of ``fire_param_layout``, logpsi [B], sign [B], status [8]).  chunk: walkers per internal pass
    (0: the whole batch in one workspace)."""
    import jax
    import jax.numpy as jnp

    _register()
    B = electrons.shape[0]
    out = (jax.ShapeDtypeStruct((B, n_params), jnp.float32), jax.ShapeDtypeStruct((B,), jnp.float32),
           jax.ShapeDtypeStruct((B,), jnp.float32), jax.ShapeDtypeStruct((8,), jnp.int32))
    attrs = _attrs(static, n_up, 0, cutoff, cutoff_1el, chunk)
    del attrs["precision"]
    return jax.ffi.ffi_call("fire_logpsi_grad", out)(R, prepared, electrons, **attrs)
