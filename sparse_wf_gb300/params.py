"""FiRE parameters: the reference's parameter tree, its initialisers, and the flat blob.

The parameter tree mirrors ``MoonLikeParams`` (``src/sparse_wf/model/wave_function.py:54-57``)
for the ``new_sparse`` embedding (``model/new_sparse_model.py:218-225, 354-397``),
the spin-unrestricted ``Orbitals`` with ``EfficientIsotropicEnvelopes``
(``model/orbitals.py:52-83``, ``model/envelopes.py:55-82``) and the ``Jastrow``
with psiformer cusps, MLP/log Jastrow and global attention
(``model/jastrow.py:189-246``).  The architecture is ``config/default.yaml``'s
model section (feature_dim 256, 4 determinants, pair widths (16, 8), 32 e-n
envelopes, 8 orbital envelopes, Jastrow width 256 / depth 2, 16 attention heads
of dimension 16) with the e-e cutoff and the 1-electron cutoff as arguments.

The device code takes the parameters as ONE float32 blob plus an int64 table of
element offsets, one per slot of ``PARAM_SLOTS`` (same order as
``enum fire_param_slot`` in ``include/fire.h``).  Every slot starts on a
64-element (256-byte) boundary.

The random initialisers restate the reference's distributions with numpy's
PCG64 (jax.random cannot be reproduced bit-for-bit without jax):

* flax ``Dense``/``Linear`` kernels: lecun normal = normal truncated to [-2, 2]
  with std sqrt(1/fan_in)/0.8796; biases zero (orbital biases: truncated normal, std 0.01);
* the reference's own ``lecun_normal`` (``model/utils.py:339-342``): standard normal
  truncated to [-1, 1] times 1/sqrt(shape[0]) -- fan-in is the FIRST axis, which for the
  per-nucleus filter kernel is n_nuc (``new_sparse_model.py:393``);
* ``scale_initializer`` (``model/utils.py:378-383``) with the e-e cutoff for BOTH the
  e-e and the e-n filters (``new_sparse_model.py:392``);
* ``envelope_sigma_initializer`` (``model/envelopes.py:28-32``);
* Jastrow scales and cusp factors are zero, ``log_bias`` and attention ``bias`` one.
"""
from __future__ import annotations

import dataclasses
from typing import Callable

import numpy as np
from scipy.special import ndtr, ndtri

FEATURE_DIM = 256
N_DET = 4
FILTER_DIMS = (16, 8)
N_ENV_EN = 32
N_ENV_ORB = 8
JAS_WIDTH = 256
ATT_HEADS = 16
ATT_DIM = 16
SLOT_ALIGN = 64


@dataclasses.dataclass(frozen=True)
class ModelDims:
    n_el: int
    n_up: int
    n_nuc: int
    cutoff: float = 5.0
    cutoff_1el: float = 20.0

    @property
    def n_dn(self) -> int:
        return self.n_el - self.n_up

    @property
    def n_orb_cols(self) -> int:
        return N_DET * self.n_el


def _slots(d: ModelDims) -> list[tuple[str, tuple[int, ...]]]:
    F, N, n, D = FEATURE_DIM, d.n_nuc, d.n_el, N_DET
    f0, f1 = FILTER_DIMS
    s = [
        # embedding: nucleus-dependent e-n filter params (new_sparse_model.py:382-397)
        ("en_scales", (N, N_ENV_EN)),
        ("en_kernel", (N, 4, f0)),
        ("en_bias", (N, f0)),
        ("en_nuc_emb", (N, F)),
        # ElecInit (new_sparse_model.py:190-215) incl. ElecNucEdge (139-158)
        ("ei_dir_W", (f0, f1)),
        ("ei_dir_b", (f1,)),
        ("ei_env_W", (N_ENV_EN, f1)),
        ("ei_gamma_W", (f1, F)),
        ("ei_edge_W", (4, F)),
        ("ei_ln_scale", (F,)),
        ("ei_ln_bias", (F,)),
        ("ei_glu_W", (F, 2 * F)),
        ("ei_dense_W", (F, F)),
        ("ei_dense_b", (F,)),
        ("ei_out_W", (F, 5 * F)),
        ("ei_out_b", (5 * F,)),
    ]
    for tag in ("same", "diff"):
        # ElecElecEdges (new_sparse_model.py:161-187) with its own PairwiseFilter (utils.py:393-433)
        s += [
            (f"ee{tag}_scale", (f0,)),
            (f"ee{tag}_kernel", (4, f0)),
            (f"ee{tag}_bias", (f0,)),
            (f"ee{tag}_dir_W", (f0, f1)),
            (f"ee{tag}_dir_b", (f1,)),
            (f"ee{tag}_env_W", (f0, f1)),
            (f"ee{tag}_gamma_W", (f1, F)),
            (f"ee{tag}_edge_W", (4, F)),
            (f"ee{tag}_edge_b", (F,)),
        ]
    s += [
        ("upd1_W", (F, F)),
        ("upd1_b", (F,)),
        ("upd2_W", (F, F)),
        ("upd2_b", (F,)),
        ("scales", (2,)),
        ("cutoff_param", (1,)),
        # orbitals (orbitals.py:52-83)
        ("orb_up_W", (F, D * n)),
        ("orb_up_b", (D * n,)),
        ("orb_dn_W", (F, D * n)),
        ("orb_dn_b", (D * n,)),
        ("env_up_sigma", (N, D, N_ENV_ORB)),
        ("env_up_pi", (N, D, N_ENV_ORB, n)),
        ("env_dn_sigma", (N, D, N_ENV_ORB)),
        ("env_dn_pi", (N, D, N_ENV_ORB, n)),
        # Jastrow (jastrow.py:48-64, 67-155, 189-246)
        ("cusp", (4,)),  # alpha_same, alpha_diff, factor_same, factor_diff
        ("jmlp1_W", (F, JAS_WIDTH)),
        ("jmlp1_b", (JAS_WIDTH,)),
        ("jmlp2_W", (JAS_WIDTH, JAS_WIDTH)),
        ("jmlp2_b", (JAS_WIDTH,)),
        ("jmlp3_W", (JAS_WIDTH, 2)),
        ("jmlp3_b", (2,)),
        ("mlp_scale", (2,)),
        ("log_bias", (1,)),
        ("att_keys", (ATT_HEADS, ATT_DIM)),
        ("att_Q_W", (F, ATT_HEADS * ATT_DIM)),
        ("att_Q_b", (ATT_HEADS * ATT_DIM,)),
        ("att_V_W", (F, ATT_HEADS * ATT_DIM)),
        ("att_V_b", (ATT_HEADS * ATT_DIM,)),
        ("att_out1_W", (2 * ATT_HEADS * ATT_DIM, JAS_WIDTH)),
        ("att_out1_b", (JAS_WIDTH,)),
        ("att_out2_W", (JAS_WIDTH, JAS_WIDTH)),
        ("att_out2_b", (JAS_WIDTH,)),
        ("att_out3_W", (JAS_WIDTH, 2)),
        ("att_out3_b", (2,)),
        ("att_scale", (2,)),
        ("att_bias", (1,)),
    ]
    return s


PARAM_SLOT_NAMES = [name for name, _ in _slots(ModelDims(2, 1, 1))]


def param_shapes(d: ModelDims) -> dict[str, tuple[int, ...]]:
    return dict(_slots(d))


# ----------------------------------------------------------------------------- initialisers
def _trunc_std_normal(rng, lo, hi, shape):
    u = rng.uniform(ndtr(lo), ndtr(hi), size=shape)
    return ndtri(u)


def _flax_lecun(rng, shape):
    fan_in = shape[0]
    std = np.sqrt(1.0 / fan_in) / 0.87962566103423978
    return _trunc_std_normal(rng, -2.0, 2.0, shape) * std


def _ref_lecun(rng, shape):
    return _trunc_std_normal(rng, -1.0, 1.0, shape) / np.sqrt(shape[0])


def _scale_init(rng, cutoff, shape):
    L = min(20.0, 0.75 * cutoff)
    base = np.linspace(0.5 * L, L, shape[-1])
    return base * (1.0 + 0.1 * rng.standard_normal(shape))


def _env_sigma_init(rng, shape):
    scale = np.geomspace(1.0, 5.0, shape[-1]) * _trunc_std_normal(rng, 0.8, 1.2, shape)
    return np.log(np.expm1(scale))


def init_params(dims: ModelDims, seed: int = 0) -> dict[str, np.ndarray]:
    """Random-init parameters with the reference's shapes and distributions.

    The two ``normalize`` scales are left at 1.0: the reference fixes them at init
    as 1/std of the embedding on an init walker (``new_sparse_model.py:378-379``);
    ``FireWaveFunction.init`` computes them on the device.
    """
    rng = np.random.default_rng(seed)
    shp = param_shapes(dims)
    p: dict[str, np.ndarray] = {}

    def put(name, fn: Callable):
        p[name] = np.asarray(fn(shp[name]), np.float64)

    put("en_scales", lambda s: _scale_init(rng, dims.cutoff, s))
    put("en_kernel", lambda s: _ref_lecun(rng, s))
    put("en_bias", lambda s: rng.standard_normal(s) * 2.0)
    put("en_nuc_emb", lambda s: rng.standard_normal(s))
    put("ei_dir_W", lambda s: _flax_lecun(rng, s))
    put("ei_dir_b", np.zeros)
    put("ei_env_W", lambda s: _flax_lecun(rng, s))
    put("ei_gamma_W", lambda s: _flax_lecun(rng, s))
    put("ei_edge_W", lambda s: _flax_lecun(rng, s))
    put("ei_ln_scale", np.ones)
    put("ei_ln_bias", np.zeros)
    put("ei_glu_W", lambda s: _flax_lecun(rng, s))
    put("ei_dense_W", lambda s: _flax_lecun(rng, s))
    put("ei_dense_b", np.zeros)
    put("ei_out_W", lambda s: _flax_lecun(rng, s))
    put("ei_out_b", np.zeros)
    for tag in ("same", "diff"):
        put(f"ee{tag}_scale", lambda s: _scale_init(rng, dims.cutoff, s))
        put(f"ee{tag}_kernel", lambda s: _ref_lecun(rng, s))
        put(f"ee{tag}_bias", lambda s: rng.standard_normal(s))
        put(f"ee{tag}_dir_W", lambda s: _flax_lecun(rng, s))
        put(f"ee{tag}_dir_b", np.zeros)
        put(f"ee{tag}_env_W", lambda s: _flax_lecun(rng, s))
        put(f"ee{tag}_gamma_W", lambda s: _flax_lecun(rng, s))
        put(f"ee{tag}_edge_W", lambda s: _flax_lecun(rng, s))
        put(f"ee{tag}_edge_b", np.zeros)
    for k in (1, 2):
        put(f"upd{k}_W", lambda s: _flax_lecun(rng, s))
        put(f"upd{k}_b", np.zeros)
    put("scales", np.ones)
    put("cutoff_param", lambda s: np.full(s, 10.0))
    for spin in ("up", "dn"):
        put(f"orb_{spin}_W", lambda s: _flax_lecun(rng, s))
        put(f"orb_{spin}_b", lambda s: _trunc_std_normal(rng, -2.0, 2.0, s) * 0.01)
    for spin in ("up", "dn"):
        put(f"env_{spin}_sigma", lambda s: _env_sigma_init(rng, s))
        put(f"env_{spin}_pi", lambda s: rng.standard_normal(s) / np.sqrt(N_ENV_ORB))
    put("cusp", lambda s: np.array([1.0, 1.0, 0.0, 0.0]))
    put("jmlp1_W", lambda s: _flax_lecun(rng, s))
    put("jmlp1_b", np.zeros)
    put("jmlp2_W", lambda s: _flax_lecun(rng, s))
    put("jmlp2_b", np.zeros)
    put("jmlp3_W", lambda s: _flax_lecun(rng, s))
    put("jmlp3_b", np.zeros)
    put("mlp_scale", np.zeros)
    put("log_bias", np.ones)
    put("att_keys", lambda s: rng.standard_normal(s))
    for k in ("Q", "V"):
        put(f"att_{k}_W", lambda s: _flax_lecun(rng, s))
        put(f"att_{k}_b", np.zeros)
    for k in (1, 2, 3):
        put(f"att_out{k}_W", lambda s: _flax_lecun(rng, s))
        put(f"att_out{k}_b", np.zeros)
    put("att_scale", np.zeros)
    put("att_bias", np.ones)
    return p


def activate_jastrow(p: dict[str, np.ndarray]) -> dict[str, np.ndarray]:
    """The reference tests' convention (``tests/utils.py:73-78``): every Jastrow leaf whose
    name contains "scale" is set to one, so the Jastrow is not identically constant; the
    cusp factors are set to the psiformer values (-1/4 same spin, -1/2 opposite spin)."""
    q = dict(p)
    q["mlp_scale"] = np.ones(2)
    q["att_scale"] = np.ones(2)
    q["cusp"] = np.array([1.0, 1.0, -0.25, -0.5])
    return q


# ----------------------------------------------------------------------------- blob
def param_offsets(dims: ModelDims) -> np.ndarray:
    offs = []
    o = 0
    for _, shape in _slots(dims):
        offs.append(o)
        size = int(np.prod(shape))
        o += (size + SLOT_ALIGN - 1) // SLOT_ALIGN * SLOT_ALIGN
    offs.append(o)  # total length
    return np.array(offs, np.int64)


def pack_params(dims: ModelDims, p: dict[str, np.ndarray], dtype=np.float32) -> tuple[np.ndarray, np.ndarray]:
    """(blob, offsets): offsets has one entry per slot plus the total length."""
    offs = param_offsets(dims)
    blob = np.zeros(int(offs[-1]), dtype)
    for k, (name, shape) in enumerate(_slots(dims)):
        v = np.asarray(p[name])
        if v.shape != shape:
            raise ValueError(f"param {name}: shape {v.shape} != {shape}")
        blob[offs[k] : offs[k] + v.size] = v.reshape(-1)
    return blob, offs


def unpack_params(dims: ModelDims, blob: np.ndarray, offs: np.ndarray) -> dict[str, np.ndarray]:
    out = {}
    for k, (name, shape) in enumerate(_slots(dims)):
        size = int(np.prod(shape))
        out[name] = np.asarray(blob[offs[k] : offs[k] + size], np.float64).reshape(shape)
    return out


def cast_params(p: dict[str, np.ndarray], dtype) -> dict[str, np.ndarray]:
    return {k: np.asarray(v, dtype) for k, v in p.items()}
