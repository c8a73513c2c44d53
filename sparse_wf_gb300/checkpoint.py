"""Checkpoints: this framework's state as one npz file, and the reference's checkpoints (expanded npz or flax msgpack)
read into the parameter slots.

The reference stores a ``TrainingState`` (key, params, electrons, opt_state, width_state, spin_state, step) as a flax
msgpack blob (``TrainingState.serialize``, ``api.py:294-331``; written by ``loggers.py:180-188``) or, expanded, as one
npz per field whose keys are the "/"-joined leaf paths of the pytree (``save_expanded_checkpoint``,
``loggers.py:191-208``; ``tree_to_flat_dict``, ``tree_utils.py:94-108``).

``REFERENCE_LEAVES`` is the default mapping from those leaf paths to the parameter slots.  It is derived from the
reference's module definitions: NamedTuple fields and tuple indices of ``MoonLikeParams`` / ``EmbeddingParams``
(``model/wave_function.py:54-57``, ``model/new_sparse_model.py:134-136, 218-225``), ``setup`` attribute names
(``Orbitals``, ``model/orbitals.py:52-83``; ``Jastrow``, ``model/jastrow.py:204-245``; ``GlobalAttentionJastrow``,
``model/jastrow.py:73-83``), explicit names (``PairwiseFilter(name="beta_ee")``, ``model/new_sparse_model.py:178``)
and flax's automatic ``<Class>_<k>`` names of compact submodules in creation order (``ElecInit`` 190-215,
``ElecNucEdge`` 139-158, ``PairwiseFilter`` ``model/utils.py:393-433``, ``GatedLinearUnit`` 55-62, ``SparseMLP``
``model/sparse_fwd_lap.py:209-225``, ``MLP`` ``model/utils.py:25-52``).  ElecInit's edge module runs under a lifted
``nn.vmap`` of a function that takes the module (``jax_utils.py:108-130``), which leaves its own name in place.
No reference checkpoint or flax install was available to confirm these names against; a caller whose checkpoint
differs passes its own mapping, and every slot's shape is checked either way.
"""
from __future__ import annotations

import os
from typing import Optional

import numpy as np

from .params import ModelDims, param_shapes

_STATE_KEYS = ("electrons", "width", "pmoves", "width_i", "step")


def save(path: str, params: dict, electrons=None, width_state=None, step: Optional[int] = None) -> None:
    """Writes the parameter dict (one array per slot, keys ``param/<slot>``), the walkers, the width scheduler's
    state (``WidthSchedulerState``) and the step into one npz file."""
    out = {f"param/{k}": np.asarray(v) for k, v in params.items()}
    if electrons is not None:
        out["electrons"] = np.asarray(electrons)
    if width_state is not None:
        out["width"] = np.asarray(width_state.width, np.float32)
        out["pmoves"] = np.asarray(width_state.pmoves, np.float32)
        out["width_i"] = np.asarray(width_state.i, np.int64)
    if step is not None:
        out["step"] = np.asarray(step, np.int64)
    np.savez(path, **out)


def load(path: str, dims: ModelDims) -> dict:
    """Reads a file written by ``save``: {"params", "electrons", "width_state", "step"} (absent fields None).  Every
    parameter slot of the model must be present with its shape."""
    from .wavefunction import WidthSchedulerState

    with np.load(path) as f:
        data = {k: f[k] for k in f.files}
    shapes = param_shapes(dims)
    params = {}
    for k, shape in shapes.items():
        key = f"param/{k}"
        if key not in data:
            raise KeyError(f"checkpoint has no parameter {k!r}")
        if tuple(data[key].shape) != tuple(shape):
            raise ValueError(f"parameter {k!r} has shape {data[key].shape}, the model expects {shape}")
        params[k] = data[key]
    ws = None
    if "width" in data:
        ws = WidthSchedulerState(np.float32(data["width"]), tuple(np.float32(x) for x in data["pmoves"]),
                                 int(data["width_i"]))
    return {"params": params, "electrons": data.get("electrons"), "width_state": ws,
            "step": int(data["step"]) if "step" in data else None}


def _scalars(*paths):
    return tuple(paths)


# leaf path of every parameter slot in the reference's MoonLikeParams (see the module docstring); a tuple of paths
# stacks scalars into one slot
_EI = "embedding/elec_init/params/"
_EDGE = _EI + "ElecNucEdge_0/"
REFERENCE_LEAVES = {
    "en_scales": "embedding/dynamic_params_en/filter/scales",
    "en_kernel": "embedding/dynamic_params_en/filter/kernel",
    "en_bias": "embedding/dynamic_params_en/filter/bias",
    "en_nuc_emb": "embedding/dynamic_params_en/nuc_embedding",
    "ei_dir_W": _EDGE + "PairwiseFilter_0/Dense_0/kernel",
    "ei_dir_b": _EDGE + "PairwiseFilter_0/Dense_0/bias",
    "ei_env_W": _EDGE + "PairwiseFilter_0/Dense_1/kernel",
    "ei_gamma_W": _EDGE + "Dense_0/kernel",
    "ei_edge_W": _EDGE + "Dense_1/kernel",
    "ei_ln_scale": _EI + "LayerNorm_0/scale",
    "ei_ln_bias": _EI + "LayerNorm_0/bias",
    "ei_glu_W": _EI + "GatedLinearUnit_0/Dense_0/kernel",
    "ei_dense_W": _EI + "Dense_0/kernel",
    "ei_dense_b": _EI + "Dense_0/bias",
    "ei_out_W": _EI + "Dense_1/kernel",
    "ei_out_b": _EI + "Dense_1/bias",
    **{f"ee{t}_{k}": f"embedding/edge_{t}/params/{v}" for t in ("same", "diff") for k, v in (
        ("scale", "beta_ee/scale"), ("kernel", "beta_ee/kernel"), ("bias", "beta_ee/bias"),
        ("dir_W", "beta_ee/Dense_0/kernel"), ("dir_b", "beta_ee/Dense_0/bias"), ("env_W", "beta_ee/Dense_1/kernel"),
        ("gamma_W", "Dense_0/kernel"), ("edge_W", "Dense_1/kernel"), ("edge_b", "Dense_1/bias"))},
    "upd1_W": "embedding/updates/0/params/Linear_0/kernel",
    "upd1_b": "embedding/updates/0/params/Linear_0/bias",
    "upd2_W": "embedding/updates/0/params/Linear_1/kernel",
    "upd2_b": "embedding/updates/0/params/Linear_1/bias",
    "scales": _scalars("embedding/scales/0", "embedding/scales/1"),
    "cutoff_param": _scalars("embedding/cutoff_param"),
    "orb_up_W": "to_orbitals/params/to_orbitals_up/kernel",
    "orb_up_b": "to_orbitals/params/to_orbitals_up/bias",
    "orb_dn_W": "to_orbitals/params/to_orbitals_dn/kernel",
    "orb_dn_b": "to_orbitals/params/to_orbitals_dn/bias",
    "env_up_sigma": "to_orbitals/params/env_up/sigma",
    "env_up_pi": "to_orbitals/params/env_up/pi",
    "env_dn_sigma": "to_orbitals/params/env_dn/sigma",
    "env_dn_pi": "to_orbitals/params/env_dn/pi",
    "cusp": _scalars(*(f"jastrow/params/pairwise_cusps/{k}"
                       for k in ("alpha_same", "alpha_diff", "factor_same", "factor_diff"))),
    "jmlp1_W": "jastrow/params/mlp/Linear_0/kernel",
    "jmlp1_b": "jastrow/params/mlp/Linear_0/bias",
    "jmlp2_W": "jastrow/params/mlp/Linear_1/kernel",
    "jmlp2_b": "jastrow/params/mlp/Linear_1/bias",
    "jmlp3_W": "jastrow/params/mlp/Linear_2/kernel",
    "jmlp3_b": "jastrow/params/mlp/Linear_2/bias",
    "mlp_scale": "jastrow/params/mlp_scale",
    "log_bias": _scalars("jastrow/params/log_bias"),
    "att_keys": "jastrow/params/att/register_keys",
    "att_Q_W": "jastrow/params/att/Q_W/kernel",
    "att_Q_b": "jastrow/params/att/Q_W/bias",
    "att_V_W": "jastrow/params/att/V_W/kernel",
    "att_V_b": "jastrow/params/att/V_W/bias",
    "att_out1_W": "jastrow/params/att/out/Dense_0/kernel",
    "att_out1_b": "jastrow/params/att/out/Dense_0/bias",
    "att_out2_W": "jastrow/params/att/out/Dense_1/kernel",
    "att_out2_b": "jastrow/params/att/out/Dense_1/bias",
    "att_out3_W": "jastrow/params/att/out/Dense_2/kernel",
    "att_out3_b": "jastrow/params/att/out/Dense_2/bias",
    "att_scale": "jastrow/params/att/scale",
    "att_bias": "jastrow/params/att/bias",
}


# ------------------------------------------------------------------------ flax msgpack (no dependency)
# flax.serialization writes the state dict with msgpack (the published MessagePack format) and three extension types:
# 1 = ndarray, payload msgpack (shape, dtype name, C-order bytes); 2 = complex scalar; 3 = numpy scalar, payload
# msgpack (dtype name, bytes).  The reader below decodes that subset of MessagePack.
class _Unpacker:
    def __init__(self, data: bytes):
        self.d = memoryview(data)
        self.i = 0

    def _take(self, n):
        b = self.d[self.i:self.i + n]
        if len(b) != n:
            raise ValueError("truncated msgpack data")
        self.i += n
        return bytes(b)

    def _uint(self, n):
        return int.from_bytes(self._take(n), "big")

    def _ext(self, code, payload):
        if code == 1:
            shape, dtype, buf = _Unpacker(payload).value()
            return np.frombuffer(buf, dtype=np.dtype(dtype)).reshape(shape).copy()
        if code == 3:
            dtype, buf = _Unpacker(payload).value()
            return np.frombuffer(buf, dtype=np.dtype(dtype))[0]
        if code == 2:
            re, im = _Unpacker(payload).value()
            return complex(re, im)
        raise ValueError(f"unknown msgpack extension type {code}")

    def value(self):
        t = self._uint(1)
        if t <= 0x7F:
            return t
        if t >= 0xE0:
            return t - 0x100
        if 0x80 <= t <= 0x8F:
            return self._map(t & 0x0F)
        if 0x90 <= t <= 0x9F:
            return [self.value() for _ in range(t & 0x0F)]
        if 0xA0 <= t <= 0xBF:
            return self._take(t & 0x1F).decode()
        simple = {0xC0: None, 0xC2: False, 0xC3: True}
        if t in simple:
            return simple[t]
        if t in (0xC4, 0xC5, 0xC6):
            return self._take(self._uint({0xC4: 1, 0xC5: 2, 0xC6: 4}[t]))
        if t in (0xC7, 0xC8, 0xC9):
            n = self._uint({0xC7: 1, 0xC8: 2, 0xC9: 4}[t])
            code = int.from_bytes(self._take(1), "big", signed=True)
            return self._ext(code, self._take(n))
        if t == 0xCA:
            return float(np.frombuffer(self._take(4), ">f4")[0])
        if t == 0xCB:
            return float(np.frombuffer(self._take(8), ">f8")[0])
        if 0xCC <= t <= 0xCF:
            return self._uint(1 << (t - 0xCC))
        if 0xD0 <= t <= 0xD3:
            return int.from_bytes(self._take(1 << (t - 0xD0)), "big", signed=True)
        if 0xD4 <= t <= 0xD8:
            code = int.from_bytes(self._take(1), "big", signed=True)
            return self._ext(code, self._take(1 << (t - 0xD4)))
        if t in (0xD9, 0xDA, 0xDB):
            return self._take(self._uint({0xD9: 1, 0xDA: 2, 0xDB: 4}[t])).decode()
        if t in (0xDC, 0xDD):
            return [self.value() for _ in range(self._uint(2 if t == 0xDC else 4))]
        if t in (0xDE, 0xDF):
            return self._map(self._uint(2 if t == 0xDE else 4))
        raise ValueError(f"unsupported msgpack type byte 0x{t:02x}")

    def _map(self, n):
        out = {}
        for _ in range(n):
            k = self.value()
            out[k] = self.value()
        return out


def _flatten(tree, prefix=""):
    out = {}
    for k, v in tree.items():
        path = f"{prefix}{k}"
        if isinstance(v, dict):
            out.update(_flatten(v, path + "/"))
        else:
            out[path] = v
    return out


def read_reference_msgpack(path: str) -> dict:
    """The reference's msgpack checkpoint (``chkpt<step>.msgpk``) as {"/"-joined leaf path: array}, the paths of the
    whole TrainingState ("params/embedding/...", "electrons", "step", ...)."""
    with open(path, "rb") as f:
        state = _Unpacker(f.read()).value()
    if not isinstance(state, dict):
        raise ValueError("a flax checkpoint holds a state dict at its top level")
    return _flatten(state)


def _gather(leaves: dict, src, shape):
    if isinstance(src, tuple) and len(src) == 2 and callable(src[1]):
        path, fn = src
    else:
        path, fn = src, None
    if isinstance(path, tuple):  # scalars stacked into one slot
        missing = [q for q in path if q not in leaves]
        if missing:
            raise KeyError(f"the checkpoint has no leaf {missing[0]!r}")
        a = np.array([np.asarray(leaves[q]).reshape(()) for q in path])
        used = set(path)
    else:
        if path not in leaves:
            raise KeyError(f"the checkpoint has no leaf {path!r}")
        a = np.asarray(leaves[path])
        used = {path}
    a = fn(a) if fn is not None else a
    if a.shape != tuple(shape) and a.size == int(np.prod(shape)) and a.ndim == 0:
        a = a.reshape(shape)
    return a, used


def params_from_leaves(leaves: dict, dims: ModelDims, mapping: Optional[dict] = None) -> dict:
    """Parameter slots from a {leaf path: array} dict of MoonLikeParams leaves (default mapping REFERENCE_LEAVES).
    Every slot of the model must be mapped and match its shape; unmapped leaves are reported."""
    mapping = REFERENCE_LEAVES if mapping is None else mapping
    shapes = param_shapes(dims)
    missing = [k for k in shapes if k not in mapping]
    if missing:
        raise KeyError(f"no mapping for the parameter slots {missing}")
    params, used = {}, set()
    for slot, src in mapping.items():
        if slot not in shapes:
            raise KeyError(f"{slot!r} is not a parameter slot of the model")
        a, u = _gather(leaves, src, shapes[slot])
        if tuple(a.shape) != tuple(shapes[slot]):
            raise ValueError(f"{src!r} gives shape {a.shape} for {slot!r}, the model expects {shapes[slot]}")
        params[slot] = a.astype(np.float64)
        used |= u
    return {"params": params, "unused_leaves": sorted(set(leaves) - used)}


def load_reference_msgpack(path: str, dims: ModelDims, mapping: Optional[dict] = None) -> dict:
    """Parameters and walkers of the reference's msgpack checkpoint: {"params", "electrons", "step",
    "unused_leaves"} (the params subtree's leaves not mapped to a slot)."""
    leaves = read_reference_msgpack(path)
    sub = {k[len("params/"):]: v for k, v in leaves.items() if k.startswith("params/")}
    out = params_from_leaves(sub, dims, mapping)
    out["electrons"] = leaves.get("electrons")
    out["step"] = int(np.asarray(leaves["step"])) if "step" in leaves else None
    return out


def load_reference_params(directory: str, dims: ModelDims, mapping: Optional[dict] = None) -> dict:
    """Parameters from the reference's expanded checkpoint (``<directory>/params.npz``, keys the "/"-joined leaf paths
    of ``MoonLikeParams``).  mapping: {slot: leaf path, a tuple of scalar leaf paths, or (leaf path, transform)} with
    transform a callable applied to the array (a transpose or reshape where the reference's layout differs); default
    REFERENCE_LEAVES.  Every slot of the model must be mapped and match its shape; unmapped leaves are reported."""
    with np.load(os.path.join(directory, "params.npz")) as f:
        leaves = {k: f[k] for k in f.files}
    return params_from_leaves(leaves, dims, mapping)
