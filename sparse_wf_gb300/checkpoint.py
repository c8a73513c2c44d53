"""Checkpoints: this framework's state as one npz file, and the reference's expanded checkpoints read through an
explicit name mapping.

The reference stores a ``TrainingState`` (key, params, electrons, opt_state, width_state, spin_state, step) as a flax
msgpack blob (``api.py:285-331``) or, expanded, as one npz per field whose keys are the "/"-joined leaf paths of the
pytree (``save_expanded_checkpoint``, ``loggers.py:191-208``; ``tree_to_flat_dict``, ``tree_utils.py:94-108``).
Those leaf paths carry the names flax gives to modules (including the ones inside lifted transforms), which cannot be
checked here without flax or a real checkpoint; ``load_reference_params`` therefore takes the mapping from leaf paths
to parameter slots from the caller and checks every shape against the model's, instead of guessing names.
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


def load_reference_params(directory: str, dims: ModelDims, mapping: dict) -> dict:
    """Parameters from the reference's expanded checkpoint (``<directory>/params.npz``, keys the "/"-joined leaf paths
    of ``MoonLikeParams``).  mapping: {slot: leaf path, or (leaf path, transform)} with transform a callable applied
    to the array (a transpose or reshape where the reference's layout differs).  Every slot of the model must be
    mapped and match its shape; unmapped leaves are reported."""
    with np.load(os.path.join(directory, "params.npz")) as f:
        leaves = {k: f[k] for k in f.files}
    shapes = param_shapes(dims)
    missing = [k for k in shapes if k not in mapping]
    if missing:
        raise KeyError(f"no mapping for the parameter slots {missing}")
    params, used = {}, set()
    for slot, src in mapping.items():
        if slot not in shapes:
            raise KeyError(f"{slot!r} is not a parameter slot of the model")
        path, fn = (src, None) if isinstance(src, str) else src
        if path not in leaves:
            raise KeyError(f"the checkpoint has no leaf {path!r} (mapped to {slot!r})")
        a = np.asarray(leaves[path])
        a = fn(a) if fn is not None else a
        if tuple(a.shape) != tuple(shapes[slot]):
            raise ValueError(f"leaf {path!r} gives shape {a.shape} for {slot!r}, the model expects {shapes[slot]}")
        params[slot] = a.astype(np.float64)
        used.add(path)
    return {"params": params, "unused_leaves": sorted(set(leaves) - used)}
