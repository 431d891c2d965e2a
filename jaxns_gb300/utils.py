"""Result utilities with jaxns's names: sample_evidence, save_results / load_results.

sample_evidence (utils.py:433-484) runs on the device (gbns_sample_evidence).  The JSON
format of save_results / load_results is the reference's (utils.py:588-640 with
internals/namedtuple_utils.py:34-103): a NamedTuple is {"type": "__namedtuple__",
"__class__": module.Class, "__data__": {...}} and an array is {"type": "__jax_ndarray__" or
"__ndarray__", "__dtype__", "__data__": base64 of the raw bytes, "__shape__"}.  Results are
written under the reference's class path, so jaxns.utils.load_results reads them, and files
that jaxns wrote load here.
"""
from __future__ import annotations

import base64
import ctypes
import json
import warnings
from typing import Any

import numpy as np
import torch

from . import _ffi
from .public import NestedSamplerResults, SampleCollection, TerminationCondition

# class path written for each NamedTuple of this package, and the classes a file may name
_REFERENCE_PATHS = {
    NestedSamplerResults: "jaxns.nested_samplers.common.types.NestedSamplerResults",
    TerminationCondition: "jaxns.nested_samplers.common.types.TerminationCondition",
    SampleCollection: "jaxns.nested_samplers.common.types.SampleCollection",
}
_BY_NAME = {cls.__name__: cls for cls in _REFERENCE_PATHS}


def sample_evidence(key, num_live_points_per_sample, log_L_samples, S: int = 100) -> torch.Tensor:
    """S samples of log Z with the shrinkage simulated (T_i ~ Beta(n_i, 1)); on the device,
    FP64.  key: a jax-layout key (2 x uint32)."""
    n = torch.as_tensor(num_live_points_per_sample)
    L = torch.as_tensor(log_L_samples)
    dev = L.device if L.is_cuda else torch.device("cuda")
    n = n.to(device=dev, dtype=torch.int32).contiguous()
    L = L.to(device=dev, dtype=torch.float64).contiguous()
    if n.shape != L.shape or n.dim() != 1:
        raise ValueError("num_live_points_per_sample and log_L_samples must be 1-D of equal length")
    k = torch.tensor(np.asarray(key, np.uint32).view(np.int32), device=dev)
    out = torch.empty(int(S), dtype=torch.float64, device=dev)
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    _ffi.call("gbns_sample_evidence", p(k), p(n), p(L), ctypes.c_longlong(L.numel()), ctypes.c_int(int(S)), p(out),
              ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream))
    return out


def _is_namedtuple(obj) -> bool:
    return isinstance(obj, tuple) and hasattr(obj, "_asdict") and hasattr(obj, "_fields")


def _serialise(obj):
    if _is_namedtuple(obj):
        path = _REFERENCE_PATHS.get(type(obj), f"{type(obj).__module__}.{type(obj).__name__}")
        return {"type": "__namedtuple__", "__class__": path,
                "__data__": {k: _serialise(v) for k, v in obj._asdict().items()}}
    if isinstance(obj, torch.Tensor):
        obj = obj.detach().cpu().numpy()
    if isinstance(obj, np.ndarray):
        obj = np.ascontiguousarray(obj)
        return {"type": "__jax_ndarray__", "__dtype__": str(obj.dtype),
                "__data__": base64.b64encode(obj.tobytes()).decode("utf-8"), "__shape__": list(obj.shape)}
    if isinstance(obj, (np.floating, np.integer)):
        return obj.item()
    if isinstance(obj, (list, tuple)):
        return [_serialise(v) for v in obj]
    if isinstance(obj, dict):
        return {k: _serialise(v) for k, v in obj.items()}
    return obj


def _deserialise(obj):
    if isinstance(obj, dict) and obj.get("type") == "__namedtuple__":
        name = obj["__class__"].rsplit(".", 1)[-1]
        data = {k: _deserialise(v) for k, v in obj["__data__"].items()}
        cls = _BY_NAME.get(name)
        return cls(**data) if cls is not None else data
    if isinstance(obj, dict) and obj.get("type") in ("__ndarray__", "__jax_ndarray__"):
        raw = base64.b64decode(obj["__data__"])
        return np.frombuffer(raw, dtype=obj["__dtype__"]).reshape(obj["__shape__"]).copy()
    if isinstance(obj, list):
        return [_deserialise(v) for v in obj]
    if isinstance(obj, dict):
        return {k: _deserialise(v) for k, v in obj.items()}
    return obj


def save_pytree(pytree, save_file: str):
    if not _is_namedtuple(pytree):
        raise ValueError(f"Expected NamedTuple, got {type(pytree)}")
    with open(save_file, "w") as fp:
        json.dump(_serialise(pytree), fp, indent=2)


def save_results(results: NestedSamplerResults, save_file: str):
    """Write results as JSON in the reference's format."""
    if not save_file.lower().endswith(".json"):
        warnings.warn(f"Filename {save_file} does not end with .json. "
                      f"We let this pass, but you should consider using a .json file extension.")
    save_pytree(results, save_file)


def load_pytree(save_file: str) -> Any:
    with open(save_file, "r") as fp:
        return _deserialise(json.load(fp))


def load_results(save_file: str) -> NestedSamplerResults:
    """Read results written by save_results here or by jaxns (arrays come back as numpy)."""
    return load_pytree(save_file)
