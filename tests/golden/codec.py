"""JSON codec for the plan payload fixtures in this directory.

A plan payload is the nested dict that the reference's
``PreparedLindbladProblem.to_payload()`` produces (centrex_tlf/lindblad/plan_static.py:58-68):
plain dicts/lists/numbers plus numpy arrays and Python complex scalars.  JSON cannot hold
either of those, so arrays are stored as base64 of their little-endian bytes and complex
scalars as a two-element list tagged ``__complex__``.  Test infrastructure only.
"""

from __future__ import annotations

import base64
import json
from pathlib import Path
from typing import Any

import numpy as np

HERE = Path(__file__).resolve().parent


def encode(obj: Any) -> Any:
    if isinstance(obj, np.ndarray):
        arr = np.ascontiguousarray(obj)
        dtype = arr.dtype.newbyteorder("<")
        return {
            "__ndarray__": base64.b64encode(arr.astype(dtype, copy=False).tobytes()).decode("ascii"),
            "dtype": dtype.str,
            "shape": list(arr.shape),
        }
    if isinstance(obj, (np.bool_, bool)):
        return bool(obj)
    if isinstance(obj, (np.integer,)):
        return int(obj)
    if isinstance(obj, (np.floating,)):
        return float(obj)
    if isinstance(obj, (complex, np.complexfloating)):
        return {"__complex__": [float(obj.real), float(obj.imag)]}
    if isinstance(obj, dict):
        return {str(k): encode(v) for k, v in obj.items()}
    if isinstance(obj, (list, tuple)):
        return [encode(v) for v in obj]
    return obj


def decode(obj: Any) -> Any:
    if isinstance(obj, dict):
        if "__ndarray__" in obj:
            raw = base64.b64decode(obj["__ndarray__"])
            return np.frombuffer(raw, dtype=np.dtype(obj["dtype"])).reshape(obj["shape"]).copy()
        if "__complex__" in obj:
            re, im = obj["__complex__"]
            return complex(re, im)
        return {k: decode(v) for k, v in obj.items()}
    if isinstance(obj, list):
        return [decode(v) for v in obj]
    return obj


def save(name: str, obj: Any) -> Path:
    path = HERE / f"{name}.json"
    path.write_text(json.dumps(encode(obj), separators=(",", ":")))
    return path


def load(name: str) -> Any:
    return decode(json.loads((HERE / f"{name}.json").read_text()))
