"""Restart records of the continuation drivers (core/include/curvami/RestartManager.h).

The binary layout is the reference's, so that records written by either side load in the
other: the 8-byte magic "CURVRES\\0", int32 format version 1, int32 step k, float64 lambda,
ds, the last load increment and the external work, int32 n, then x[n] and the last state
increment[n] as float64, little-endian. A record that is not one, has another version, is
truncated or belongs to a problem with another number of dofs is rejected (None), never
half-read.
"""
from __future__ import annotations

import struct

import numpy as np

MAGIC = b"CURVRES\x00"
FORMAT_VERSION = 1
_HEAD = struct.Struct("<8si i dddd i")


def save(path: str, k: int, lam: float, ds: float, dl_old: float, W_ext: float, x, dU_old) -> bool:
    """RestartManager::save: the solver state after accepted step k - 1 (k the next step)."""
    x = np.ascontiguousarray(x, np.float64)
    dU = np.ascontiguousarray(dU_old, np.float64)
    if x.shape != dU.shape:
        return False
    with open(path, "wb") as f:
        f.write(_HEAD.pack(MAGIC, FORMAT_VERSION, int(k), float(lam), float(ds), float(dl_old), float(W_ext), x.size))
        f.write(x.astype("<f8").tobytes())
        f.write(dU.astype("<f8").tobytes())
    return True


def load(path: str, expected_ns: int = -1):
    """RestartManager::load: (k, lambda, ds, dl_old, W_ext, x, dU_old), or None when the file
    is absent, not a restart record, of another format version, truncated, or of another
    size than expected_ns (when given)."""
    try:
        with open(path, "rb") as f:
            data = f.read()
    except OSError:
        return None
    if len(data) < _HEAD.size:
        return None
    magic, version, k, lam, ds, dl, W, ns = _HEAD.unpack_from(data, 0)
    if magic != MAGIC or version != FORMAT_VERSION or ns < 0:
        return None
    if expected_ns >= 0 and ns != expected_ns:
        return None
    need = _HEAD.size + 16 * ns
    if len(data) < need:
        return None
    x = np.frombuffer(data, "<f8", ns, _HEAD.size).astype(np.float64)
    dU = np.frombuffer(data, "<f8", ns, _HEAD.size + 8 * ns).astype(np.float64)
    return k, lam, ds, dl, W, x, dU
