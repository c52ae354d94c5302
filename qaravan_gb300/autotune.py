"""Choice of tile size and fusion width for the sweep engine.

``choose(nbits, dtype)`` returns ``(tile_bits, width)`` for a vector of
``2^nbits`` entries: a cached measurement when one exists, else the defaults
measured on GB300 for the 28-qubit brickwork (complex64: width 4, 14-bit
tiles; complex128: width 3, 13-bit tiles -- the shared-memory cap).
``tune(nbits, dtype)`` times the candidate configurations on a seeded Haar
brickwork of ``nbits`` bits and stores the fastest in the cache, a JSON file
at ``$QGB_AUTOTUNE_CACHE`` (default ``~/.cache/qaravan_gb300/autotune.json``).
"""
from __future__ import annotations

import json
import os
import time

import torch

_DEFAULT = {torch.complex64: (14, 4), torch.complex128: (13, 3)}
CANDIDATES = [(12, 2), (12, 3), (12, 4), (13, 3), (13, 4), (14, 3), (14, 4)]


def cache_path():
    return os.environ.get("QGB_AUTOTUNE_CACHE", os.path.join(os.path.expanduser("~"), ".cache", "qaravan_gb300",
                                                             "autotune.json"))


def _key(nbits, dtype):
    return f"{'c64' if dtype == torch.complex64 else 'c128'}:{int(nbits)}"


def _load():
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def choose(nbits, dtype=torch.complex64):
    entry = _load().get(_key(nbits, dtype))
    if entry:
        return int(entry["tile_bits"]), int(entry["width"])
    tile, width = _DEFAULT[dtype]
    return min(tile, nbits), width


def tune(nbits, dtype=torch.complex64, depth=4, reps=3, device="cuda"):
    """Measure every candidate on a seeded brickwork; cache and return the best (tile_bits, width)."""
    from . import _lib, workloads
    from .compiler import compile_ops
    from .engine import Executor
    from .statevector import gates_to_ops
    gates = workloads.brickwork_gates(nbits, depth, 4242)
    ops = gates_to_ops(gates, nbits)
    isz = 8 if dtype == torch.complex64 else 16
    state = torch.empty(2 ** nbits, dtype=dtype, device=device)
    best, best_t = None, float("inf")
    for tile, width in CANDIDATES:
        if isz == 16 and (tile > 13 or width > 4):
            continue
        plan = compile_ops(ops, nbits, mode="sweep", width=width, tile_bits=min(tile, nbits),
                           max_sweep_k=5 if isz == 8 else 4, itemsize=isz)
        ex = Executor(plan, dtype, device)
        L = _lib.lib()
        for _ in range(reps + 1):
            _lib.check(L.qgb_init_basis(state.data_ptr(), _lib.dtype_code(dtype), nbits, 0, 1, 0,
                                        _lib.stream_ptr()), "init")
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            ex.run(state)
            torch.cuda.synchronize()
            t = time.perf_counter() - t0
        if t < best_t:
            best, best_t = (min(tile, nbits), width), t
    data = _load()
    data[_key(nbits, dtype)] = {"tile_bits": best[0], "width": best[1], "seconds": best_t}
    os.makedirs(os.path.dirname(cache_path()), exist_ok=True)
    with open(cache_path(), "w") as f:
        json.dump(data, f, indent=1)
    return best
