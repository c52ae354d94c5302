"""The project's autotuner: execution choices measured on the GPU, cached per
(workload kind, qubit count, dtype).

Three kinds of choice:

* ``sv``: how a statevector circuit runs -- ``(mode, fusion_width,
  tile_bits)``: one HBM pass per fused block of 4-6 qubits (6-qubit blocks run
  on the tensor cores, fewer bits on the CUDA cores), up to four 5-qubit blocks
  per pass on the tensor cores (``tcsweep``), or shared-memory tile sweeps of
  2-4-qubit blocks with 12-14-bit tiles. Used by ``StatevectorSim``
  when its ``mode`` is ``"auto"``.
* ``traj``: the tile bits of the persistent trajectory kernel (11-14). Used by
  ``TrajectorySim``.
* ``sweep``: ``(tile_bits, fusion_width)`` of tile sweeps over a vector of
  ``nbits`` bits (density matrices on the CUDA cores, ``DensityMatrixBatch``).

``choose_*`` returns a cached measurement when there is one; otherwise, with
``QGB_AUTOTUNE=1`` in the environment, it measures every candidate on a
seeded workload of that size the first time the size is seen and caches the
fastest; otherwise it returns the defaults measured on GB300 (complex64
statevectors: 6-qubit fused blocks on the tensor cores from 13 qubits, else
4-qubit blocks; complex128: 3-qubit blocks in 13-bit tile sweeps;
trajectories: 13-bit tiles for complex64, 12 for complex128). The cache is a
JSON file at ``$QGB_AUTOTUNE_CACHE`` (default
``~/.cache/qaravan_gb300/autotune.json``). ``select`` is the decision rule
alone (fastest measured candidate), separate from the timing so that it can
be checked without a GPU.
"""
from __future__ import annotations

import json
import os

import torch

SV_CANDIDATES = {
    torch.complex64: [("fused", 6, 14), ("fused", 5, 14), ("fused", 4, 14), ("tcsweep", 5, 13), ("sweep", 4, 14),
                      ("sweep", 3, 12)],
    torch.complex128: [("sweep", 3, 13), ("sweep", 2, 13), ("sweep", 4, 12), ("fused", 3, 13), ("fused", 2, 13)],
}
TRAJ_CANDIDATES = {torch.complex64: [11, 12, 13, 14], torch.complex128: [11, 12, 13]}
SWEEP_CANDIDATES = [(12, 2), (12, 3), (12, 4), (13, 3), (13, 4), (14, 3), (14, 4)]


def cache_path():
    return os.environ.get("QGB_AUTOTUNE_CACHE", os.path.join(os.path.expanduser("~"), ".cache", "qaravan_gb300",
                                                             "autotune.json"))


def enabled():
    return os.environ.get("QGB_AUTOTUNE", "0") not in ("0", "", "off")


def _key(kind, nbits, dtype):
    return f"{kind}:{'c64' if dtype == torch.complex64 else 'c128'}:{int(nbits)}"


def load():
    try:
        with open(cache_path()) as f:
            data = json.load(f)
        return data if isinstance(data, dict) else {}
    except (OSError, ValueError):
        return {}


def store(kind, nbits, dtype, choice, timings):
    data = load()
    data[_key(kind, nbits, dtype)] = {"choice": list(choice) if isinstance(choice, tuple) else choice,
                                      "seconds": {json.dumps(list(c) if isinstance(c, tuple) else c): t
                                                  for c, t in timings}}
    path = cache_path()
    os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(data, f, indent=1)
    os.replace(tmp, path)


def cached(kind, nbits, dtype):
    e = load().get(_key(kind, nbits, dtype))
    if not e:
        return None
    c = e["choice"]
    return tuple(c) if isinstance(c, list) else c


def select(candidates, measure):
    """Measure every candidate (``measure(c)`` -> seconds, ``None`` when it
    cannot run) and return ``(fastest, [(candidate, seconds)])``; ties keep
    the earlier candidate."""
    timings, best, best_t = [], None, float("inf")
    for c in candidates:
        t = measure(c)
        if t is None:
            continue
        timings.append((c, float(t)))
        if t < best_t:
            best, best_t = c, float(t)
    if best is None:
        raise RuntimeError("no autotuning candidate could run")
    return best, timings


# ------------------------------------------------------------ defaults

def default_sv(n, dtype):
    from . import _lib
    if dtype == torch.complex64:
        tc = n >= 13 and _lib.lib().qgb_get_dense_impl() >= 1
        return ("fused", 6 if tc else 4, 14)
    return ("sweep", 3, 13)


def default_traj(n, dtype):
    return min(13 if dtype == torch.complex64 else 12, n)


def default_sweep(nbits, dtype):
    tile, width = (14, 4) if dtype == torch.complex64 else (13, 3)
    return min(tile, nbits), width


# ------------------------------------------------------------- choices

def choose_sv(n, dtype=torch.complex64):
    c = cached("sv", n, dtype)
    if c is not None:
        return c
    if enabled():
        return tune_sv(n, dtype)[0]
    return default_sv(n, dtype)


def choose_traj(n, dtype=torch.complex64):
    c = cached("traj", n, dtype)
    if c is not None:
        return int(c)
    if enabled():
        return tune_traj(n, dtype)[0]
    return default_traj(n, dtype)


def choose(nbits, dtype=torch.complex64):
    """(tile_bits, fusion_width) of tile sweeps over 2^nbits entries."""
    c = cached("sweep", nbits, dtype)
    if c is not None:
        return int(c[0]), int(c[1])
    if enabled():
        return tune(nbits, dtype)[0]
    return default_sweep(nbits, dtype)


# --------------------------------------------------------- measurement

def _event_seconds(fn, reps):
    fn()  # warm-up (plans, caches, first-launch costs)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(reps):
        fn()
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / 1e3 / reps


def tune_sv(n, dtype=torch.complex64, depth=4, reps=3, measure=None):
    """Every statevector candidate on a seeded Haar brickwork of n qubits;
    caches and returns ``(best, timings)``."""
    if measure is None:
        from . import StatevectorSim, _lib, workloads
        from .circuits import Circuit
        circ = Circuit(workloads.brickwork_gates(n, depth, 4242), n=n)
        state = torch.empty(2 ** n, dtype=dtype, device="cuda")
        code = _lib.dtype_code(dtype)

        def measure(c):
            mode, width, tile = c
            try:
                ex = StatevectorSim(circ, dtype=dtype, mode=mode, fusion_width=width, tile_bits=tile).compile()
            except Exception:
                return None

            def run():
                _lib.check(_lib.lib().qgb_init_basis(state.data_ptr(), code, n, 0, 1, 0, _lib.stream_ptr()), "init")
                ex.run(state)
            return _event_seconds(run, reps)
    best, timings = select([tuple(c) for c in SV_CANDIDATES[dtype]], measure)
    store("sv", n, dtype, best, timings)
    return best, timings


def tune_traj(n, dtype=torch.complex64, ntraj=None, steps=2, measure=None):
    """Tile bits of the persistent trajectory kernel on the noisy TFI Trotter
    circuit (depolarising 1e-3, damping 5e-4 after every gate)."""
    if measure is None:
        from . import workloads
        from .trajectories import TrajectorySim
        circ = workloads.tfi_trotter_circuit(n, 0.05, steps)
        T = ntraj or max(64, min(1024, 2 ** max(0, 28 - n)))

        def measure(tile):
            if tile > n:
                return None
            sim = TrajectorySim(circ, T, p_dep=1e-3, gamma=5e-4, seed=5, dtype=dtype, tile_bits=tile)
            return _event_seconds(sim.run, 2)
    cands = [t for t in TRAJ_CANDIDATES[dtype] if t <= n] or [n]
    best, timings = select(cands, measure)
    store("traj", n, dtype, best, timings)
    return best, timings


def tune(nbits, dtype=torch.complex64, depth=4, reps=3, measure=None):
    """(tile_bits, width) of tile sweeps on a seeded brickwork of nbits bits."""
    isz = 8 if dtype == torch.complex64 else 16
    cands = [(min(t, nbits), w) for t, w in SWEEP_CANDIDATES if not (isz == 16 and (t > 13 or w > 4))]
    cands = list(dict.fromkeys(cands))
    if measure is None:
        from . import _lib, workloads
        from .compiler import compile_ops
        from .engine import Executor
        from .statevector import gates_to_ops
        ops = gates_to_ops(workloads.brickwork_gates(nbits, depth, 4242), nbits)
        state = torch.empty(2 ** nbits, dtype=dtype, device="cuda")
        code = _lib.dtype_code(dtype)

        def measure(c):
            tile, width = c
            plan = compile_ops(ops, nbits, mode="sweep", width=width, tile_bits=tile,
                               max_sweep_k=5 if isz == 8 else 4, itemsize=isz)
            ex = Executor(plan, dtype, "cuda")

            def run():
                _lib.check(_lib.lib().qgb_init_basis(state.data_ptr(), code, nbits, 0, 1, 0, _lib.stream_ptr()),
                           "init")
                ex.run(state)
            return _event_seconds(run, reps)
    best, timings = select(cands, measure)
    store("sweep", nbits, dtype, best, timings)
    return best, timings
