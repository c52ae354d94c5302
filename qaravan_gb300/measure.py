"""Measurement and sampling on a device statevector (CUDA kernels in
``csrc/measure.cu``).

Mirrors ``measure_sv`` / ``measure_and_collapse_sv`` / ``pretty_print_sv``
(``tensorQ/statevector_sim.py:185-215``, ``core/utils.py:52-90``):

* outcome probabilities are the diagonal of the reduced density matrix of the
  measured sites, which ``rdm_from_sv`` (``:182-183``) builds with the sites in
  ascending order -- so outcome bit strings list the measured sites ascending,
  whatever order ``meas_sites`` has;
* outcomes are drawn on the device (float64 prefix sums, binary search on
  Philox4x32-10 uniforms seeded from ``rng``), not with ``numpy.random.choice``:
  the same distribution, a different random stream;
* the collapsed state keeps the unmeasured sites in their order and is
  renormalised; like the reference, it reads the outcome string in
  ``meas_sites`` order when it builds the projector (``:198-208``), which
  differs from the ascending order of the sampled string when ``meas_sites``
  is unsorted.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib


def outcome_probs(state, n, meas_sites):
    """float64 device tensor of the 2^m outcome probabilities, measured sites ascending."""
    _lib.require_cuda(state)
    sites = sorted(int(q) for q in meas_sites)
    m = len(sites)
    L = _lib.lib()
    nbytes = L.qgb_probs_scratch_bytes(n, m)
    scratch = torch.empty(max(nbytes // 8, 1), dtype=torch.float64, device=state.device)
    probs = torch.empty(2 ** m, dtype=torch.float64, device=state.device)
    _lib.check(L.qgb_outcome_probs(state.data_ptr(), _lib.dtype_code(state.dtype), n, _lib.int_array(sites), m,
                                   probs.data_ptr(), scratch.data_ptr(), scratch.numel() * 8,
                                   _lib.stream_ptr(state.device)), "outcome_probs")
    return probs


def sample_outcomes(probs, shots, seed):
    """int64 device tensor of ``shots`` outcome indices drawn from ``probs`` (device float64)."""
    m = int(round(np.log2(probs.numel())))
    L = _lib.lib()
    nbytes = L.qgb_sample_scratch_bytes(m)
    scratch = torch.empty(max(nbytes // 8, 1), dtype=torch.float64, device=probs.device)
    out = torch.empty(int(shots), dtype=torch.int64, device=probs.device)
    _lib.check(L.qgb_sample_outcomes(probs.data_ptr(), m, int(shots), int(seed) & ((1 << 64) - 1), out.data_ptr(),
                                     scratch.data_ptr(), scratch.numel() * 8, _lib.stream_ptr(probs.device)),
               "sample_outcomes")
    return out


def _seed(rng):
    rng = np.random.default_rng() if rng is None else rng
    return int(rng.integers(0, 2 ** 63 - 1))


def measure_sv(state, n, meas_sites, shots=1, rng=None):
    probs = outcome_probs(state, n, meas_sites)
    m = len(meas_sites)
    idx = sample_outcomes(probs, shots, _seed(rng)).cpu().numpy()
    outs = [np.binary_repr(int(i), width=m) for i in idx]
    return outs[0] if shots == 1 else outs


def collapse_sv(state, n, meas_sites, outcome, probs=None):
    """Post-measurement state for the outcome string ``outcome`` (read in
    ``meas_sites`` order, as the reference's projector does)."""
    sites = list(meas_sites)
    sidx = sorted(sites)
    m = len(sites)
    bits = "".join(outcome[sites.index(s)] for s in sidx)
    if probs is None:
        probs = outcome_probs(state, n, sites)
    out = torch.empty(2 ** (n - m), dtype=state.dtype, device=state.device)
    _lib.check(_lib.lib().qgb_collapse(state.data_ptr(), _lib.dtype_code(state.dtype), n, _lib.int_array(sidx), m,
                                       int(bits, 2), probs.data_ptr(), out.data_ptr(), _lib.stream_ptr(state.device)),
               "collapse")
    return out


def measure_and_collapse_sv(state, n, meas_sites, rng=None):
    probs = outcome_probs(state, n, meas_sites)
    m = len(meas_sites)
    outcome = np.binary_repr(int(sample_outcomes(probs, 1, _seed(rng)).cpu().item()), width=m)
    return outcome, collapse_sv(state, n, meas_sites, outcome, probs)


def pretty_print_sv(sv, threshold=1e-3):
    """Basis-state expansion of a state, amplitudes above ``threshold`` (``core/utils.py:77-89``)."""
    n = int(round(np.log2(len(sv))))
    terms = [f"{sv[i]:.4f}|{np.binary_repr(i, width=n)}⟩" for i in np.where(np.abs(sv) > threshold)[0]]
    return " + ".join(terms)


def pretty_print_dm(dmat, threshold=1e-3):
    """A density matrix as a mixture of its eigenvectors, weights above
    ``threshold`` by decreasing magnitude, each written as ``pretty_print_sv``
    does (``core/utils.py:52-75``)."""
    dmat = np.asarray(dmat)
    evals, evecs = np.linalg.eigh(dmat)
    order = np.argsort(np.abs(evals))[::-1]
    out = []
    for ev, vec in zip(evals[order], evecs[:, order].T):
        if abs(ev) > threshold:
            out.append(f"{ev.real:.4f} * ({pretty_print_sv(vec, threshold)})")
    return "\n ".join(out)
