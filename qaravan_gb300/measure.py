"""Measurement and sampling on a device statevector.

Mirrors ``measure_sv`` / ``measure_and_collapse_sv`` / ``pretty_print_sv``
(``tensorQ/statevector_sim.py:185-215``, ``core/utils.py:52-90``): outcome
probabilities are the diagonal of the reduced density matrix of the measured
sites (here: marginal sums of ``|psi|^2`` on the device), outcomes are
bitstrings in the order of ``meas_sites``, and the collapsed state keeps the
unmeasured sites in their original order, renormalised.
"""
from __future__ import annotations

import numpy as np
import torch


def outcome_probs(state, n, meas_sites):
    p = (state.reshape([2] * n).abs() ** 2).to(torch.float64)
    keep = list(meas_sites)
    rest = [q for q in range(n) if q not in keep]
    p = p.permute(*keep, *rest).reshape(2 ** len(keep), -1).sum(dim=1)
    return p.cpu().numpy()


def measure_sv(state, n, meas_sites, shots=1, rng=None):
    rng = np.random.default_rng() if rng is None else rng
    probs = outcome_probs(state, n, meas_sites)
    probs = probs / probs.sum()
    outs = [np.binary_repr(i, width=len(meas_sites)) for i in range(len(probs))]
    if shots == 1:
        return str(outs[rng.choice(len(probs), p=probs)])
    return [str(outs[i]) for i in rng.choice(len(probs), p=probs, size=shots)]


def measure_and_collapse_sv(state, n, meas_sites, rng=None):
    outcome = measure_sv(state, n, meas_sites, rng=rng)
    t = state.reshape([2] * n)
    idx = [slice(None)] * n
    for q, b in zip(meas_sites, outcome):
        idx[q] = int(b)
    out = t[tuple(idx)].reshape(-1).clone()
    out /= torch.linalg.vector_norm(out)
    return outcome, out


def pretty_print_sv(sv, threshold=1e-3):
    n = int(round(np.log2(len(sv))))
    terms = [f"{sv[i]:.4f}|{np.binary_repr(i, width=n)}⟩" for i in np.where(np.abs(sv) > threshold)[0]]
    return " + ".join(terms)
