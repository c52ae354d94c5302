"""NCON tensor-network contraction, written from the published label convention.

TEST INFRASTRUCTURE ONLY. Nothing in the shipped package imports this module.

The reference (qaravan, pinned dependency ``ncon_torch==0.3`` in
``requirements.txt:7``) does all of its contraction arithmetic through
``ncon_torch.ncon`` / ``ncon_torch.permute``. That package is not vendored in the
reference tree and cannot be installed here, so this is a restatement of the
published NCON convention (Pfeifer, Haegeman & Verstraete, "NCON: A tensor
network contractor for MATLAB", arXiv:1402.0939):

* every tensor carries one integer label per axis;
* a positive label appears exactly twice and is summed over (contracted);
  if both occurrences sit on the same tensor it is a partial trace;
* negative labels are open; the result's axes are ordered -1, -2, -3, ...;
* positive labels are contracted in ascending order (the default order).

Arithmetic is ``tensordot`` + ``transpose`` on NumPy arrays, or the torch
equivalents on torch tensors, so it follows the reference's call sites
(``tensorQ/statevector_sim.py:136,139``; ``tensorQ/density_matrix_sim.py:42``)
operation for operation.
"""
from __future__ import annotations

import numpy as np

try:  # torch is optional for the oracle; the reference's torch backend uses it
    import torch
except Exception:  # pragma: no cover
    torch = None


def _is_torch(t) -> bool:
    return torch is not None and torch.is_tensor(t)


def _tensordot(a, b, axes_a, axes_b):
    if _is_torch(a) or _is_torch(b):
        return torch.tensordot(a, b, dims=(list(axes_a), list(axes_b)))
    return np.tensordot(a, b, axes=(list(axes_a), list(axes_b)))


def _transpose(t, perm):
    perm = [int(p) for p in perm]
    if _is_torch(t):
        return t.permute(*perm)
    return np.transpose(t, perm)


def _trace_pair(t, ax1, ax2):
    if _is_torch(t):
        return torch.diagonal(t, dim1=ax1, dim2=ax2).sum(-1)
    return np.trace(t, axis1=ax1, axis2=ax2)


def permute(t, perm):
    """Axis permutation (the ``ncon_torch.permute`` call site at
    ``tensorQ/statevector_sim.py:136``)."""
    return _transpose(t, perm)


def _self_traces(t, labels):
    labels = list(labels)
    while True:
        seen = {}
        pair = None
        for ax, lab in enumerate(labels):
            if lab > 0 and lab in seen:
                pair = (seen[lab], ax)
                break
            seen[lab] = ax
        if pair is None:
            return t, labels
        a1, a2 = pair
        t = _trace_pair(t, a1, a2)
        labels = [lab for ax, lab in enumerate(labels) if ax not in (a1, a2)]


def ncon(tensors, index_lists, con_order=None):
    """Contract ``tensors`` according to ``index_lists`` (NCON convention)."""
    tensors = list(tensors)
    labels = [list(int(x) for x in l) for l in index_lists]
    if len(tensors) != len(labels):
        raise ValueError("one label list per tensor is required")
    for i, (t, l) in enumerate(zip(tensors, labels)):
        if t.ndim != len(l):
            raise ValueError(f"tensor {i} has {t.ndim} axes but {len(l)} labels")
        tensors[i], labels[i] = _self_traces(t, l)

    if con_order is None:
        con_order = sorted({lab for l in labels for lab in l if lab > 0})
    for lab in con_order:
        holders = [i for i, l in enumerate(labels) if lab in l]
        if not holders:
            continue  # already removed together with an earlier common label
        if len(holders) != 2:
            raise ValueError(f"label {lab} must appear on exactly two tensors")
        i, j = holders
        common = [x for x in labels[i] if x > 0 and x in labels[j]]
        ax_i = [labels[i].index(x) for x in common]
        ax_j = [labels[j].index(x) for x in common]
        new = _tensordot(tensors[i], tensors[j], ax_i, ax_j)
        new_labels = [x for x in labels[i] if x not in common] + \
                     [x for x in labels[j] if x not in common]
        tensors[i], labels[i] = new, new_labels
        del tensors[j], labels[j]

    # remaining tensors share no labels: outer product in list order
    t, l = tensors[0], labels[0]
    for t2, l2 in zip(tensors[1:], labels[1:]):
        t = _tensordot(t, t2, [], [])
        l = l + l2
    if len(l) == 0:
        return t
    order = sorted(range(len(l)), key=lambda ax: -l[ax])  # -1, -2, -3, ...
    return _transpose(t, order)
