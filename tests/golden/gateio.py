"""Pack / unpack gate lists to flat NumPy arrays for the golden fixtures."""
from __future__ import annotations

import numpy as np


class FixtureGate:
    """Minimal gate object (``name``, ``indices``, ``matrix``) read back from a fixture."""

    def __init__(self, name, indices, matrix):
        self.name = name
        self.indices = [int(i) for i in indices]
        self.span = len(self.indices)
        self.matrix = matrix
        self.time = None
        self.normalize = True

    def get_local_dim(self):
        return 2

    def shallow_copy(self):
        import copy
        return copy.copy(self)

    def dag(self):
        import copy
        g = copy.copy(self)
        g.matrix = np.asarray(self.matrix).conj().T
        return g


def pack_gates(gates, prefix="g"):
    ks = np.array([len(g.indices) for g in gates], dtype=np.int32)
    idx = np.full((len(gates), 8), -1, dtype=np.int32)
    mats, offs = [], [0]
    names = []
    for i, g in enumerate(gates):
        idx[i, :len(g.indices)] = g.indices
        m = np.asarray(g.matrix, dtype=np.complex128).reshape(-1)
        mats.append(m)
        offs.append(offs[-1] + m.size)
        names.append(g.name)
    return {
        f"{prefix}_k": ks, f"{prefix}_idx": idx,
        f"{prefix}_mats": np.concatenate(mats) if mats else np.zeros(0, np.complex128),
        f"{prefix}_offs": np.array(offs, dtype=np.int64),
        f"{prefix}_names": np.array(names),
    }


def unpack_gates(z, prefix="g"):
    ks, idx, mats, offs = z[f"{prefix}_k"], z[f"{prefix}_idx"], z[f"{prefix}_mats"], z[f"{prefix}_offs"]
    names = z[f"{prefix}_names"]
    out = []
    for i, k in enumerate(ks):
        d = int(round(np.sqrt(offs[i + 1] - offs[i])))
        m = mats[offs[i]:offs[i + 1]].reshape(d, d)
        out.append(FixtureGate(str(names[i]), idx[i, :k], m))
    return out
