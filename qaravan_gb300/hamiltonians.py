"""Transverse-field Ising model: Pauli-sum terms and first/second-order Trotter circuits.

Mirrors the reference's ``TFI`` (``core/hamiltonians.py:261-272``), its term
list (``:18-88``) and ``trotter_circ`` / ``layer_from_group``
(``:112-198``) for the ``['x', 'zz']`` grouping: H = jz * sum Z_i Z_{i+1} +
h * sum X_i, full Pauli operators (no 1/2), positive signs. Order-1 Trotter
applies per step ``R1 = expm(-i dt h X)`` on every site, then
``R2 = expm(-i dt jz ZZ)`` on even pairs, then odd pairs.
"""
from __future__ import annotations

import numpy as np
import scipy.linalg

from .circuits import Circuit
from .gates import Gate
from .paulis import pauli_X, pauli_Z


class TFI:
    def __init__(self, num_x, jz=1, h=0, periodic_x=False):
        if periodic_x:
            raise NotImplementedError("open chains only")
        self.num_sites = num_x
        self.jz, self.h = jz, h
        self.terms = [(jz, [i, i + 1], ['z', 'z']) for i in range(num_x - 1)]
        if abs(h) > 1e-10:
            self.terms += [(h, [i], ['x']) for i in range(num_x)]
        self.op_grouping = ['x', 'zz']

    def pauli_sum(self):
        """``[(coeff, pauli_string), ...]`` over all terms."""
        out = []
        for c, sites, ops in self.terms:
            s = ['i'] * self.num_sites
            for q, o in zip(sites, ops):
                s[q] = o
            out.append((float(c), ''.join(s)))
        return out

    def matrix(self):
        from functools import reduce
        n = self.num_sites
        H = np.zeros((2 ** n, 2 ** n), dtype=complex)
        for c, s in self.pauli_sum():
            H += c * reduce(np.kron, [{'i': np.eye(2), 'x': pauli_X, 'z': pauli_Z}[ch] for ch in s])
        return H

    def _layer(self, group, t):
        n = self.num_sites
        if group == 'x':
            m = scipy.linalg.expm(-1j * t * self.h * pauli_X)
            return [Gate('R1', [i], m) for i in range(n)]
        m = scipy.linalg.expm(-1j * t * self.jz * np.kron(pauli_Z, pauli_Z))
        gl = [Gate('R2', [i, i + 1], m) for i in range(0, n - 1, 2)]
        gl += [Gate('R2', [i, i + 1], m) for i in range(1, n - 1, 2)]
        return gl

    def trotter_circ(self, step_size, num_steps, order=1):
        gl = []
        if order == 1:
            layers = [self._layer(g, step_size) for g in self.op_grouping]
            for _ in range(num_steps):
                for layer in layers:
                    gl += layer
        elif order == 2:
            l0h = self._layer(self.op_grouping[0], step_size / 2)
            l0 = self._layer(self.op_grouping[0], step_size)
            l1 = self._layer(self.op_grouping[1], step_size)
            gl += l0h
            for _ in range(num_steps - 1):
                gl += l1 + l0
            gl += l1 + l0h
        else:
            raise NotImplementedError("Only first and second order Trotter decomposition is supported")
        return Circuit(gl, self.num_sites)
