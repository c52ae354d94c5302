"""Gate objects with the reference's index and matrix conventions.

Host-side mirror of ``core/gates.py`` and ``core/param_gates.py`` of the
reference, so circuits can be built where the reference package is not
installed. Reference gate objects work too: every simulator here reads only
``.name``, ``.indices``, ``.matrix`` (NumPy or torch), ``.span`` and, for
noise carriers, ``.nm`` / ``.time`` / ``.dd``, and ``Reset.normalize``.

Conventions kept (they decide the numbers):

* a gate's matrix is indexed by its ``indices`` list in order, ``indices[0]``
  being the most-significant bit of the row/column index
  (``tensorQ/statevector_sim.py:124-140``);
* ``CNOT(indices)`` takes ``(target, control)`` and stores ascending sites,
  transposing the matrix when the target is the larger site
  (``core/gates.py:135-170,217-220``);
* rotations carry no factor 1/2: ``RX(t) = expm(-i t X)``
  (``core/param_gates.py:51-103``);
* ``Reset`` is a projector followed by renormalisation
  (``core/gates.py:172-187``, ``core/base_sim.py:25-28``).

Only qubits (local dimension 2) are supported by the CUDA path.
"""
from __future__ import annotations

import copy
from functools import reduce

import numpy as np
import scipy.linalg
import torch

from .paulis import pauli_X, pauli_Y, pauli_Z, pauli_mapping


def _is_torch(x) -> bool:
    return torch.is_tensor(x)


class Gate:
    """Dense gate on ``indices`` (``core/gates.py:32-55``)."""

    def __init__(self, name, indices, matrix, time=None):
        self.name = name
        self.indices = [indices] if isinstance(indices, (int, np.integer)) else list(indices)
        self.indices = [int(i) for i in self.indices]
        self.span = len(self.indices)
        self.matrix = matrix
        self.time = time

    def __str__(self):
        return f"{self.name} gate on site(s) {self.indices}"

    def to_superop(self):
        m = self.matrix
        if _is_torch(m):
            m = m.detach().cpu().numpy()
        return np.kron(np.conj(m), m).reshape([self.get_local_dim()] * 4 * self.span)

    def get_local_dim(self):
        return int(round(self.matrix.shape[0] ** (1 / self.span)))

    def dag(self):
        g = copy.deepcopy(self)
        g.matrix = g.matrix.conj().T
        return g

    def shallow_copy(self):
        # Gate(self.name, self.indices, self.matrix, time=self.time) without re-validating the indices
        g = Gate.__new__(Gate)
        g.name, g.indices, g.matrix, g.time = self.name, [int(i) for i in self.indices], self.matrix, self.time
        g.span = len(g.indices)
        return g


def embed_operator(num_sites, active_sites, local_ops, local_dim=2, dense=False, factor=False):
    """Operator on ``num_sites`` sites from local ones (``core/gates.py:8-30``):
    a Pauli string (one character per active site), one ndarray on contiguous
    ``active_sites`` (inserted at the first of them), or a list of one-site
    matrices (``factor``: each halved, the spin-1/2 convention); dense, or a
    SciPy CSR matrix."""
    import scipy.sparse as sp
    if isinstance(local_ops, str):
        local_ops = [pauli_mapping[op] for op in local_ops]
    if isinstance(local_ops, np.ndarray):
        full = [np.eye(local_dim, dtype=complex) for i in range(num_sites) if i not in active_sites]
        full.insert(active_sites[0], local_ops)
        return reduce(np.kron, full)
    if dense:
        full = [np.eye(local_dim, dtype=complex) for _ in range(num_sites)]
        for site, op in zip(active_sites, local_ops):
            full[site] = op / 2 if factor else op
        return reduce(np.kron, full)
    full = [sp.eye(local_dim, format="csr", dtype=complex) for _ in range(num_sites)]
    for site, op in zip(active_sites, local_ops):
        full[site] = sp.csr_matrix(op / 2 if factor else op)
    return reduce(sp.kron, full)


class SuperOp:
    """A superoperator on ``span`` contiguous sites from ``start_idx``
    (``core/gates.py:57-79``), in the layout of ``Gate.to_superop``;
    ``DensityMatrixSim`` applies its matrix as is (``tensorQ/density_matrix_sim.py:38-42``).
    The reference's class has no ``shallow_copy``, so its simulators (which copy
    the circuit) cannot run one; here it copies like a gate."""

    def __init__(self, name, span, matrix, start_idx=0, time=0.0):
        self.name = name
        self.start_idx = start_idx
        self.indices = [start_idx + i for i in range(span)]
        self.span = span
        self.matrix = matrix
        self.shape = matrix.shape
        self.time = time

    def shift(self, new_start_idx):
        return SuperOp(self.name, self.span, self.matrix, start_idx=new_start_idx, time=self.time)

    def shallow_copy(self):
        return self.shift(self.start_idx)

    def get_local_dim(self):
        return int(round(np.prod(self.shape) ** (1 / (4 * self.span))))

    def __str__(self):
        return f"{self.name} superoperator on site(s) {self.indices}"


class ID(Gate):
    """Idling / noise carrier (``core/gates.py:81-95``)."""

    def __init__(self, local_dim, time, indices, nm, dd=False):
        super().__init__("ID", indices, matrix=None, time=time)
        self.matrix = np.eye(local_dim ** self.span)
        self.dd = dd
        self.nm = nm

    def to_superop(self):
        return self.nm.get_superop(self.time, self.dd).reshape([self.get_local_dim()] * 4 * self.span)

    def shallow_copy(self):
        # The reference's ID inherits Gate.shallow_copy and silently drops its
        # noise model on Circuit.copy(); here the carrier keeps it.
        return ID(self.get_local_dim(), self.time, self.indices, self.nm, self.dd)


class CUGate(Gate):
    """Controlled ``subgate`` (``core/gates.py:102-135``): ``indices`` = (targets
    ascending and adjacent, control), the control next to the targets; the
    subgate acts when the control is 1. A control above the targets
    (``bottom_heavy``) moves to the front of the stored indices; a control below
    them keeps its place with the matrix transposed to (control, targets) order
    by the reference's reshape. Long-range controls are not implemented, as in
    the reference."""

    def __init__(self, indices, subgate):
        from scipy.linalg import block_diag
        d = subgate.get_local_dim()
        sub = np.asarray(subgate.matrix)
        s = sub.shape[0]
        idx = np.array([int(i) for i in indices])
        if np.min(np.abs(idx[:-1] - idx[-1])) > 1:
            raise NotImplementedError("Long range CUGate has not been implemented yet")
        mat = block_diag(*([np.eye(s), sub] + [np.eye(s)] * (d - 2)))
        if idx[-2] < idx[-1]:
            mat = mat.reshape(d, s, d, s).transpose(1, 0, 3, 2).reshape(d * s, d * s)
            bottom = False
        elif idx[-1] < idx[0]:
            idx = np.concatenate(([idx[-1]], idx[:-1]))
            bottom = True
        else:
            raise ValueError("indices does not have allowed ordering")
        super().__init__(f"CU{d}", [int(i) for i in idx], mat)
        self.bottom_heavy = bottom


class CNOTGate(Gate):
    """``indices = (target, control)`` (``core/gates.py:137-170``)."""

    def __init__(self, indices, matrix, n):
        d = int(np.sqrt(matrix.shape[0]))
        indices = [int(i) for i in indices]
        if abs(indices[0] - indices[1]) > 1:
            temp = np.array(indices) + 1
            if temp[0] % n < temp[1] % n:
                mat, bottom = matrix, False
            else:
                indices = indices[::-1]
                mat = matrix.reshape(d, d, d, d).transpose(1, 0, 3, 2).reshape(d * d, d * d)
                bottom = True
        else:
            if indices[0] < indices[1]:
                mat, bottom = matrix, False
            else:
                indices = indices[::-1]
                mat = matrix.reshape(d, d, d, d).transpose(1, 0, 3, 2).reshape(d * d, d * d)
                bottom = True
        super().__init__(f"CNOT{d}", indices, mat)
        self.bottom_heavy = bottom


class Reset(Gate):
    """Projector onto ``reset_to`` then renormalise (``core/gates.py:172-187``)."""

    def __init__(self, indices, reset_to: str, normalize=True, time=None):
        up = np.array([[1, 0], [0, 0]])
        down = np.array([[0, 0], [0, 1]])
        matrix = reduce(np.kron, [up if b == '0' else down for b in reset_to])
        super().__init__("Reset", indices, matrix, time=time)
        self.reset_to = reset_to
        self.normalize = normalize

    def shallow_copy(self):
        return Reset(self.indices, self.reset_to, self.normalize, self.time)


def SX(indices):
    return Gate("SX", indices, (1 / np.sqrt(2)) * np.array([[1, -1j], [-1j, 1]]))


def X(indices):
    return Gate("X", indices, np.array([[0, 1], [1, 0]]))


def Y(indices):
    return Gate("Y", indices, pauli_Y)


def Z(indices):
    return Gate("Z", indices, pauli_Z)


def H(indices):
    return Gate("H", indices, np.array([[1, 1], [1, -1]]) / np.sqrt(2))


def SDG(indices):
    return Gate("SDG", indices, np.array([[1, 0], [0, -1j]]))


def CNOT(indices, n=1000):
    """``indices = (target, control)`` (``core/gates.py:217-220``)."""
    return CNOTGate(indices, np.array([[1, 0, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0], [0, 1, 0, 0]]), n=n)


def CZ(indices):
    return Gate("CZ", indices, np.diag([1, 1, 1, -1]).astype(complex))


def SWAP(indices):
    return Gate("SWAP", indices, np.array([[1, 0, 0, 0], [0, 0, 1, 0], [0, 1, 0, 0], [0, 0, 0, 1]]))


def iSWAP(indices):
    return Gate("iSWAP", indices, np.array([[1, 0, 0, 0], [0, 0, 1j, 0], [0, 1j, 0, 0], [0, 0, 0, 1]]))


def proj_up(indices):
    return Gate("P0", indices, np.array([[1, 0], [0, 0]]))


def proj_down(indices):
    return Gate("P1", indices, np.array([[0, 0], [0, 1]]))


def random_unitary(size):
    """The reference's (non-Haar) generator, ``core/gates.py:289-293``."""
    a = np.random.rand(size, size) + 1.j * np.random.rand(size, size)
    _, u = np.linalg.eigh(a @ a.conj().T)
    return u


def is_unitary(u):
    eye = np.eye(u.shape[0])
    return np.allclose(u @ u.conj().T, eye, atol=1e-10) and np.allclose(u.conj().T @ u, eye, atol=1e-10)


pauli_gate_map = {'x': X, 'y': Y, 'z': Z}


def pauli_string_to_gates(string):
    return [pauli_gate_map[op](i) for i, op in enumerate(string) if op != 'i']


# ---------------------------------------------------------------- parametrised

_XT = torch.tensor([[0, 1], [1, 0]], dtype=torch.complex128)
_YT = torch.tensor([[0, -1.j], [1.j, 0]], dtype=torch.complex128)
_ZT = torch.tensor([[1, 0], [0, -1]], dtype=torch.complex128)
_xxN, _yyN, _zzN = np.kron(pauli_X, pauli_X), np.kron(pauli_Y, pauli_Y), np.kron(pauli_Z, pauli_Z)
_xxT, _yyT, _zzT = torch.kron(_XT, _XT), torch.kron(_YT, _YT), torch.kron(_ZT, _ZT)


def _arr(x, backend):
    if backend == "torch":
        return torch.stack([torch.stack([torch.as_tensor(e, dtype=torch.complex128) for e in row])
                            for row in x]).to(torch.complex128)
    return np.array(x, dtype=np.complex128)


class ParamGate(Gate):
    """Angle-parametrised gate (``core/param_gates.py:21-49``). Torch angles keep
    the autograd graph through ``torch.linalg.matrix_exp``.

    With torch angles the matrix is built when ``matrix`` is first read (the
    reference builds it in the constructor): the values are the same, computed
    from the angles as they were at construction (an angle changed in place
    afterwards still contributes its gradient, at the old value). Paths that
    take the angles directly, such as the complex64 adjoint, never build it."""

    def __init__(self, name, indices, *args):
        super().__init__(name, indices, None)
        self.backend = "torch" if _is_torch(args[0]) else "numpy"
        if type(args[0]) == np.ndarray:  # a matrix (core/param_gates.py:26-29), angles solved from it
            self.matrix = args[0]
            self.angles = self.solve_angles()
        else:
            self.angles = args
            if self.backend == "torch":
                self._angle_values = tuple(a.detach().clone() if _is_torch(a) else a for a in args)
                self._angle_versions = tuple(a._version if _is_torch(a) else None for a in args)
                self._built = {}  # shared with shallow copies, which then share the built matrix
                self._lazy = True
            else:
                self.matrix = self.construct_matrix()
                self._angle_matrix = self.matrix  # identity marks "matrix still the one built from the angles"

    @property
    def matrix(self):
        if self.__dict__.get("_lazy"):
            self._build_matrix()
        return self.__dict__.get("_matrix")

    @matrix.setter
    def matrix(self, m):
        self.__dict__["_lazy"] = False
        self.__dict__["_matrix"] = m

    def matrix_pending(self):
        """True while the matrix built from torch angles has not been read yet."""
        return bool(self.__dict__.get("_lazy"))

    def angle_values(self):
        """The angles' values at construction (detached)."""
        v = self.__dict__.get("_angle_values")
        return v if v is not None else tuple(a.detach() if _is_torch(a) else a for a in self.angles)

    def angles_unchanged(self):
        """True while no torch angle was modified in place since construction
        (the live angles then hold the construction-time values)."""
        vers = self.__dict__.get("_angle_versions")
        return vers is None or all(not _is_torch(a) or a._version == v for a, v in zip(self.angles, vers))

    def _build_matrix(self):
        m = self._built.get("matrix")
        if m is None:
            live = self.angles
            args = live
            if any(_is_torch(a) and a._version != v for a, v in zip(live, self._angle_versions)):
                # changed in place since construction: the construction-time value, same gradient
                args = tuple(v + (a - a.detach()) if _is_torch(a) else a for a, v in zip(live, self._angle_values))
            self.angles = args
            try:
                m = self.construct_matrix()
            finally:
                self.angles = live
            self._built["matrix"] = m
        self.matrix = m
        self._angle_matrix = m

    def get_local_dim(self):
        return 2 if self.__dict__.get("_lazy") else super().get_local_dim()

    def __str__(self):
        return f"{self.name} gate on site(s) {self.indices} with angle(s) {self.angles}"

    def update_matrix(self, mat):
        self.matrix = mat

    def construct_matrix(self):
        raise NotImplementedError

    def solve_angles(self):
        return "unsolved"

    def built_from_angles(self):
        """True while ``matrix`` is the one constructed from ``angles`` (not
        replaced by ``update_matrix`` / ``Circuit.update_gate``)."""
        if self.__dict__.get("_lazy"):
            return True
        return self.matrix is not None and self.matrix is getattr(self, "_angle_matrix", None)

    def shallow_copy(self):
        # The reference rebuilds the gate from its angles (core/param_gates.py:48-49).
        # While the matrix is still the one built from those angles the rebuild
        # would recompute the same values, so the copy shares it instead.
        if self.built_from_angles():
            g = copy.copy(self)
            g.indices = list(self.indices)
            return g
        return type(self)(self.indices, *self.angles)

    def _expm(self, gen_np, gen_t):
        t = self.angles[0]
        if self.backend == "torch":
            return torch.linalg.matrix_exp(-1.j * t * gen_t)
        return scipy.linalg.expm(-1.j * t * gen_np)


class RX(ParamGate):
    def __init__(self, indices, *args):
        super().__init__("RX", indices, *args)

    def construct_matrix(self):
        return self._expm(pauli_X, _XT)


class RY(ParamGate):
    def __init__(self, indices, *args):
        super().__init__("RY", indices, *args)

    def construct_matrix(self):
        return self._expm(pauli_Y, _YT)


class RZ(ParamGate):
    def __init__(self, indices, *args):
        super().__init__("RZ", indices, *args)

    def construct_matrix(self):
        return self._expm(pauli_Z, _ZT)


class RXX(ParamGate):
    def __init__(self, indices, *args):
        super().__init__("RXX", indices, *args)

    def construct_matrix(self):
        return self._expm(_xxN, _xxT)


class RYY(ParamGate):
    def __init__(self, indices, *args):
        super().__init__("RYY", indices, *args)

    def construct_matrix(self):
        return self._expm(_yyN, _yyT)


class RZZ(ParamGate):
    def __init__(self, indices, *args):
        super().__init__("RZZ", indices, *args)

    def construct_matrix(self):
        return self._expm(_zzN, _zzT)


class XYCoupling(ParamGate):
    def __init__(self, indices, *args):
        super().__init__("XYCoupling", indices, *args)

    def construct_matrix(self):
        return self._expm(_xxN + _yyN, _xxT + _yyT)


class HeisenbergCoupling(ParamGate):
    def __init__(self, indices, *args):
        super().__init__("HeisenbergCoupling", indices, *args)

    def construct_matrix(self):
        return self._expm(_xxN + _yyN + _zzN, _xxT + _yyT + _zzT)


class CPhase(ParamGate):
    def __init__(self, indices, *args):
        super().__init__("CPhase", indices, *args)

    def construct_matrix(self):
        xp = torch if self.backend == "torch" else np
        ph = xp.exp(1.j * self.angles[0])
        return _arr([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, 0], [0, 0, 0, ph]], self.backend)

    def solve_angles(self):
        return (np.angle(self.matrix[3, 3]),)


class U(ParamGate):
    """``U(indices, theta, phi, lambda)`` (``core/param_gates.py:118-158``)."""

    def __init__(self, indices, *args):
        super().__init__("U", indices, *args)

    def construct_matrix(self):
        t, p, l = self.angles
        xp = torch if self.backend == "torch" else np
        return _arr([[xp.cos(t / 2), -xp.exp(1j * l) * xp.sin(t / 2)],
                     [xp.exp(1j * p) * xp.sin(t / 2), xp.exp(1j * (p + l)) * xp.cos(t / 2)]], self.backend)

    def solve_angles(self):
        # as core/param_gates.py:131-142, the stored matrix loses the phase of its
        # top-left entry (a U built from a matrix simulates without that global phase)
        self.matrix = self.matrix / np.exp(1.j * np.angle(self.matrix[0, 0]))
        m = self.matrix
        t = np.arccos(np.clip(m[0, 0].real, -1, 1)) * 2
        if abs(np.sin(t / 2)) > 1e-12:
            l = np.angle(-m[0, 1] / np.sin(t / 2))
            p = np.angle(m[1, 1] / m[0, 0]) - l
        else:
            l = p = np.angle(m[1, 1]) / 2
        return t, p, l

    def decompose(self, basis='ZSX'):
        """RZ / SX sequence of ``core/param_gates.py:144-156`` (first applied
        first), from the angles solved from the matrix."""
        if basis != 'ZSX':
            raise NotImplementedError(f"{basis} basis decomposition has not been implemented")
        t, p, l = self.solve_angles()
        i = self.indices
        return list(reversed([RZ(i, p + np.pi), SX(i), RZ(i, t + np.pi), SX(i), RZ(i, l)]))


class Givens(ParamGate):
    def __init__(self, indices, *args):
        super().__init__("Givens", indices, *args)

    def construct_matrix(self):
        th = self.angles[0]
        xp = torch if self.backend == "torch" else np
        c, s = xp.cos(th / 2), xp.sin(th / 2)
        return _arr([[1, 0, 0, 0], [0, c, -s, 0], [0, s, c, 0], [0, 0, 0, 1]], self.backend)

    def solve_angles(self):
        return (np.arccos(self.matrix[1, 1]) * 2,)  # core/param_gates.py:185-187


def kak_unitary(params):
    """15-parameter two-qubit unitary (``core/param_gates.py:247-259``)."""
    backend = "torch" if _is_torch(params) else "numpy"
    xp = torch if backend == "torch" else np
    xx, yy, zz = (_xxT, _yyT, _zzT) if backend == "torch" else (_xxN, _yyN, _zzN)
    expm = torch.linalg.matrix_exp if backend == "torch" else scipy.linalg.expm
    left = xp.kron(U(0, *params[0:3]).matrix, U(0, *params[3:6]).matrix)
    right = xp.kron(U(0, *params[9:12]).matrix, U(0, *params[12:15]).matrix)
    arg = sum(p * P for p, P in zip(params[6:9], [xx, yy, zz]))
    return left @ expm(1.j * arg) @ right
