"""Noise channels as Kraus lists and superoperators.

Host-side mirror of ``core/noise.py``: ``Noise.get_superop`` = sum of
``kron(conj K, K)`` (``:5-13``), ``QubitNoise`` T1/T2 Kraus (``:25-49``),
``PauliNoise`` (``:90-163``), ``PauliLindbladNoise`` (``:166-210``) and
``gate_time`` (``:212-230``). Two helpers name the channels used by the noisy
workloads: ``depolarizing(p)`` is ``PauliNoise(['i','x','y','z'],
[1-p, p/3, p/3, p/3])`` and ``amplitude_damping(gamma)`` is the two-operator
channel ``K0 = diag(1, sqrt(1-gamma))``, ``K1 = sqrt(gamma)|0><1|`` (the exact
``QubitNoise`` with ``t2 = inf``, whose other two operators vanish).
"""
from __future__ import annotations

import numpy as np

from .gates import pauli_string_to_gates
from .paulis import pauli_commute, pauli_mapping, pauli_multiply, pauli_strings


def _embed_dense(s):
    from functools import reduce
    return reduce(np.kron, [pauli_mapping[c] for c in s])


class Noise:
    def get_kraus(self, *args, **kwargs):
        raise NotImplementedError

    def get_superop(self, *args, **kwargs):
        return sum(np.kron(np.conj(k), k) for k in self.get_kraus(*args, **kwargs))


class ThermalNoise(Noise):
    def __init__(self, t1, t2, one_site_time, two_site_time, local_dim, coupling=1.0):
        self.t1, self.t2 = t1, t2
        self.idling_t2 = coupling * t2 + (1 - coupling) * t1 * 2
        self.one_site_time, self.two_site_time = one_site_time, two_site_time
        self.local_dim = local_dim
        self.coupling = coupling


class QubitNoise(ThermalNoise):
    def __init__(self, t1, t2, one_qubit_time, two_qubit_time, coupling=1.0):
        super().__init__(t1, t2, one_qubit_time, two_qubit_time, 2, coupling)

    def get_kraus(self, time, dd=False):
        t2 = self.t2 if not dd else self.idling_t2
        p1 = 1 - np.exp(-time / self.t1)
        p2 = 1 - np.exp(-time / t2)
        p1c, p2c = 1 - p1, 1 - p2
        k = [np.zeros((2, 2)) for _ in range(4)]
        k[0][0, 0] = np.sqrt(p2)
        k[0][1, 1] = -np.sqrt(p2 * p1c)
        k[1][0, 1] = -np.sqrt(p1 * p2)
        k[2][0, 0] = np.sqrt(p2c)
        k[2][1, 1] = np.sqrt(p1c * p2c)
        k[3][0, 1] = np.sqrt(p1 * p2c)
        return k


class PauliNoise(Noise):
    def __init__(self, strings, probs):
        assert abs(np.sum(probs) - 1) < 1e-3, f"Probabilities must sum to 1, but got {np.sum(probs)}"
        self.probs = [p for p in probs if abs(p) > 1e-6]
        self.strings = [s for s, p in zip(strings, probs) if abs(p) > 1e-6]
        self.num_sites = len(strings[0])
        self.local_dim = 2

    def sample_string(self, rng=None):
        r = np.random if rng is None else rng
        return self.strings[r.choice(len(self.strings), p=self.probs)]

    def symp_matrix(self, full=False):
        s = pauli_strings(self.num_sites) if full else self.strings
        return np.array([[(-1) ** (not pauli_commute(a, b)) for a in s] for b in s])

    def ptm(self):
        f = []
        for s in pauli_strings(self.num_sites):
            f.append(sum(p if pauli_commute(s, s2) else -p for s2, p in zip(self.strings, self.probs)))
        return np.diag(f)

    def fidelities(self):
        return self.symp_matrix() @ self.probs

    def get_kraus(self, *args, **kwargs):
        return [np.emath.sqrt(p) * _embed_dense(s) for p, s in zip(self.probs, self.strings)]

    def pinv(self):
        """The inverse channel as a (quasi-probability) Pauli channel: fidelities
        inverted and mapped back through the full symplectic matrix
        (``core/noise.py:131-135``)."""
        inv_fid = 1 / np.diag(self.ptm())
        inv_probs = np.linalg.inv(self.symp_matrix(full=True)) @ inv_fid
        return PauliNoise(pauli_strings(self.num_sites), inv_probs)

    def compose(self, other):
        acc = {}
        for s1, p1 in zip(self.strings, self.probs):
            for s2, p2 in zip(other.strings, other.probs):
                s, _ = pauli_multiply(s1, s2)
                acc[s] = acc.get(s, 0) + p1 * p2
        return PauliNoise(list(acc), list(acc.values()))

    def sample(self, rng=None):
        return pauli_string_to_gates(self.sample_string(rng))

    def __str__(self):
        """``{string: probability rounded to 3 decimals}`` (``core/noise.py:156-158``)."""
        return str({str(s): np.around(p, 3) for s, p in zip(self.strings, self.probs)})


class PauliLindbladNoise(Noise):
    def __init__(self, strings, lindblad_coefficients, dense=True):
        self.strings = strings
        self.lindblad_coefficients = lindblad_coefficients
        self.rates = [0.5 * (1 - np.exp(-2 * lam)) for lam in lindblad_coefficients]
        self.num_sites = len(strings[0])
        self.local_dim = 2
        self.gamma = np.exp(2 * sum(lindblad_coefficients))
        self.superop = self.make_superop() if dense else None

    def get_kraus_for_string(self, i):
        d = 2 ** self.num_sites
        return [np.emath.sqrt(1 - self.rates[i]) * np.eye(d),
                np.emath.sqrt(self.rates[i]) * _embed_dense(self.strings[i])]

    def get_superop_for_string(self, i):
        """sum_k conj(K) (x) K over the two Kraus operators of generator i (``core/noise.py:183-185``)."""
        return sum(np.kron(np.conj(k), k) for k in self.get_kraus_for_string(i))

    def make_superop(self):
        """Product of the generators' superoperators (``core/noise.py:187-189``)."""
        ops = [self.get_superop_for_string(i) for i in range(len(self.strings))]
        return np.linalg.multi_dot(ops) if len(ops) > 1 else ops[0]

    def get_superop(self, *args, **kwargs):
        return self.superop

    def get_kraus(self, *args, **kwargs):
        raise NotImplementedError("PauliLindbladNoise is defined by its superoperator")

    def sample_string(self, rng=None):
        """Each generator fires independently with its rate; the fired strings
        multiply (phases dropped) (``core/noise.py:194-200``)."""
        rng = np.random.default_rng() if rng is None else rng
        flags = [rng.random() < r for r in self.rates]
        out = 'i' * self.num_sites
        for s, f in zip(self.strings, flags):
            if f:
                out, _ = pauli_multiply(out, s)
        return out

    def sample(self, rng=None):
        return pauli_string_to_gates(self.sample_string(rng))

    def inv_sample(self, rng=None):
        """A layer of the inverse channel and its quasi-probability prefactor
        gamma * (-1)^(layer non-empty) (``core/noise.py:206-210``)."""
        layer = self.sample(rng)
        return layer, self.gamma * (-1) ** (len(layer) != 0)


def random_pauli_channel(n, n_strings=5, c=0.1):
    """Pauli channel on n sites: the identity with weight 1 and n_strings - 1
    random strings with weights c * U[0, 1), normalised, from NumPy's global
    random state (``core/noise.py:232-236``)."""
    from .paulis import random_pauli_string
    strings = ['i' * n] + [random_pauli_string(n) for _ in range(n_strings - 1)]
    probs = np.array([1.0] + [c * np.random.rand() for _ in range(n_strings - 1)])
    return PauliNoise(strings, probs / np.sum(probs))


def depolarizing(p):
    """Single-qubit depolarising channel with the p/3 convention."""
    return PauliNoise(['i', 'x', 'y', 'z'], [1 - p, p / 3, p / 3, p / 3])


class AmplitudeDamping(Noise):
    """``K0 = diag(1, sqrt(1-gamma))``, ``K1 = sqrt(gamma)|0><1|``."""

    def __init__(self, gamma):
        self.gamma = float(gamma)
        self.num_sites = 1
        self.local_dim = 2

    def get_kraus(self, *args, **kwargs):
        g = self.gamma
        return [np.array([[1, 0], [0, np.sqrt(1 - g)]], dtype=complex),
                np.array([[0, np.sqrt(g)], [0, 0]], dtype=complex)]


def amplitude_damping(gamma):
    return AmplitudeDamping(gamma)


def gate_time(gate, nm):
    if gate.time is not None:
        return gate.time
    if gate.name[0:4] == "CNOT":
        return nm.two_site_time
    if gate.name[0:2] in ("RZ", "SW"):
        return 0.0
    if gate.name[0:2] == "CU":
        return 4 * nm.two_site_time
    if gate.span == 1:
        return nm.one_site_time
    if gate.span == 2:
        return nm.two_site_time
    raise ValueError("Gate span > 2 not supported for automatic timing.")
