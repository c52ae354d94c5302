"""Circuit container and builders.

Host-side mirror of ``core/circuits.py`` (``Circuit`` ``:8-170``,
``compose_circuits`` ``:172-175``, ``circ_to_mat`` ``:177-192``,
``two_local_circ`` ``:206-217``, rotation layers ``:219-251``) and of the
skeleton helpers in ``core/skeletons.py`` (``nn_edges`` ``:30-47``,
``brickwall_skeleton`` ``:49-64``). Layering is the reference's greedy
as-soon-as-possible placement; it keeps per-qubit gate order, which is all the
simulators rely on.
"""
from __future__ import annotations

import copy
from functools import reduce

import numpy as np

from .gates import ID, Gate, SuperOp, random_unitary, kak_unitary, RX, RY, RZ, RXX, RYY, RZZ, HeisenbergCoupling


class Circuit:
    def __init__(self, gate_list, n=None, local_dim=2, meas_sites=None, requires_decomp=False):
        self.gate_list = list(gate_list)
        if len(self.gate_list) != 0:
            if n is None:
                n = int(max(max(g.indices) for g in self.gate_list) + 1)
            self.num_sites = n
            self.local_dim = self.gate_list[0].get_local_dim()
        else:
            self.num_sites = n
            self.local_dim = local_dim
        self.layers = None
        self.built = False
        self.meas_sites = meas_sites
        self.requires_decomp = requires_decomp

    def update_gate(self, gate_idx, new_array):
        self.gate_list[gate_idx].matrix = new_array
        if self.layers is not None:
            self.construct_layers()

    def decompose(self, basis='ZSX'):
        out = []
        for g in self.gate_list:
            if g.name == "U" and getattr(g, "angles", None) is not None and hasattr(g, "decompose"):
                out.extend(g.decompose(basis))
            else:
                out.append(g)
        self.gate_list = out

    def construct_layers(self):
        """Greedy ASAP layering (``core/circuits.py:42-63``)."""
        layers, occupied = [], []
        for g in self.gate_list:
            gi = set(g.indices)
            li = len(layers) - 1
            while li >= 0 and not (gi & occupied[li]):
                li -= 1
            if li < len(layers) - 1:
                layers[li + 1].append(g)
                occupied[li + 1] |= gi
            else:
                layers.append([g])
                occupied.append(set(gi))
        self.layers = layers

    def add_noise(self, nm):
        """Noise insertion (``core/circuits.py:65-84``)."""
        from .noise import ThermalNoise, gate_time
        layers = []
        for layer in self.layers:
            if any(isinstance(g, SuperOp) for g in layer):  # layers holding a superoperator stay noiseless
                layers.append(layer)
                continue
            if isinstance(nm, ThermalNoise):
                t = max(gate_time(g, nm) for g in layer)
                active = set(np.concatenate([g.indices for g in layer]))
                layer = layer + [ID(nm.local_dim, t, i, nm=nm, dd=(i not in active))
                                 for i in range(self.num_sites)]
            else:
                layer = layer + [ID(2, 0.0, list(range(self.num_sites)), nm=nm)]
            layers.append(layer)
        self.layers = layers

    def build(self, nm=None):
        if not self.built:
            if self.requires_decomp:
                self.decompose()
            self.construct_layers()
            if nm is not None:
                self.add_noise(nm)
            self.built = True
        return self

    def old_build(self, nm=None):
        """The reference's deprecated form of ``build`` (``core/circuits.py:97-107``):
        a deep copy, decomposed, layered and with noise; this circuit is left unchanged."""
        c = copy.deepcopy(self)
        c.decompose()
        c.construct_layers()
        if nm is not None:
            c.add_noise(nm)
        c.built = True
        return c

    def add_meas(self, meas_sites):
        self.meas_sites = meas_sites

    def draw(self):
        """Not drawn (the reference's ``draw`` returns None as well, ``core/circuits.py:159-161``)."""
        return None

    def dag(self):
        return Circuit([g.dag() for g in self.gate_list[::-1]], n=self.num_sites, local_dim=self.local_dim)

    def to_matrix(self):
        return circ_to_mat(self)

    def ops(self):
        """Flat op sequence in execution order (layers if built, else gate list)."""
        if self.layers is not None:
            return [op for layer in self.layers for op in layer]
        return list(self.gate_list)

    def __str__(self):
        if self.layers is not None:
            return " \n\n".join(" \n".join(str(g) for g in layer) for layer in self.layers)
        return " \n".join(str(g) for g in self.gate_list)

    def __getitem__(self, key):
        if isinstance(key, int):
            return self.gate_list[key]
        if isinstance(key, slice):
            return Circuit(self.gate_list[key], n=self.num_sites, local_dim=self.local_dim)
        raise TypeError("Invalid index type.")

    def __len__(self):
        return len(self.gate_list)

    def __add__(self, other):
        return compose_circuits([self, other])

    def __mul__(self, other):
        if isinstance(other, int) and other >= 0:
            if other == 0:
                return Circuit([], n=self.num_sites, local_dim=self.local_dim)
            if other == 1:
                return self.copy()
            return compose_circuits([self] * other)
        raise TypeError("Circuit multiplication only supports non-negative integers")

    __rmul__ = __mul__

    def copy(self):
        c = Circuit([g.shallow_copy() for g in self.gate_list], n=self.num_sites,
                    local_dim=self.local_dim, meas_sites=self.meas_sites)
        if self.layers is not None:
            c.layers = [[g.shallow_copy() for g in layer] for layer in self.layers]
        c.built = self.built
        return c


def shift_gate_list(circ, start_site):
    """Deep copies of the circuit's gates with every site index moved by
    ``start_site`` (``core/circuits.py:194-204``)."""
    out = []
    for g in circ.gate_list:
        h = copy.deepcopy(g)
        h.indices = np.array(g.indices) + start_site
        out.append(h)
    return out


def compose_circuits(circ_list):
    gl = [g for c in circ_list for g in c.gate_list]
    return Circuit(gl, n=int(np.max([c.num_sites for c in circ_list])))


def circ_to_mat(circ, n=None):
    """Dense unitary by Kronecker products per layer (``core/circuits.py:177-192``)."""
    if circ.layers is None:
        circ.construct_layers()
    n = circ.num_sites if n is None else n
    mats = []
    for layer in circ.layers:
        layer = list(layer)
        missing = set(range(n)) - set(np.concatenate([g.indices for g in layer]))
        for i in missing:
            layer.append(ID(circ.local_dim, 0.0, [i], None))
        layer.sort(key=lambda g: g.indices[0])
        mats.append(reduce(np.kron, [np.asarray(g.matrix) for g in layer]))
    return np.linalg.multi_dot(mats[::-1]) if len(mats) > 1 else mats[0]


def nn_edges(Lx, Ly=1):
    edges = []
    for row in range(Ly):
        for col in range(Lx):
            idx = row * Lx + col
            if col < Lx - 1:
                edges.append((idx, idx + 1))
            if row < Ly - 1:
                edges.append((idx, idx + Lx))
    return edges


def brickwall_skeleton(Lx, Ly=1, depth=1):
    """Even horizontal, odd horizontal, even vertical, odd vertical edges
    (``core/skeletons.py:49-64``)."""
    edges = nn_edges(Lx, Ly)
    h = [e for e in edges if abs(e[0] - e[1]) == 1]
    v = [e for e in edges if abs(e[0] - e[1]) != 1]
    sk = [e for e in h if e[0] % 2 == 0] + [e for e in h if e[0] % 2 != 0]
    sk += [e for e in v if (e[0] // Lx) % 2 == 0] + [e for e in v if (e[0] // Lx) % 2 != 0]
    return sk * depth


def two_local_circ(skeleton, params=None, mag=None):
    gl = []
    for i, idx in enumerate(skeleton):
        if mag is None and params is None:
            mat = random_unitary(4)
        elif params is not None:
            mat = kak_unitary(params[15 * i:15 * (i + 1)])
        else:
            mat = kak_unitary(np.random.rand(15) * mag)
        gl.append(Gate("rand_U", list(idx), mat))
    return Circuit(gl)


def _layer(cls, sites, params, n_default):
    params = np.random.rand(n_default) * np.pi if params is None else params
    return Circuit([cls(s, params[i]) for i, s in enumerate(sites)])


def rx_layer(n, params=None):
    return _layer(RX, [[i] for i in range(n)], params, n)


def ry_layer(n, params=None):
    return _layer(RY, [[i] for i in range(n)], params, n)


def rz_layer(n, params=None):
    return _layer(RZ, [[i] for i in range(n)], params, n)


def rxx_layer(skeleton, params=None):
    return _layer(RXX, [list(e) for e in skeleton], params, len(skeleton))


def ryy_layer(skeleton, params=None):
    return _layer(RYY, [list(e) for e in skeleton], params, len(skeleton))


def rzz_layer(skeleton, params=None):
    return _layer(RZZ, [list(e) for e in skeleton], params, len(skeleton))


def heisenberg_layer(skeleton, params=None):
    return _layer(HeisenbergCoupling, [list(e) for e in skeleton], params, len(skeleton))
