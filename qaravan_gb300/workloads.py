"""Seeded synthetic workloads: Haar brickwork, TFI Trotter, hardware-efficient ansatz.

The reference publishes no dataset; these generators build its benchmark
circuit families from a ``numpy.random.default_rng(seed)`` stream so every run
(and the oracle) sees the same gates.

* Haar SU(d): QR of a complex Ginibre matrix with the phase of ``diag(R)``
  divided out (Mezzadri, "How to generate random matrices from the classical
  compact groups", 2007), then divided by ``det^(1/d)``. The reference's own
  ``random_unitary`` helpers are not Haar (``core/gates.py:289-293`` uses the
  eigenvectors of ``a a^dagger``), so gates are generated here and wrapped as
  ``Gate("rand_U", idx, M)`` the way ``two_local_circ`` does
  (``core/circuits.py:206-217``).
* Brickwork depth unit: Haar SU(2) on every site, then Haar SU(4) on the even
  pairs and then the odd pairs of ``brickwall_skeleton(n)``
  (``core/skeletons.py:49-64``). Depth 20 on 12 sites is 240 + 220 = 460 gates;
  on 28 sites it is 560 + 540 = 1100 gates.
* TFI Trotter: ``TFI(n, jz, h).trotter_circ(dt, steps)``.
* Hardware-efficient ansatz: per layer ``RY(theta)`` and ``RZ(phi)`` on every
  qubit, then ``CNOT([q+1, q])`` (target q+1, control q) for q = 0..n-2.
"""
from __future__ import annotations

import numpy as np

from .circuits import Circuit, brickwall_skeleton
from .gates import Gate, RY, RZ, CNOT
from .hamiltonians import TFI


def haar_unitary(d, rng):
    z = (rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d))) / np.sqrt(2.0)
    q, r = np.linalg.qr(z)
    ph = np.diag(r) / np.abs(np.diag(r))
    q = q * ph[None, :]
    det = np.linalg.det(q)
    return q / det ** (1.0 / d)


def brickwork_gates(n, depth, seed):
    """Gate list of the seeded Haar brickwork (one SU(2) layer + even + odd SU(4) per depth unit)."""
    rng = np.random.default_rng(seed)
    sk = brickwall_skeleton(n, 1, 1)
    gl = []
    for _ in range(depth):
        for q in range(n):
            gl.append(Gate("rand_U", [q], haar_unitary(2, rng)))
        for e in sk:
            gl.append(Gate("rand_U", list(e), haar_unitary(4, rng)))
    return gl


def brickwork_circuit(n, depth, seed):
    return Circuit(brickwork_gates(n, depth, seed), n=n)


def tfi_trotter_circuit(n, dt=0.05, steps=40, jz=1.0, h=1.0):
    return TFI(n, jz=jz, h=h).trotter_circ(dt, steps)


def hea_params(n, layers, seed):
    rng = np.random.default_rng(seed)
    return rng.uniform(0.0, 2 * np.pi, size=(layers, n, 2))


def hea_circuit(n, layers, params):
    """``params[l, q] = (theta, phi)``; NumPy floats or a torch tensor (keeps autograd)."""
    gl = []
    for l in range(layers):
        for q in range(n):
            gl.append(RY([q], params[l][q][0]))
            gl.append(RZ([q], params[l][q][1]))
        for q in range(n - 1):
            gl.append(CNOT([q + 1, q], n))
    return Circuit(gl, n=n)


def noisy_brickwork_circuit(n, depth, seed, p=1e-3):
    """Haar brickwork with a single-qubit depolarising channel (``PauliNoise`` with the
    p/3 convention) on both sites after every two-qubit gate, as explicit ``ID``
    noise carriers in a built layer list (one op per layer, the order the
    density-matrix oracle applies them)."""
    from .gates import ID
    from .noise import depolarizing
    gl = brickwork_gates(n, depth, seed)
    dep = depolarizing(p)
    seq = []
    for g in gl:
        seq.append(g)
        if len(g.indices) == 2:
            seq.extend(ID(2, 0.0, [q], nm=dep) for q in g.indices)
    c = Circuit(gl, n=n)
    c.layers = [[g] for g in seq]
    c.built = True
    return c


def uneven_dm_specs(count, seed, n_range=(6, 14), depth_range=(10, 40)):
    """(n, depth, circuit seed) triples for the uneven density-matrix batch."""
    rng = np.random.default_rng(seed)
    ns = rng.integers(n_range[0], n_range[1] + 1, size=count)
    ds = rng.integers(depth_range[0], depth_range[1] + 1, size=count)
    seeds = rng.integers(0, 2 ** 31 - 1, size=count)
    return [(int(a), int(b), int(c)) for a, b, c in zip(ns, ds, seeds)]
