"""Pauli algebra for the expectation kernels.

Mirrors ``core/paulis.py`` of the reference (Pauli matrices ``:5-9``,
``pauli_commute`` ``:11-18``, ``pauli_multiply`` ``:20-47``, ``pauli_strings``
``:49-51``, ``simple_pstr`` ``:91-113``) and adds the bit-mask form the CUDA
kernels consume.

Pauli strings are lower-case ``'ixyz'`` strings, character ``q`` acting on
site ``q``. Site ``q`` is bit ``n-1-q`` of a flat amplitude index (site 0 is
the most-significant axis of the reference's ``reshape([2]*n)`` state,
``tensorQ/statevector_sim.py:36,47``).
"""
from __future__ import annotations

import itertools
import re

import numpy as np

pauli_I = np.array([[1, 0], [0, 1]], dtype=complex)
pauli_X = np.array([[0, 1], [1, 0]], dtype=complex)
pauli_Y = np.array([[0, -1.j], [1.j, 0]], dtype=complex)
pauli_Z = np.array([[1, 0], [0, -1]], dtype=complex)
pauli_mapping = {'i': pauli_I, 'x': pauli_X, 'y': pauli_Y, 'z': pauli_Z}


def pauli_commute(p1: str, p2: str) -> bool:
    anti = sum(1 for a, b in zip(p1, p2) if a != 'i' and b != 'i' and a != b)
    return anti % 2 == 0


_MUL = {  # (a, b) -> (product, phase) for single-site Paulis, a*b
    ('x', 'y'): ('z', 1j), ('y', 'z'): ('x', 1j), ('z', 'x'): ('y', 1j),
    ('y', 'x'): ('z', -1j), ('z', 'y'): ('x', -1j), ('x', 'z'): ('y', -1j),
}


def pauli_multiply(p1: str, p2: str):
    out, phase = [], 1
    for a, b in zip(p1, p2):
        if a == 'i':
            out.append(b)
        elif b == 'i':
            out.append(a)
        elif a == b:
            out.append('i')
        else:
            c, ph = _MUL[(a, b)]
            out.append(c)
            phase *= ph
    return ''.join(out), phase


def pauli_strings(n: int):
    return [''.join(p) for p in itertools.product('ixyz', repeat=n)]


def simple_pstr(spec: str, n: int, base: int = 0) -> str:
    chars = ['i'] * n
    pos = 0
    for m in re.finditer(r'([ixyzIXYZ])(\d+)', spec):
        if m.start() != pos:
            raise ValueError(f"Unparsed chunk in spec at {pos}: {spec[pos:m.start()]!r}")
        p, idx = m.group(1).lower(), int(m.group(2)) - base
        if not 0 <= idx < n:
            raise IndexError(f"site {idx + base} out of bounds for n={n} with base={base}")
        if chars[idx] != 'i':
            raise ValueError(f"duplicate assignment to site {idx + base}")
        chars[idx] = p
        pos = m.end()
    if pos != len(spec):
        raise ValueError(f"Trailing garbage in spec: {spec[pos:]!r}")
    return ''.join(chars)


def pauli_masks(pstr: str):
    """Return ``(xmask, zmask, n_y)`` of a Pauli string in flat-bit order.

    ``P|x> = i^{n_y} (-1)^{popcount(x & zmask)} |x ^ xmask>``.
    """
    n = len(pstr)
    xm = zm = 0
    ny = 0
    for q, c in enumerate(pstr.lower()):
        b = 1 << (n - 1 - q)
        if c == 'x':
            xm |= b
        elif c == 'y':
            xm |= b
            zm |= b
            ny += 1
        elif c == 'z':
            zm |= b
        elif c != 'i':
            raise ValueError(f"invalid Pauli character {c!r} in {pstr!r}")
    return xm, zm, ny


def random_pauli_string(n):
    """n characters from 'ixyz', each drawn with ``numpy.random.choice(4)`` from
    NumPy's global random state (``core/paulis.py:53-58``)."""
    chars = 'ixyz'
    return ''.join(chars[np.random.choice(len(chars))] for _ in range(n))
