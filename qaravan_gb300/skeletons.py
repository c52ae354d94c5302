"""Lattice skeletons: the edge lists circuits are built on (host mirror of
``core/skeletons.py:7-127``). Sites are numbered row-major, site = y * Lx + x."""
from __future__ import annotations

from itertools import product

import numpy as np

from .circuits import brickwall_skeleton, nn_edges

__all__ = ["index_from_coords", "coords_from_index", "horiz_filter", "even_filter", "nn_edges", "brickwall_skeleton",
           "even_skeleton", "odd_skeleton", "dress_skeleton", "all_skeletons"]


def index_from_coords(x, y, Lx):
    return y * Lx + x


def coords_from_index(idx, Lx):
    row, col = divmod(idx, Lx)
    return col, row


def horiz_filter(edge):
    """A horizontal edge joins consecutive sites."""
    return abs(edge[0] - edge[1]) == 1


def even_filter(edge, vert=False, Lx=0):
    """Horizontal edges: even first site; vertical edges: even row of the first site."""
    if not vert:
        return edge[0] % 2 == 0
    assert Lx > 0, "Lx must be provided for even filter on vertical edges"
    return coords_from_index(edge[0], Lx)[1] % 2 == 0


def _split(Lx, Ly, keep_even):
    edges = nn_edges(Lx, Ly)
    h = [e for e in edges if horiz_filter(e) and even_filter(e, vert=False, Lx=Lx) == keep_even]
    v = [e for e in edges if not horiz_filter(e) and even_filter(e, vert=True, Lx=Lx) == keep_even]
    return h + v


def even_skeleton(Lx, Ly=1, depth=1):
    """Even horizontal then even vertical edges, ``depth`` times."""
    return _split(Lx, Ly, True) * depth


def odd_skeleton(Lx, Ly=1, depth=1):
    """Odd horizontal then odd vertical edges, ``depth`` times."""
    return _split(Lx, Ly, False) * depth


def dress_skeleton(skeleton, gate_type, params=None):
    """One ``gate_type`` per edge: no parameter, one shared, or one per edge."""
    if params is not None and not isinstance(params, (list, tuple, np.ndarray)):
        params = [params] * len(skeleton)
    return [gate_type(e, params[i]) if params is not None else gate_type(e) for i, e in enumerate(skeleton)]


def all_skeletons(num_gates, Lx, Ly=1, orientation=False, a2a=False):
    """Every sequence of ``num_gates`` edges (nearest-neighbour or all-to-all
    pairs; with ``orientation`` both directions of each)."""
    pairs = nn_edges(Lx, Ly) if not a2a else [(i, j) for i in range(Lx * Ly) for j in range(Lx * Ly) if i != j]
    if orientation:
        pairs = pairs + [p[::-1] for p in pairs]
    return list(product(pairs, repeat=num_gates))
