"""Circuit compiler: gate fusion and tile-sweep planning.

The reference applies gates one at a time, layer by layer (``BaseSim.run``,
``core/base_sim.py:30-53``), each as a full contraction over the state
(``op_action``, ``tensorQ/statevector_sim.py:124-140``). This compiler turns
the same op sequence into fewer passes over HBM:

1. **Fusion** (``fuse``): ops are merged into dense blocks of at most ``width``
   bits. An op joins the latest block it depends on when the union of their
   bits stays within ``width`` (it commutes past every later block, which by
   construction shares no bit with it); earlier blocks whose bits are covered
   and that nothing in between touches are then absorbed too, which folds
   single-qubit layers into the neighbouring two-qubit gates. Matrices are
   composed on the host in complex128 (``fuse``) or, with
   ``device_fusion=True``, only the block membership is decided on the host
   (``fuse_symbolic``, same decisions) and the products run on the GPU
   (``qgb_fuse_blocks``) from the raw op matrices.
2. **Sweep planning** (``plan_sweeps``): consecutive blocks are grouped into
   sweeps whose bits fit one shared-memory tile (the low ``L`` flat bits plus up
   to ``H`` chosen high bits). A block is skipped -- and every later block
   touching its bits with it -- when the tile cannot take its bits, so blocks
   only move past blocks they commute with.

Ops are ``(bits, matrix)`` with flat bit positions in matrix order (bit
``bits[j]`` is matrix-index bit ``k-1-j``); for a statevector of ``n`` qubits,
site ``q`` is bit ``n-1-q``.
"""
from __future__ import annotations

import functools
from dataclasses import dataclass, field

import numpy as np

from ._lib import QGB_SWEEP_MAX_HIGH, QGB_SWEEP_MAX_OPS, QGB_SWEEP_MAX_TILE_BITS


@dataclass
class Op:
    bits: list
    matrix: np.ndarray  # complex128, 2^k x 2^k
    kind: str = "unitary"  # "unitary" | "nonunitary" | "channel" | "pauli_mix"
    terms: list = None  # "pauli_mix": [(coeff, Pauli string over the vector's bits, char j <-> bit nbits-1-j)]
    pair: int = None  # density matrices: id shared by the ket and bra halves of one gate (None otherwise)


@dataclass
class DenseStep:
    bits: list
    mat: int  # index into the plan's matrix list
    unitary: bool = False  # the block is unitary (every op in it is): its launch may restore group norms
    whole: bool = False  # density matrices: the ops applied up to this step form whole channels (no half gate)


@dataclass
class SweepStep:
    low_bits: int
    high_bits: list
    ops: list  # (tile-local positions in matrix order, matrix index)


@dataclass
class TcSweepStep:
    """Up to four 5-qubit blocks applied to each 8192-amplitude tile (the low
    ``low_bits`` flat bits times ``high_bits``) in one pass on the tensor cores."""
    low_bits: int
    high_bits: list
    blocks: list  # (tile positions of the block's five bits in matrix order, matrix index)
    unitary: bool = False  # every block is unitary: the pass may join the norm chain


@dataclass
class NormalizeStep:
    pass


@dataclass
class PauliMixStep:
    """v <- sum_t coeff_t P_t v over the whole vector (a Pauli channel on vec(rho)
    wider than a dense block: rho -> sum_k p_k P_k rho P_k^dagger)."""
    terms: list


@dataclass
class Recipe:
    """A fused block to be composed on the device: its bits (matrix order) and
    the ops applied to it, first applied first, as (op matrix index into
    ``Plan.op_matrices``, op bits in the op's matrix order)."""
    bits: list
    entries: list


@dataclass
class Plan:
    nbits: int
    steps: list = field(default_factory=list)
    matrices: list = field(default_factory=list)  # complex128 arrays (host-composed), or Recipe objects
    n_gates: int = 0  # original op count
    op_matrices: list = field(default_factory=list)  # raw op matrices the recipes refer to
    trace_kept: bool = False  # density matrices: every op keeps the trace, or a renormalisation follows it

    def add_matrix(self, m):
        if isinstance(m, Recipe):
            self.matrices.append(m)
        else:
            self.matrices.append(np.ascontiguousarray(m, dtype=np.complex128))
        return len(self.matrices) - 1

    @property
    def device_fused(self):
        return any(isinstance(m, Recipe) for m in self.matrices)

    def matrix_dim(self, i):
        m = self.matrices[i]
        return 2 ** len(m.bits) if isinstance(m, Recipe) else m.shape[0]

    @property
    def n_sweeps(self):
        return sum(1 for s in self.steps if isinstance(s, (DenseStep, SweepStep, TcSweepStep)))


# ----------------------------------------------------------------- algebra

@functools.lru_cache(maxsize=4096)
def _embed_index(bits, target):
    """Index maps of ``embed``: (row/col sub-index into the small matrix, same-rest mask)."""
    K, k = len(target), len(bits)
    pos = [target.index(b) for b in bits]  # position j in target order (0 = MSB)
    idx = np.arange(2 ** K)
    sub = np.zeros(2 ** K, dtype=np.int64)
    for j, p in enumerate(pos):
        sub |= ((idx >> (K - 1 - p)) & 1) << (k - 1 - j)
    other_mask = 0
    for p in range(K):
        if p not in pos:
            other_mask |= 1 << (K - 1 - p)
    rest = idx & other_mask
    return sub[:, None], sub[None, :], rest[:, None] == rest[None, :]


def embed(mat, bits, target):
    """Matrix of ``mat`` (acting on ``bits``) on the larger bit list ``target``."""
    bits, target = tuple(bits), tuple(target)
    if bits == target:
        return np.asarray(mat, dtype=np.complex128)
    rows, cols, same = _embed_index(bits, target)
    return np.where(same, np.asarray(mat, dtype=np.complex128)[rows, cols], 0)


def _union(a, b):
    out = list(a)
    for x in b:
        if x not in out:
            out.append(x)
    return out


# ------------------------------------------------------------------ fusion

@dataclass
class Block:
    bits: list
    matrix: np.ndarray
    n_ops: int = 1


def fuse(ops, width):
    """Greedy order-preserving fusion into blocks of at most ``width`` bits."""
    blocks: list = []
    last: dict = {}  # bit -> index of the latest block touching it
    for op in ops:
        bits = list(op.bits)
        if len(bits) > width:
            raise ValueError(f"op on {len(bits)} bits exceeds fusion width {width}")
        deps = [last[b] for b in bits if b in last]
        cand = max(deps) if deps else None
        if cand is not None and blocks[cand] is not None and len(_union(blocks[cand].bits, bits)) <= width:
            blk = blocks[cand]
            u = sorted(_union(blk.bits, bits), reverse=True)
            blk.matrix = embed(op.matrix, bits, u) @ embed(blk.matrix, blk.bits, u)
            blk.bits = u
            blk.n_ops += 1
            for b in bits:
                last[b] = cand
            # absorb earlier blocks covered by the union with nothing in between touching them
            for j in sorted({d for d in deps if d != cand}, reverse=True):
                bj = blocks[j]
                if bj is None or not set(bj.bits) <= set(u):
                    continue
                if any(blocks[i] is not None and set(blocks[i].bits) & set(bj.bits) for i in range(j + 1, cand)):
                    continue
                blk.matrix = blk.matrix @ embed(bj.matrix, bj.bits, u)
                blk.n_ops += bj.n_ops
                blocks[j] = None
                for b in bj.bits:
                    if last.get(b) == j:
                        last[b] = cand
            continue
        blocks.append(Block(sorted(bits, reverse=True) if len(bits) > 1 else list(bits),
                            embed(op.matrix, bits, sorted(bits, reverse=True)), 1))
        for b in bits:
            last[b] = len(blocks) - 1
    return [b for b in blocks if b is not None]


@dataclass
class SymBlock:
    bits: list
    ops: list  # indices into the fused op list, first applied first

    @property
    def n_ops(self):
        return len(self.ops)


def fuse_symbolic(ops, width):
    """The decisions of :func:`fuse` without the matrix products: blocks of at
    most ``width`` bits, each with the indices of its ops in application order
    (an absorbed earlier block's ops go in front: it is applied first)."""
    blocks: list = []
    last: dict = {}
    for oi, op in enumerate(ops):
        bits = list(op.bits)
        if len(bits) > width:
            raise ValueError(f"op on {len(bits)} bits exceeds fusion width {width}")
        deps = [last[b] for b in bits if b in last]
        cand = max(deps) if deps else None
        if cand is not None and blocks[cand] is not None and len(_union(blocks[cand].bits, bits)) <= width:
            blk = blocks[cand]
            u = sorted(_union(blk.bits, bits), reverse=True)
            blk.ops.append(oi)
            blk.bits = u
            for b in bits:
                last[b] = cand
            for j in sorted({d for d in deps if d != cand}, reverse=True):
                bj = blocks[j]
                if bj is None or not set(bj.bits) <= set(u):
                    continue
                if any(blocks[i] is not None and set(blocks[i].bits) & set(bj.bits) for i in range(j + 1, cand)):
                    continue
                blk.ops = bj.ops + blk.ops
                blocks[j] = None
                for b in bj.bits:
                    if last.get(b) == j:
                        last[b] = cand
            continue
        blocks.append(SymBlock(sorted(bits, reverse=True) if len(bits) > 1 else list(bits), [oi]))
        for b in bits:
            last[b] = len(blocks) - 1
    return [b for b in blocks if b is not None]


def recipe_matrix(recipe, op_matrices):
    """Host (complex128) composition of a :class:`Recipe` -- what the device
    computes; used to check the device kernel and the symbolic fusion."""
    m = np.eye(2 ** len(recipe.bits), dtype=np.complex128)
    for mi, bits in recipe.entries:
        m = embed(op_matrices[mi], bits, recipe.bits) @ m
    return m


# --------------------------------------------------------- sweep planning

def plan_sweeps(blocks, nbits, tile_bits, low_bits=None, max_high=QGB_SWEEP_MAX_HIGH, max_ops=QGB_SWEEP_MAX_OPS):
    """Group blocks into tile sweeps of at most ``max_ops`` blocks; returns a
    list of (low_bits, high_bits, [blocks])."""
    m = min(tile_bits, nbits, QGB_SWEEP_MAX_TILE_BITS)
    L = min(5 if low_bits is None else low_bits, m)
    if m == nbits:
        L = nbits
    H = m - L
    if H > max_high:
        H = max_high
        L = m - H
    widest = max((len(b.bits) for b in blocks), default=1)
    if m < nbits and H < widest:  # the tile must take any single block's bits
        H = min(widest, max_high, m - 1)
        L = m - H
    remaining = list(blocks)
    sweeps = []
    while remaining:
        high: list = []
        taken, rest = [], []
        blocked: set = set()
        for j, blk in enumerate(remaining):
            if len(blocked) >= nbits:  # every later block overlaps a skipped one: keep the rest in order
                rest.extend(remaining[j:])
                break
            bset = set(blk.bits)
            if bset & blocked or len(taken) >= max_ops:
                blocked |= bset
                rest.append(blk)
                continue
            need = [b for b in blk.bits if b >= L and b not in high]
            if len(high) + len(need) <= H:
                high.extend(need)
                taken.append(blk)
            else:
                blocked |= bset
                rest.append(blk)
        if not taken:
            raise RuntimeError("sweep planner made no progress (block wider than the tile)")
        # pad the tile to its full size with unused bits (more work per CTA, same traffic)
        for b in range(L, nbits):
            if len(high) >= H:
                break
            if b not in high:
                high.append(b)
        sweeps.append((L, sorted(high), taken))
        remaining = rest
    return sweeps


# ------------------------------------------------------------------- plans

def unitary_flags(ops, tol=1e-6):
    """Whether each op's matrix is unitary (max |M^H M - I| < tol), batched by size."""
    flags = [False] * len(ops)
    by_dim: dict = {}
    for i, o in enumerate(ops):
        m = np.asarray(o.matrix)
        by_dim.setdefault(m.shape[0], []).append(i)
    for d, idx in by_dim.items():
        m = np.stack([np.asarray(ops[i].matrix, dtype=np.complex128) for i in idx])
        gram = np.matmul(m.conj().transpose(0, 2, 1), m)
        gram[:, np.arange(d), np.arange(d)] -= 1
        err = np.abs(gram).reshape(len(idx), -1).max(axis=1)
        for i, e in zip(idx, err.tolist()):
            flags[i] = e < tol
    return flags


def trace_preserving(op):
    """Whether an op on vec(rho) keeps Tr rho for every rho: a half of a unitary
    gate (unitary on its bits; the other half is its conjugate) or a channel
    superoperator on 2k bits (bra bits first) whose rows with equal bra and ket
    index sum to the trace functional."""
    m = np.asarray(op.matrix, dtype=np.complex128)
    if op.pair is not None:
        return unitary_flags([op])[0]
    if op.kind != "channel":
        return False
    k2 = len(op.bits)
    k = k2 // 2
    d = 2 ** k
    diag = [(a << k) | a for a in range(d)]
    t = m[diag, :].sum(axis=0)
    want = np.zeros(4 ** k, dtype=np.complex128)
    want[diag] = 1.0
    return bool(np.abs(t - want).max() < 1e-9)


def whole_cuts(seg, groups):
    """For each group of segment op indices (in application order): whether the
    ops applied up to and including it leave no gate with only one of its
    halves (ket or bra) applied. At such a cut the ops applied so far are whole
    channels, which keep the trace."""
    open_pairs: set = set()
    out = []
    for g in groups:
        for i in g:
            p = seg[i].pair
            if p is not None:
                open_pairs ^= {p}
        out.append(not open_pairs)
    return out


def _pair_offsets(ops):
    """Offset from each op to the other half of its pair (0 when unpaired): the
    pairing structure, independent of the ids."""
    first: dict = {}
    out = [0] * len(ops)
    for i, o in enumerate(ops):
        if o is None or o.pair is None:
            continue
        if o.pair in first:
            j = first.pop(o.pair)
            out[i], out[j] = j - i, i - j
        else:
            first[o.pair] = i
    return out


# Plans whose block matrices are all device-composed (Recipe) depend on the op
# matrices only through the unitarity flags: such a plan is kept per structure
# (op bits, flags, options) and reused with new op matrices, so a circuit run
# again with other values (a variational loop, the same circuit rebuilt) skips
# the fusion planner. Bounded, least recently used first out.
_PLAN_CACHE: "dict" = {}
_PLAN_CACHE_SIZE = 32


def _cached_plan(key, ops):
    tpl = _PLAN_CACHE.pop(key, None)
    if tpl is None:
        return None
    _PLAN_CACHE[key] = tpl  # most recently used last
    plan = Plan(nbits=tpl.nbits, steps=tpl.steps, matrices=tpl.matrices, n_gates=tpl.n_gates,
                trace_kept=tpl.trace_kept)
    plan.op_matrices = [np.ascontiguousarray(o.matrix, dtype=np.complex128) for o in ops if o is not None]
    return plan


def _remember_plan(key, plan):
    if plan.matrices and all(isinstance(m, Recipe) for m in plan.matrices):
        _PLAN_CACHE[key] = plan
        while len(_PLAN_CACHE) > _PLAN_CACHE_SIZE:
            _PLAN_CACHE.pop(next(iter(_PLAN_CACHE)))


def compile_ops(ops, nbits, mode="sweep", width=2, tile_bits=13, low_bits=None, max_sweep_k=5, itemsize=8,
                device_fusion=False):
    """Compile an op sequence (with ``None`` marking a renormalisation point)
    into a :class:`Plan`.

    ``mode``: ``"gate"`` one pass per op; ``"fused"`` one pass per fused block of
    ``width`` bits; ``"sweep"`` fused blocks grouped into shared-memory tile sweeps;
    ``"tcsweep"`` 5-qubit blocks, up to four per pass, on the tensor cores
    (statevectors of at least 14 qubits; otherwise as ``"fused"``).
    ``itemsize`` (8 for complex64, 16 for complex128) caps the tile at 128 KiB
    of shared memory. ``device_fusion``: block matrices are left as
    :class:`Recipe` objects for the executor to compose on the GPU.
    """
    tile_bits = min(tile_bits, 14 if itemsize <= 8 else 13)
    # unitarity of every op with a matrix, batched once (the plan key, trace checks and fusion use it)
    mops = [o for o in ops if o is not None and o.kind != "pauli_mix"]
    ucache = dict(zip(map(id, mops), unitary_flags(mops))) if mops else {}
    # density matrices: does every op keep the trace, or is it followed by a renormalisation?
    dm = any(o is not None and (o.pair is not None or o.kind == "channel") for o in ops)
    trace_kept = False
    tp_flags = ()
    if dm:
        trace_kept = True
        pending_loss = False
        tp_list = []
        tpc: dict = {}  # channel ops sharing one superoperator array: checked once
        for o in ops:
            if o is None:
                pending_loss = False
                continue
            if o.kind == "pauli_mix":
                tp = True
            elif o.pair is not None:
                tp = ucache[id(o)]
            else:
                tp = tpc.get(id(o.matrix))
                if tp is None:
                    tp = tpc[id(o.matrix)] = trace_preserving(o)
            tp_list.append(tp)
            pending_loss |= not tp
        trace_kept = not pending_loss
        tp_flags = tuple(tp_list)
    key = None
    if device_fusion and mode != "gate" and ops and not any(o is not None and o.kind == "pauli_mix" for o in ops):
        flags = [ucache[id(o)] for o in ops if o is not None]
        key = (nbits, mode, width, tile_bits, low_bits, max_sweep_k, itemsize,
               tuple(None if o is None else tuple(o.bits) for o in ops), tuple(flags), tuple(_pair_offsets(ops)),
               tp_flags)
        plan = _cached_plan(key, ops)
        if plan is not None:
            return plan
    plan = Plan(nbits=nbits, n_gates=sum(1 for o in ops if o is not None), trace_kept=trace_kept)
    segments, cur = [], []
    for o in ops:
        if o is None or o.kind == "pauli_mix":
            segments.append(cur)
            segments.append(o)
            cur = []
        else:
            cur.append(o)
    segments.append(cur)
    for seg in segments:
        if seg is None:
            plan.steps.append(NormalizeStep())
            continue
        if isinstance(seg, Op):  # a Pauli mixture: its own pass
            plan.steps.append(PauliMixStep(list(seg.terms)))
            continue
        if not seg:
            continue
        uflags = [ucache[id(o)] for o in seg]
        if mode == "gate":
            for o, u, w_ in zip(seg, uflags, whole_cuts(seg, [[i] for i in range(len(seg))])):
                plan.steps.append(DenseStep(list(o.bits), plan.add_matrix(o.matrix), u, w_))
            continue
        # tensor-core tile sweeps: 5-qubit blocks, four at most per 13-bit tile, one state of >= 14
        # qubits; density-matrix segments keep the trace chain of the dense passes instead
        tcs = (mode == "tcsweep" and nbits >= 14 and max(len(o.bits) for o in seg) <= 5
               and not any(o.pair is not None or o.kind == "channel" for o in seg))
        w = 5 if tcs else max(width, max(len(o.bits) for o in seg))
        if device_fusion:
            base = len(plan.op_matrices)
            plan.op_matrices.extend(np.ascontiguousarray(o.matrix, dtype=np.complex128) for o in seg)
            sym = fuse_symbolic(seg, w)
            blocks = [Block(b.bits, Recipe(list(b.bits), [(base + i, list(seg[i].bits)) for i in b.ops]), b.n_ops)
                      for b in sym]
            bflags = [all(uflags[i] for i in b.ops) for b in sym]
            wflags = whole_cuts(seg, [b.ops for b in sym])
        else:
            blocks = fuse(seg, w)
            bflags = [bool(np.abs(b.matrix.conj().T @ b.matrix - np.eye(b.matrix.shape[0])).max() < 1e-6)
                      for b in blocks]
            wflags = [all(o.pair is None for o in seg)] * len(blocks)  # membership unknown here
        if tcs:
            _plan_tc_sweeps(plan, blocks, bflags, nbits, low_bits)
            continue
        if mode in ("fused", "tcsweep") or w > max_sweep_k or tile_bits <= 0:
            for b, u, w_ in zip(blocks, bflags, wflags):
                plan.steps.append(DenseStep(list(b.bits), plan.add_matrix(b.matrix), u, w_))
            continue
        for L, high, taken in plan_sweeps(blocks, nbits, tile_bits, low_bits):
            tpos = {b: b for b in range(L)}
            for h, b in enumerate(high):
                tpos[b] = L + h
            sops = [([tpos[b] for b in blk.bits], plan.add_matrix(blk.matrix)) for blk in taken]
            plan.steps.append(SweepStep(L, list(high), sops))
    if key is not None:
        _remember_plan(key, plan)
    return plan


TCS_MAX_BLOCKS = 4  # QGB_TCS_MAX_BLOCKS


def _plan_tc_sweeps(plan, blocks, bflags, nbits, low_bits=None):
    """Tensor-core tile sweeps of 13-bit tiles (low bits >= 4, runs of 128
    bytes) holding up to four blocks; every block is widened to exactly five
    tile bits (identity on the added ones, the lowest free tile bits first, so
    that tile bit 0 -- adjacent amplitudes -- is a target where possible)."""
    flag = {id(b): f for b, f in zip(blocks, bflags)}
    lb = 4 if low_bits is None else max(4, min(int(low_bits), 13))
    for L, high, taken in plan_sweeps(blocks, nbits, 13, lb, max_high=9, max_ops=TCS_MAX_BLOCKS):
        tpos = {b: b for b in range(L)}
        for h, b in enumerate(high):
            tpos[b] = L + h
        tile = sorted(tpos)
        entries = []
        for blk in taken:
            bits = list(blk.bits)
            full = bits + [b for b in tile if b not in bits][:5 - len(bits)]
            if isinstance(blk.matrix, Recipe):
                mat = Recipe(full, blk.matrix.entries)
            else:
                mat = embed(blk.matrix, bits, full)
            entries.append(([tpos[b] for b in full], plan.add_matrix(mat)))
        plan.steps.append(TcSweepStep(L, list(high), entries, all(flag[id(b)] for b in taken)))


def plan_flops(plan):
    """(algorithmic bytes, flops) per vector element summed over passes: bytes
    are two vector passes (read + write) per dense/sweep step; flops are
    8 * 2^k per element per dense op of width k."""
    passes, flops = 0, 0
    for s in plan.steps:
        if isinstance(s, DenseStep):
            passes += 1
            flops += 8 * 2 ** len(s.bits)
        elif isinstance(s, SweepStep):
            passes += 1
            flops += sum(8 * 2 ** len(p) for p, _ in s.ops)
        elif isinstance(s, TcSweepStep):
            passes += 1
            flops += sum(8 * 2 ** len(p) for p, _ in s.blocks)
    return passes, flops
