"""Plan executor: runs a compiled :class:`~qaravan_gb300.compiler.Plan` on
device-resident vectors through the C ABI.

All gate matrices of a plan are uploaded once, packed into one device buffer
in the state's dtype (the reference instead converts and copies every gate
matrix host-to-device inside ``StatevectorSim.apply_gate``,
``tensorQ/statevector_sim.py:19-29,50-52``). A plan compiled with device
fusion uploads only the raw op matrices and the block tables (one pinned copy)
and composes the fused blocks on the GPU (``qgb_fuse_blocks``). Every launch
goes to the current torch stream; nothing synchronises, so a run can be
captured in a CUDA graph.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np
import torch

from . import _lib
from .compiler import DenseStep, NormalizeStep, PauliMixStep, Plan, Recipe, SweepStep, TcSweepStep

# Unitary fused blocks control the norm on the tensor-core path, removing the
# round-toward-zero shrinkage of tensor-core accumulation (~1e-7 of the norm per
# pass). "chain" (default, one state): consecutive unitary blocks form a norm
# chain (qgb_op_action_unitary_chain), each pass scaling its output back to the
# chain's reference norm. "row": every amplitude group's norm is restored in the
# pass (qgb_op_action_unitary; also what batches use under "chain"), ~10 % of the
# kernel's speed. "off": neither. QGB_NORM_RESTORE=chain|row|0 or set_norm_restore().
_NORM_MODES = {"1": "chain", "chain": "chain", "row": "row", "0": "off", "off": "off"}
_NORM_RESTORE = _NORM_MODES.get(os.environ.get("QGB_NORM_RESTORE", "chain"), "chain")


# Complex64 density matrices on the tensor cores keep their trace by a trace
# chain: the trace is measured (qgb_dm_trace_factor) where the ops applied so
# far are whole channels, at most every _TRACE_EPOCH tensor-core passes, and the
# next tensor-core pass multiplies its matrix by reference / measured trace
# (qgb_op_action_scaled). QGB_TRACE_CHAIN=0 or set_trace_chain(False) turns it off.
_TRACE_EPOCH = 4
_TRACE_CHAIN = os.environ.get("QGB_TRACE_CHAIN", "1") not in ("0", "off")


def set_trace_chain(on=True):
    """Process-wide trace chain of complex64 density matrices (default on)."""
    global _TRACE_CHAIN
    _TRACE_CHAIN = bool(on)


def tc_eligible(code, nbits, k, batch=1):
    """Whether the library runs a dense op of width k on a vector of nbits bits on
    the tensor cores (its own rule: complex64, 4-6 bits -- 4 only in its default
    mode --, at least one 8192-amplitude tile, one operator for the batch)."""
    if code != _lib.QGB_C64 or nbits < 13 or not 4 <= k <= 6:
        return False
    impl = _lib.lib().qgb_get_dense_impl()
    return impl >= 2 or (impl == 1 and k >= 5)


def set_norm_restore(mode="chain"):
    """Process-wide norm control of unitary tensor-core blocks: "chain" (default),
    "row", or "off" (True / False mean "chain" / "off")."""
    global _NORM_RESTORE
    if mode is True:
        mode = "chain"
    elif mode is False:
        mode = "off"
    if mode not in ("chain", "row", "off"):
        raise ValueError(f"norm restore mode {mode!r} (chain, row, off)")
    _NORM_RESTORE = mode


_FUSE_BLOCK = np.dtype([("out", "<i8"), ("k", "<i4"), ("op_begin", "<i4"), ("op_end", "<i4"), ("pad", "<i4")])
_FUSE_ENTRY = np.dtype([("k", "<i4"), ("pos", "<i4", (6,)), ("pad", "<i4"), ("mat", "<i8")])


def real_dtype(dtype):
    return torch.float32 if dtype == torch.complex64 else torch.float64


class Scratch:
    """Caller-owned scratch for reductions (grown on demand, never inside a run)."""

    def __init__(self, device):
        self.device = device
        self.buf = None

    def get(self, nbytes):
        if self.buf is None or self.buf.numel() * 8 < nbytes:
            self.buf = torch.empty((nbytes + 7) // 8, dtype=torch.float64, device=self.device)
        return self.buf


# fusion tables per plan structure: id(recipe list) -> (that list, op sizes, tables ...)
_LAYOUT_CACHE: dict = {}


class Executor:
    def __init__(self, plan: Plan, dtype=torch.complex64, device="cuda", mode_normalize="sv"):
        self.plan = plan
        self.dtype = dtype
        self.code = _lib.dtype_code(dtype)
        self.device = torch.device(device)
        self.normalize_kind = mode_normalize  # "sv": divide by the 2-norm; "dm": by the trace
        if plan.device_fused:
            offs = self._fuse_on_device(plan)
        else:
            offs, flat = [], []
            o = 0
            for m in plan.matrices:
                offs.append(o)
                flat.append(m.reshape(-1))
                o += m.size
            host = np.concatenate(flat) if flat else np.zeros(1, np.complex128)
            pinned = torch.from_numpy(host).to(dtype=dtype)
            if torch.cuda.is_available():
                pinned = pinned.pin_memory()
            self.mats = pinned.to(device=self.device, non_blocking=True)
            self._pinned = pinned  # alive until the copy is ordered before any use
            self.h2d_bytes = self.mats.numel() * self.mats.element_size()
        self.mat_offsets = offs
        self.itemsize = self.mats.element_size()
        self._steps = []
        for s in plan.steps:
            if isinstance(s, DenseStep):
                nb = plan.nbits
                sites = [nb - 1 - b for b in s.bits]
                self._steps.append(("dense", _lib.int_array(sites), len(sites), offs[s.mat], s.unitary, s.whole,
                                    tc_eligible(self.code, nb, len(sites))))
            elif isinstance(s, SweepStep):
                sw = _lib.Sweep()
                sw.low_bits = s.low_bits
                sw.n_high = len(s.high_bits)
                for i, b in enumerate(s.high_bits):
                    sw.high_bits[i] = b
                sw.n_ops = len(s.ops)
                for i, (pos, mi) in enumerate(s.ops):
                    sw.op_k[i] = len(pos)
                    for j, p in enumerate(pos):
                        sw.op_pos[i][j] = p
                    sw.op_mat[i] = offs[mi]
                self._steps.append(("sweep", sw))
            elif isinstance(s, TcSweepStep):
                ts = _lib.TcSweep()
                ts.low_bits = s.low_bits
                for i, b in enumerate(s.high_bits):
                    ts.high_bits[i] = b
                ts.n_blocks = len(s.blocks)
                for i, (pos, mi) in enumerate(s.blocks):
                    for j, p in enumerate(pos):
                        ts.block_pos[i][j] = p
                    ts.block_mat[i] = offs[mi]
                self._steps.append(("tcsweep", ts, s.unitary))
            elif isinstance(s, NormalizeStep):
                self._steps.append(("normalize",))
            elif isinstance(s, PauliMixStep):
                if len(s.terms) > 128:
                    raise NotImplementedError("Pauli channels of more than 128 terms")
                strings = "".join(t[1].lower() for t in s.terms).encode()
                self._steps.append(("pauli_mix", strings, _lib.double_array([t[0] for t in s.terms]), len(s.terms)))
        self.scratch = Scratch(self.device)
        self.norm = torch.empty(1, dtype=torch.float64, device=self.device)
        self.launches = 0

    def _fuse_on_device(self, plan):
        """Uploads the raw op matrices (complex128) and the block/entry tables in
        one pinned buffer and composes every block matrix on the GPU; returns the
        element offset of each plan matrix in ``self.mats``."""
        L = _lib.lib()
        if L.qgb_fuse_block_bytes() != _FUSE_BLOCK.itemsize or L.qgb_fuse_entry_bytes() != _FUSE_ENTRY.itemsize:
            raise _lib.QgbError("fusion table layout mismatch with the library")
        op_mats = list(plan.op_matrices)
        recipes = []
        for m in plan.matrices:
            if isinstance(m, Recipe):
                recipes.append(m)
            else:  # a host matrix: a one-entry recipe on its own bit order
                k = int(np.log2(m.shape[0]))
                op_mats.append(np.ascontiguousarray(m, dtype=np.complex128))
                bits = list(range(k - 1, -1, -1))
                recipes.append(Recipe(bits, [(len(op_mats) - 1, bits)]))
        # the tables depend on the plan's structure only: kept with its (shared) recipe list
        all_recipes = len(recipes) == len(plan.matrices) and len(recipes) > 0
        hit = _LAYOUT_CACHE.get(id(plan.matrices)) if all_recipes else None
        if hit is not None and hit[0] is plan.matrices and hit[1] == [m.size for m in op_mats]:
            _, _, op_off, n_op_elems, blocks, ents, n_ent, offs, out = hit
        else:
            op_off, o = [], 0
            for m in op_mats:
                op_off.append(o)
                o += m.size
            n_op_elems = max(o, 1)
            blocks = np.zeros(len(recipes), dtype=_FUSE_BLOCK)
            n_ent = sum(len(r.entries) for r in recipes)
            ents = np.zeros(max(n_ent, 1), dtype=_FUSE_ENTRY)
            offs, out, e = [], 0, 0
            for i, r in enumerate(recipes):
                k = len(r.bits)
                offs.append(out)
                blocks[i] = (out, k, e, e + len(r.entries), 0)
                pos_of = {b: j for j, b in enumerate(r.bits)}
                for mi, obits in r.entries:
                    ents["k"][e] = len(obits)
                    ents["pos"][e, :len(obits)] = [pos_of[b] for b in obits]
                    ents["mat"][e] = op_off[mi]
                    e += 1
                out += 4 ** k
            if all_recipes:
                _LAYOUT_CACHE[id(plan.matrices)] = (plan.matrices, [m.size for m in op_mats], op_off, n_op_elems,
                                                    blocks, ents, n_ent, offs, out)
                while len(_LAYOUT_CACHE) > 32:
                    _LAYOUT_CACHE.pop(next(iter(_LAYOUT_CACHE)))
        opm = np.concatenate([m.reshape(-1) for m in op_mats]) if op_mats else np.zeros(1, np.complex128)
        sections = [opm.view(np.uint8), blocks.view(np.uint8), ents.view(np.uint8)]
        starts, nbytes = [], 0
        for sec in sections:
            starts.append(nbytes)
            nbytes += (sec.size + 15) // 16 * 16
        host = np.zeros(nbytes, dtype=np.uint8)
        for st0, sec in zip(starts, sections):
            host[st0:st0 + sec.size] = sec
        pinned = torch.from_numpy(host)
        if torch.cuda.is_available():
            pinned = pinned.pin_memory()
        dev = pinned.to(device=self.device, non_blocking=True)
        self._pinned = pinned  # alive until the copy is ordered before any use
        self._fuse_tables = dev
        self.h2d_bytes = nbytes
        self.mats = torch.empty(max(out, 1), dtype=self.dtype, device=self.device)
        base = dev.data_ptr()
        _lib.check(L.qgb_fuse_blocks(self.mats.data_ptr(), self.code, self.mats.numel(), base + starts[1],
                                     len(recipes), base + starts[2], n_ent, base + starts[0], n_op_elems,
                                     _lib.stream_ptr(self.device)), "fuse_blocks")
        return offs

    def run(self, state: torch.Tensor, batch: int = 1, stride: int = 0, mats: torch.Tensor | None = None,
            mat_stride: int = 0, events: list | None = None):
        """Apply the plan in place to ``batch`` vectors at ``stride`` elements apart.
        ``mats`` (optional) replaces the packed matrices, ``mat_stride`` elements per vector.
        ``events`` (optional list) receives ``(kind, start, end)`` CUDA events around each launch."""
        _lib.require_cuda(state)
        if state.dtype != self.dtype:
            raise _lib.QgbError(f"state dtype {state.dtype} does not match plan dtype {self.dtype}")
        L = _lib.lib()
        nb = self.plan.nbits
        st = _lib.stream_ptr(state.device)
        ptr = state.data_ptr()
        mats = self.mats if mats is None else mats
        mptr = mats.data_ptr()
        launches = 0
        link = 0  # position in the current norm chain of consecutive unitary blocks
        # trace chain: one complex64 density matrix whose ops keep the trace
        tchain = (_TRACE_CHAIN and self.normalize_kind == "dm" and self.code == _lib.QGB_C64 and batch == 1
                  and mats is self.mats and self.plan.trace_kept
                  and any(s[0] == "dense" and s[6] for s in self._steps))
        if tchain:
            if getattr(self, "_tchain", None) is None:
                self._tchain = torch.zeros(4, dtype=torch.float64, device=self.device)
            tptr = self._tchain.data_ptr()
            _lib.check(L.qgb_dm_trace_factor(ptr, self.code, nb // 2, tptr, 1, st), "dm_trace_factor")
            launches += 1
            t_since, t_pending = 0, False  # tensor-core passes since the last measurement; a factor waits
        for s in self._steps:
            if events is not None and s[0] != "normalize":
                e0 = torch.cuda.Event(enable_timing=True)
                e0.record()
            if s[0] == "dense" and tchain:
                _, sites, k, off, unitary, whole, on_tc = s
                if on_tc and t_pending:
                    _lib.check(L.qgb_op_action_scaled(ptr, self.code, nb, sites, k, mptr + off * self.itemsize,
                                                      tptr + 8, st), "op_action")
                    t_pending = False
                else:
                    _lib.check(L.qgb_op_action(ptr, self.code, nb, sites, k, mptr + off * self.itemsize, 0, 1, 0,
                                               st), "op_action")
                launches += 1
                t_since += int(on_tc)
                if whole and t_since >= _TRACE_EPOCH:
                    _lib.check(L.qgb_dm_trace_factor(ptr, self.code, nb // 2, tptr, 0, st), "dm_trace_factor")
                    launches += 1
                    t_since, t_pending = 0, True
            elif s[0] == "dense":
                _, sites, k, off, unitary = s[:5]
                # per-vector matrices (mat_stride) need not be unitary: only the plan's own are flagged
                mode = _NORM_RESTORE if (unitary and mats is self.mats) else "off"
                if mode == "chain" and batch == 1:
                    if getattr(self, "_chain", None) is None:
                        self._chain = torch.zeros(6, dtype=torch.float64, device=self.device)
                    _lib.check(L.qgb_op_action_unitary_chain(ptr, self.code, nb, sites, k, mptr + off * self.itemsize,
                                                             0, 1, stride, self._chain.data_ptr(), link, st),
                               "op_action")
                    link += 1
                else:
                    fn = L.qgb_op_action if mode == "off" else L.qgb_op_action_unitary
                    _lib.check(fn(ptr, self.code, nb, sites, k, mptr + off * self.itemsize,
                                  mat_stride if mat_stride else 0, batch, stride, st), "op_action")
                    link = 0
                launches += 1
            elif s[0] == "sweep":
                _lib.check(L.qgb_apply_sweep(ptr, self.code, nb, C.byref(s[1]), mptr, mat_stride, batch, stride, st),
                           "apply_sweep")
                launches += 1
                link = 0
            elif s[0] == "tcsweep":
                if batch != 1 or mats is not self.mats:
                    raise _lib.QgbError("tensor-core sweeps run one state with the plan's own matrices")
                if s[2] and _NORM_RESTORE != "off":
                    if getattr(self, "_chain", None) is None:
                        self._chain = torch.zeros(6, dtype=torch.float64, device=self.device)
                    _lib.check(L.qgb_apply_tc_sweep(ptr, self.code, nb, C.byref(s[1]), mptr, self._chain.data_ptr(),
                                                    link, st), "apply_tc_sweep")
                    link += 1
                else:
                    _lib.check(L.qgb_apply_tc_sweep(ptr, self.code, nb, C.byref(s[1]), mptr, None, 0, st),
                               "apply_tc_sweep")
                    link = 0
                launches += 1
            elif s[0] == "pauli_mix":
                _, strings, coeff, nterms = s
                if getattr(self, "_mix_buf", None) is None or self._mix_buf.numel() < state.numel():
                    self._mix_buf = torch.empty(state.numel(), dtype=self.dtype, device=state.device)
                tmp = self._mix_buf[:state.numel()]
                _lib.check(L.qgb_pauli_apply(ptr, tmp.data_ptr(), self.code, nb, strings, coeff, nterms, batch,
                                             stride, st), "pauli_apply")
                flat, dim = state.view(-1), 2 ** nb
                for b in range(batch):  # only the vectors (a stride may leave gaps)
                    o = b * (stride if batch > 1 else 0)
                    flat[o:o + dim].copy_(tmp[o:o + dim])
                launches += 1 + batch
                link = 0
            else:
                launches += self.normalize(state, batch, stride)
                link = 0
                if tchain:  # the trace is 1 again: a new reference
                    _lib.check(L.qgb_dm_trace_factor(ptr, self.code, nb // 2, tptr, 1, st), "dm_trace_factor")
                    launches += 1
                    t_since, t_pending = 0, False
            if events is not None and s[0] != "normalize":
                e1 = torch.cuda.Event(enable_timing=True)
                e1.record()
                events.append((s[0], e0, e1))
        self.launches = launches
        return state

    def normalize(self, state, batch=1, stride=0):
        """Renormalise in place (2-norm for statevectors, trace for density matrices)."""
        L = _lib.lib()
        nb = self.plan.nbits
        st = _lib.stream_ptr(state.device)
        if self.norm.numel() < batch:
            self.norm = torch.empty(batch, dtype=torch.float64, device=self.device)
        if self.normalize_kind == "sv":
            nbytes = L.qgb_reduce_scratch_bytes(nb, 1, batch)
            buf = self.scratch.get(nbytes)
            _lib.check(L.qgb_norm2(state.data_ptr(), self.code, nb, batch, stride, self.norm.data_ptr(),
                                   buf.data_ptr(), nbytes, st), "norm2")
            scale = torch.rsqrt(self.norm[:batch])
        else:
            n = nb // 2
            nbytes = L.qgb_reduce_scratch_bytes(nb, 1, batch)
            buf = self.scratch.get(nbytes)
            _lib.check(L.qgb_dm_trace(state.data_ptr(), self.code, n, batch, stride, self.norm.data_ptr(),
                                      buf.data_ptr(), nbytes, st), "dm_trace")
            scale = 1.0 / self.norm[:batch]
        _lib.check(L.qgb_scale(state.data_ptr(), self.code, nb, scale.data_ptr(), batch, stride, st), "scale")
        self._last_scale = scale  # keep alive until the launch is ordered
        return 3
