"""Uneven batches of noisy density-matrix circuits.

The reference runs one ``DensityMatrixSim`` at a time, every op a full ncon
contraction over the rank-2n tensor (``tensorQ/density_matrix_sim.py:38-42``,
``core/base_sim.py:30-53``). ``DensityMatrixBatch`` runs many circuits of
different qubit counts and depths together:

* every circuit whose vec(rho) fits in shared memory (complex64: up to 7
  qubits, 2^14 entries; complex128: up to 6) is one CTA of a single
  ``qgb_batch_small`` launch that stages the whole vector once, applies all of
  its fused ops, and writes trace, purity and ``Re Tr(rho Z_i)`` in float64
  from its epilogue;
* larger complex64 circuits (8-14 qubits) run in ONE persistent launch on
  the tensor cores (``qgb_dm_batch_run``): every circuit is compiled into
  fused 6-bit passes on vec(rho) (narrower blocks widened with identity bits),
  the passes of all circuits become work items (pass, range of 8192-entry
  tiles) ordered pass by pass across circuits, each item waits for its
  circuit's previous pass, the trace chain corrects the tensor cores'
  rounding as in the single-circuit path, and each circuit's last pass writes
  its trace, purity and ``Re Tr(rho Z_i)``;
* other circuits (complex128, or plans with Reset or wide Pauli channels) run
  their compiled plans (tile size and fusion width from
  ``qaravan_gb300.autotune``) on parallel CUDA streams, followed by float64
  reductions;
* ``run(graph=True)`` captures all of it in one CUDA graph and replays it.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib, autotune
from .compiler import DenseStep, Plan, Recipe, compile_ops, embed, fuse
from .engine import Executor


def _circuit_dtype(dtype):
    return np.dtype([("offset", "<i8"), ("out_offset", "<i8"), ("nbits", "<i4"), ("op_begin", "<i4"),
                     ("op_end", "<i4"), ("flags", "<i4"), ("dm_sites", "<i4"), ("pad", "<i4")])


_OP_DTYPE = np.dtype([("k", "<i4"), ("pos", "<i4", (6,)), ("pad", "<i4"), ("mat", "<i8")])
_DMB_CIRC = np.dtype([("state", "<u8"), ("n", "<i4"), ("first_pass", "<i4"), ("n_passes", "<i4"), ("out_row", "<i4")])
_DMB_PASS = np.dtype([("mat", "<u8"), ("circ", "<i4"), ("bits", "<i4", (6,)), ("flags", "<i4"), ("tslot", "<i4"),
                      ("pad", "<i4")])
_DMB_HEAD, _DMB_TAIL, _DMB_LAST, _DMB_FIRST = 1, 2, 4, 8
_TRACE_EPOCH = 4  # tensor-core passes per trace-chain epoch (as the single-circuit executor)



def widen_plan(plan, width=6):
    """A copy of a plan of dense steps with every block widened to exactly
    ``width`` bits (identity on the added bits, the lowest free ones)."""
    new = Plan(nbits=plan.nbits, n_gates=plan.n_gates, trace_kept=plan.trace_kept)
    new.op_matrices = plan.op_matrices
    for st in plan.steps:
        m = plan.matrices[st.mat]
        bits = list(st.bits)
        full = bits + [b for b in range(plan.nbits) if b not in bits][:width - len(bits)]
        mat = Recipe(full, m.entries) if isinstance(m, Recipe) else embed(m, bits, full)
        new.steps.append(DenseStep(full, new.add_matrix(mat), st.unitary, st.whole))
    return new


def chain_flags(plan, first_index):
    """Per dense step of a density-matrix plan: (flags, trace slot) of the
    persistent launch -- first / last pass, and the trace chain: a tail pass
    (a whole-channel cut after at least four passes of the epoch) measures its
    output trace, the next pass divides its matrix by it (its slot: the tail
    pass's index in the pass table)."""
    out, t_since, pending = [], 0, None
    nsteps = len(plan.steps)
    for j, st in enumerate(plan.steps):
        flags, slot = 0, -1
        if j == 0:
            flags |= _DMB_FIRST
        if j == nsteps - 1:
            flags |= _DMB_LAST
        if plan.trace_kept and pending is not None:
            flags |= _DMB_HEAD
            slot, pending = pending, None
        t_since += 1
        if plan.trace_kept and st.whole and t_since >= _TRACE_EPOCH and j != nsteps - 1:
            flags |= _DMB_TAIL
            slot = first_index + j
            pending, t_since = slot, 0
        out.append((flags, slot))
    return out


class DensityMatrixBatch:
    """Run ``DensityMatrixSim``-like circuits together.

    ``sims``: list of ``DensityMatrixSim`` objects (their circuits, noise
    models and initial state |0...0> are used; Reset is supported on the
    per-stream path only)."""

    def __init__(self, sims, dtype=torch.complex64, device="cuda", width=4, small_max_bits=None, max_streams=8):
        self.sims = list(sims)
        self.dtype = dtype
        self.device = torch.device(device)
        self.code = _lib.dtype_code(dtype)
        self.isz = 8 if dtype == torch.complex64 else 16
        self.small_max = small_max_bits if small_max_bits is not None else (14 if self.isz == 8 else 13)
        self.width = min(width, 4)
        L = _lib.lib()
        if L.qgb_batch_circuit_bytes() != _circuit_dtype(dtype).itemsize or L.qgb_batch_op_bytes() != _OP_DTYPE.itemsize:
            raise _lib.QgbError("batch table layout mismatch with the library")
        self.nmax = max(s.num_sites for s in self.sims)
        self.ncols = 2 + self.nmax
        self.out = torch.zeros(len(self.sims), self.ncols, dtype=torch.float64, device=self.device)
        small, large = [], []
        for i, s in enumerate(self.sims):
            ops = s.op_sequence()
            nb = 2 * s.num_sites
            one_kernel = None not in ops and not any(o.kind == "pauli_mix" for o in ops)  # else per-circuit plans
            (small if (nb <= self.small_max and one_kernel) else large).append((i, s, ops))
        self._prep_small(small)
        persistent = [x for x in large if self._persistent_ok(x)]
        self._prep_persistent(persistent)
        done = {x[0] for x in persistent}
        self._prep_large([x for x in large if x[0] not in done], max_streams)
        self.graph = None

    # ------------------------------------------------------------ small path
    def _prep_small(self, small):
        self.small = small
        if not small:
            return
        circs = np.zeros(len(small), dtype=_circuit_dtype(self.dtype))
        op_rows, mats, moff = [], [], 0
        off = 0
        max_bits, max_k = 1, 1
        for j, (i, s, ops) in enumerate(small):
            nb = 2 * s.num_sites
            blocks = fuse(ops, max(self.width, max(len(o.bits) for o in ops))) if ops else []
            if any(len(b.bits) > 4 for b in blocks):
                blocks = fuse(ops, max(len(o.bits) for o in ops))
            begin = len(op_rows)
            for b in blocks:
                row = np.zeros((), dtype=_OP_DTYPE)
                row["k"] = len(b.bits)
                row["pos"][:len(b.bits)] = b.bits
                row["mat"] = moff
                op_rows.append(row)
                mats.append(b.matrix.reshape(-1))
                moff += b.matrix.size
                max_k = max(max_k, len(b.bits))
            circs[j] = (off, i * self.ncols, nb, begin, len(op_rows), 1, s.num_sites, 0)
            off += 4 ** s.num_sites
            off += off & 1  # 16-byte alignment for complex64
            max_bits = max(max_bits, nb)
        if max_k > 4:
            raise NotImplementedError("batched small circuits take fused ops of at most 4 bits")
        self.small_states = torch.zeros(max(off, 2), dtype=self.dtype, device=self.device)
        self.small_circs = torch.from_numpy(circs.view(np.uint8).copy()).to(self.device)
        ops_arr = np.array(op_rows, dtype=_OP_DTYPE) if op_rows else np.zeros(1, dtype=_OP_DTYPE)
        self.small_ops = torch.from_numpy(ops_arr.view(np.uint8).copy()).to(self.device)
        host = np.concatenate(mats) if mats else np.zeros(2, np.complex128)
        self.small_mats = torch.from_numpy(host).to(self.dtype).to(self.device)
        self.small_max_bits, self.small_max_k = max_bits, max_k
        self.small_state_offsets = {i: int(circs[j]["offset"]) for j, (i, s, ops) in enumerate(small)}

    # ------------------------------------------------------- persistent path
    def _persistent_ok(self, item):
        _, s, ops = item
        return (self.isz == 8 and _lib.lib().qgb_get_dense_impl() >= 1 and 8 <= s.num_sites <= 14
                and None not in ops and not any(o.kind == "pauli_mix" for o in ops) and len(ops) > 0)

    def _prep_persistent(self, items):
        self.pers = []
        if not items:
            return
        L = _lib.lib()
        if L.qgb_dm_batch_circuit_bytes() != _DMB_CIRC.itemsize or L.qgb_dm_batch_pass_bytes() != _DMB_PASS.itemsize:
            raise _lib.QgbError("density-matrix batch table layout mismatch with the library")
        circs = np.zeros(len(items), dtype=_DMB_CIRC)
        rows = []
        for ci, (i, s, ops) in enumerate(items):
            nb = 2 * s.num_sites
            plan = widen_plan(compile_ops(ops, nb, mode="fused", width=6, itemsize=8, device_fusion=True), 6)
            ex = Executor(plan, self.dtype, self.device, mode_normalize="dm")
            state = torch.empty(4 ** s.num_sites, dtype=self.dtype, device=self.device)
            first = len(rows)
            for (flags, slot), st in zip(chain_flags(plan, first), plan.steps):
                r = np.zeros((), dtype=_DMB_PASS)
                r["mat"] = ex.mats.data_ptr() + ex.mat_offsets[st.mat] * ex.itemsize
                r["circ"] = ci
                r["bits"] = st.bits
                r["flags"] = flags
                r["tslot"] = slot
                rows.append(r)
            circs[ci] = (state.data_ptr(), s.num_sites, first, len(plan.steps), ci)
            self.pers.append((i, s, ex, state))
        passes = np.array(rows, dtype=_DMB_PASS)
        # a pass of a large circuit: one item per SM (one wave)
        per_pass = torch.cuda.get_device_properties(self.device).multi_processor_count
        nitems = L.qgb_dm_batch_items(circs.ctypes.data, len(circs), per_pass)
        nbytes = L.qgb_dm_batch_table_bytes(len(circs), len(passes), nitems)
        if nitems < 1 or nbytes == 0:
            raise _lib.QgbError("density-matrix batch table size query failed")
        host = torch.empty(nbytes, dtype=torch.uint8)
        if torch.cuda.is_available():
            host = host.pin_memory()
        _lib.check(L.qgb_dm_batch_build(host.data_ptr(), nbytes, circs.ctypes.data, len(circs), passes.ctypes.data,
                                        len(passes), per_pass), "dm_batch_build")
        self._pers_table = host.to(self.device, non_blocking=True)
        self._pers_host = host  # alive until the copy is ordered before any use
        wbytes = L.qgb_dm_batch_work_bytes(len(circs), nitems)
        self._pers_work = torch.empty((wbytes + 15) // 16 * 16, dtype=torch.uint8, device=self.device)
        self._pers_out = torch.zeros(len(circs), 16, dtype=torch.float64, device=self.device)
        self._pers_rows = torch.tensor([i for i, *_ in self.pers], dtype=torch.int64, device=self.device)
        self._pers_sizes = (len(circs), len(passes), nitems, nbytes, self._pers_work.numel())
        self.persistent_passes = len(passes)
        self.persistent_items = nitems

    def _launch_persistent(self):
        L = _lib.lib()
        nc, npass, nitems, nbytes, wbytes = self._pers_sizes
        _lib.check(L.qgb_dm_batch_run(self._pers_table.data_ptr(), nbytes, nc, npass, nitems,
                                      self._pers_out.data_ptr(), nc, 16, self._pers_work.data_ptr(), wbytes,
                                      _lib.stream_ptr(self.device)), "dm_batch_run")
        self.out.index_copy_(0, self._pers_rows, self._pers_out[:, :self.ncols])

    # ------------------------------------------------------------ large path
    def _prep_large(self, large, max_streams):
        self.large = []
        tc = self.isz == 8 and _lib.lib().qgb_get_dense_impl() >= 1
        for i, s, ops in large:
            nb = 2 * s.num_sites
            if tc and nb >= 13:  # 6-qubit fused blocks on the tensor cores, one HBM pass each
                plan = compile_ops(ops, nb, mode="fused", width=6, itemsize=self.isz, device_fusion=True)
            else:
                tile, width = autotune.choose(nb, self.dtype)
                plan = compile_ops(ops, nb, mode="sweep", width=width, tile_bits=tile,
                                   max_sweep_k=5 if self.isz == 8 else 4, itemsize=self.isz, device_fusion=True)
            ex = Executor(plan, self.dtype, self.device, mode_normalize="dm")
            state = torch.empty(4 ** s.num_sites, dtype=self.dtype, device=self.device)
            L = _lib.lib()
            nbytes = max(L.qgb_reduce_scratch_bytes(nb, max(s.num_sites, 1), 1), 8)
            scratch = torch.empty(nbytes // 8 + 1, dtype=torch.float64, device=self.device)
            self.large.append((i, s, ex, state, scratch, nbytes))
        n_streams = min(max_streams, len(self.large))
        self.streams = [torch.cuda.Stream(self.device) for _ in range(max(n_streams, 0))]

    def _launch_large(self, item):
        i, s, ex, state, scratch, nbytes = item
        L = _lib.lib()
        n = s.num_sites
        st = _lib.stream_ptr(self.device)
        _lib.check(L.qgb_init_basis(state.data_ptr(), self.code, 2 * n, 0, 1, 0, st), "init")
        ex.run(state)
        base = self.out.data_ptr() + i * self.ncols * 8
        _lib.check(L.qgb_dm_trace(state.data_ptr(), self.code, n, 1, 0, base, scratch.data_ptr(), nbytes, st),
                   "dm_trace")
        _lib.check(L.qgb_norm2(state.data_ptr(), self.code, 2 * n, 1, 0, base + 8, scratch.data_ptr(), nbytes, st),
                   "norm2")
        zs = "".join('i' * q + 'z' + 'i' * (n - q - 1) for q in range(n)).encode()
        _lib.check(L.qgb_dm_pauli_expectation(state.data_ptr(), self.code, n, zs, None, n, 1, 0, base + 16,
                                              scratch.data_ptr(), nbytes, st), "dm_pauli_expectation")

    def _launch_all(self):
        L = _lib.lib()
        if self.pers:
            self._launch_persistent()
        main = torch.cuda.current_stream(self.device)
        for s in self.streams:
            s.wait_stream(main)
        for j, item in enumerate(self.large):
            with torch.cuda.stream(self.streams[j % len(self.streams)]):
                self._launch_large(item)
        if self.small:
            _lib.check(L.qgb_batch_small(self.small_states.data_ptr(), self.code, self.small_circs.data_ptr(),
                                         len(self.small), self.small_ops.data_ptr(), self.small_mats.data_ptr(),
                                         self.small_max_bits, self.small_max_k, self.out.data_ptr(),
                                         _lib.stream_ptr(self.device)), "batch_small")
        for s in self.streams:
            main.wait_stream(s)

    @property
    def launches(self):
        n = 1 if self.small else 0
        if self.pers:
            n += 2  # the persistent kernel and the copy of its result rows
        for item in self.large:
            n += 1 + item[2].plan.n_sweeps + 3 * 2 + 1
        return n

    def run(self, graph=False):
        if not graph:
            self._launch_all()
            return self
        if self.graph is None:
            self._launch_all()
            torch.cuda.synchronize(self.device)
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, capture_error_mode="thread_local"):
                self._launch_all()
            self.graph = g
        self.graph.replay()
        return self

    def results(self):
        """Per circuit: trace, purity Tr(rho^2) and Re Tr(rho Z_i) (float64)."""
        out = self.out.cpu().numpy()
        res = []
        for i, s in enumerate(self.sims):
            n = s.num_sites
            res.append({"trace": out[i, 0], "purity": out[i, 1], "z": out[i, 2:2 + n].copy()})
        return res

    def density_matrix(self, i):
        n = self.sims[i].num_sites
        d = 2 ** n
        if i in getattr(self, "small_state_offsets", {}):
            o = self.small_state_offsets[i]
            return self.small_states[o:o + d * d].reshape(d, d)
        for item in self.large + self.pers:
            if item[0] == i:
                return item[3].reshape(d, d)
        raise KeyError(i)
