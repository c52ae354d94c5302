"""Plan executor: runs a compiled :class:`~qaravan_gb300.compiler.Plan` on
device-resident vectors through the C ABI.

All gate matrices of a plan are uploaded once, packed into one device buffer
in the state's dtype (the reference instead converts and copies every gate
matrix host-to-device inside ``StatevectorSim.apply_gate``,
``tensorQ/statevector_sim.py:19-29,50-52``). Every launch goes to the current
torch stream; nothing synchronises, so a run can be captured in a CUDA graph.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from .compiler import DenseStep, NormalizeStep, Plan, SweepStep


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


class Executor:
    def __init__(self, plan: Plan, dtype=torch.complex64, device="cuda", mode_normalize="sv"):
        self.plan = plan
        self.dtype = dtype
        self.code = _lib.dtype_code(dtype)
        self.device = torch.device(device)
        self.normalize_kind = mode_normalize  # "sv": divide by the 2-norm; "dm": by the trace
        offs, flat = [], []
        o = 0
        for m in plan.matrices:
            offs.append(o)
            flat.append(m.reshape(-1))
            o += m.size
        self.mat_offsets = offs
        host = np.concatenate(flat) if flat else np.zeros(1, np.complex128)
        pinned = torch.from_numpy(host).to(dtype=dtype)
        if torch.cuda.is_available():
            pinned = pinned.pin_memory()
        self.mats = pinned.to(device=self.device, non_blocking=True)
        self._pinned = pinned  # alive until the copy is ordered before any use
        self.itemsize = self.mats.element_size()
        self.h2d_bytes = self.mats.numel() * self.itemsize
        self._steps = []
        for s in plan.steps:
            if isinstance(s, DenseStep):
                nb = plan.nbits
                sites = [nb - 1 - b for b in s.bits]
                self._steps.append(("dense", _lib.int_array(sites), len(sites), offs[s.mat]))
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
            elif isinstance(s, NormalizeStep):
                self._steps.append(("normalize",))
        self.scratch = Scratch(self.device)
        self.norm = torch.empty(1, dtype=torch.float64, device=self.device)
        self.launches = 0

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
        for s in self._steps:
            if events is not None and s[0] != "normalize":
                e0 = torch.cuda.Event(enable_timing=True)
                e0.record()
            if s[0] == "dense":
                _, sites, k, off = s
                if mat_stride:
                    _lib.check(L.qgb_op_action(ptr, self.code, nb, sites, k, mptr + off * self.itemsize,
                                               mat_stride, batch, stride, st), "op_action")
                else:
                    _lib.check(L.qgb_op_action(ptr, self.code, nb, sites, k, mptr + off * self.itemsize, 0,
                                               batch, stride, st), "op_action")
                launches += 1
            elif s[0] == "sweep":
                _lib.check(L.qgb_apply_sweep(ptr, self.code, nb, C.byref(s[1]), mptr, mat_stride, batch, stride, st),
                           "apply_sweep")
                launches += 1
            else:
                launches += self.normalize(state, batch, stride)
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
