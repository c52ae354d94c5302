"""Batched noisy trajectories on GB300.

The reference's Monte-Carlo path (``MonteCarloSim``,
``tensorQ/monte_carlo_sim.py:14-35``, driven by ``trotter_mc_sim``,
``applications/trotter.py:61-78``) runs one CPU statevector per sample and
supports Pauli channels only. ``TrajectorySim`` runs ``ntraj`` trajectories
of a circuit together on the GPU with, after every gate and on each of its
sites, a depolarising channel (I w.p. 1-p, X/Y/Z w.p. p/3, the
``PauliNoise(['i','x','y','z'], ...)`` convention of ``core/noise.py:90-129``)
followed by amplitude damping (Kraus ``diag(1, sqrt(1-gamma))`` and
``sqrt(gamma)|0><1|``, the ``t2 = inf`` case of ``QubitNoise``,
``core/noise.py:29-49``). Amplitude damping is unravelled exactly: each
site's jump probability is ``gamma * P(site = 1)`` of the current state.
The average over trajectories converges to ``DensityMatrixSim`` with the same
channels.

Each gate is one ``qgb_traj_step`` call (a fused gate + noise kernel and a
per-trajectory decision kernel); ``run(graph=True)`` captures the whole gate
sequence in one CUDA graph and replays it.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from .statevector import _to_np, circuit_ops, pauli_expectations


class TrajectorySim:
    def __init__(self, circ, ntraj, p_dep=0.0, gamma=0.0, seed=0, dtype=torch.complex64, device="cuda",
                 log=False):
        self.circ = circ
        self.n = circ.num_sites
        self.ntraj = int(ntraj)
        self.p_dep, self.gamma, self.seed = float(p_dep), float(gamma), int(seed)
        self.dtype = dtype
        self.device = torch.device(device)
        if self.device.type != "cuda":
            raise _lib.QgbError("qaravan_gb300 runs on CUDA devices only")
        self.gates = [g for g in circuit_ops(circ) if not (g.name == "ID" and getattr(g, "nm", None) is not None)]
        for g in self.gates:
            if len(g.indices) > 2:
                raise NotImplementedError("trajectory gates act on at most two sites")
            if g.name == "Reset":
                raise NotImplementedError("Reset inside noisy trajectories is not supported")
        self.log = log
        self._prepare()

    def _prepare(self):
        n, T = self.n, self.ntraj
        L = _lib.lib()
        flat, offs, o = [], [], 0
        for g in self.gates:
            m = _to_np(g.matrix).reshape(-1)
            offs.append(o)
            flat.append(m)
            o += m.size
        host = np.concatenate(flat) if flat else np.zeros(1, np.complex128)
        self.mats = torch.from_numpy(host).to(self.dtype).pin_memory().to(self.device, non_blocking=True)
        self.h2d_bytes = self.mats.numel() * self.mats.element_size()
        self.offs = offs
        self.state = torch.empty(T, 2 ** n, dtype=self.dtype, device=self.device)
        self.kraus = torch.zeros(T, 2, 4, dtype=self.dtype, device=self.device)
        nblk = L.qgb_traj_blocks(n)
        self.partials = torch.empty(T * nblk * 4, dtype=torch.float64, device=self.device)
        ng = len(self.gates)
        if self.log:
            self.pauli_log = torch.zeros(ng, T, 2, dtype=torch.uint8, device=self.device)
            self.jump_log = torch.zeros(ng, T, 2, dtype=torch.uint8, device=self.device)
        self._site_arrays = [_lib.int_array(g.indices) for g in self.gates]
        self.graph = None

    def _launch_all(self):
        L = _lib.lib()
        n, T = self.n, self.ntraj
        code = _lib.dtype_code(self.dtype)
        st = _lib.stream_ptr(self.device)
        sv = self.state.data_ptr()
        stride = 2 ** n
        isz = self.mats.element_size()
        _lib.check(L.qgb_init_basis(sv, code, n, 0, T, stride, st), "init_basis")
        prev, kprev = None, 0
        for i, g in enumerate(self.gates):
            plog = self.pauli_log[i].data_ptr() if self.log else None
            jlog = self.jump_log[i].data_ptr() if self.log else None
            _lib.check(L.qgb_traj_step(sv, code, n, T, stride, self._site_arrays[i], len(g.indices),
                                       self.mats.data_ptr() + self.offs[i] * isz, prev, kprev,
                                       self.kraus.data_ptr(), self.p_dep, self.gamma, self.seed, i,
                                       self.partials.data_ptr(), plog, jlog, st), "traj_step")
            prev, kprev = self._site_arrays[i], len(g.indices)
        if kprev:
            _lib.check(L.qgb_traj_step(sv, code, n, T, stride, None, 0, None, prev, kprev, self.kraus.data_ptr(),
                                       0.0, 0.0, self.seed, len(self.gates), self.partials.data_ptr(), None, None,
                                       st), "traj_step")

    @property
    def launches(self):
        return 1 + 2 * len(self.gates) + 1

    def run(self, graph=False):
        """All trajectories through the whole circuit; returns the (ntraj, 2^n) states."""
        if not graph:
            self._launch_all()
            return self.state
        if self.graph is None:
            self._launch_all()  # warm-up outside capture
            torch.cuda.synchronize(self.device)
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, capture_error_mode="thread_local"):
                self._launch_all()
            self.graph = g
        self.graph.replay()
        return self.state

    def time_gates(self):
        """One run with CUDA events around every gate's launches on the launching
        stream: a list of (gate index, union bits, lowest union bit, ms). The
        union is the gate's sites plus the previous gate's (pending damping)."""
        L = _lib.lib()
        n, T = self.n, self.ntraj
        code = _lib.dtype_code(self.dtype)
        st = _lib.stream_ptr(self.device)
        stream = torch.cuda.current_stream(self.device)
        sv, isz = self.state.data_ptr(), self.mats.element_size()
        _lib.check(L.qgb_init_basis(sv, code, n, 0, T, 2 ** n, st), "init_basis")
        rows, prev, kprev, prev_sites = [], None, 0, []
        for i, g in enumerate(self.gates):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            _lib.check(L.qgb_traj_step(sv, code, n, T, 2 ** n, self._site_arrays[i], len(g.indices),
                                       self.mats.data_ptr() + self.offs[i] * isz, prev, kprev, self.kraus.data_ptr(),
                                       self.p_dep, self.gamma, self.seed, i, self.partials.data_ptr(), None, None, st),
                       "traj_step")
            e1.record(stream)
            union = set(g.indices) | set(prev_sites)
            rows.append((i, len(union), n - 1 - max(union), e0, e1))
            prev, kprev, prev_sites = self._site_arrays[i], len(g.indices), list(g.indices)
        torch.cuda.synchronize(self.device)
        return [(i, k, lo, e0.elapsed_time(e1)) for i, k, lo, e0, e1 in rows]

    def expectations(self, terms):
        """(ntraj, nterms) float64 of c_t <psi|P_t|psi> per trajectory."""
        return pauli_expectations(self.state, self.n, terms, batch=self.ntraj, stride=2 ** self.n)

    def mean_expectations(self, terms):
        e = self.expectations(terms)
        e = e.reshape(self.ntraj, -1)
        return e.mean(dim=0), e.std(dim=0)


def philox_uniform(event, traj, stream, seed):
    out = C.c_double()
    _lib.lib().qgb_philox_uniform(event, traj, stream, seed, C.byref(out))
    return out.value


def z_terms(n):
    """<Z_i> and <Z_i Z_{i+1}> as Pauli-sum terms (the trajectory workload's outputs)."""
    zs = [(1.0, 'i' * q + 'z' + 'i' * (n - q - 1)) for q in range(n)]
    zz = [(1.0, 'i' * q + 'zz' + 'i' * (n - q - 2)) for q in range(n - 1)]
    return zs + zz
