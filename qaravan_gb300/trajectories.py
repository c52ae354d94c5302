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

Two execution modes:

* ``"persistent"`` (default): one ``qgb_traj_run`` launch for the whole run.
  The circuit is cut on the host into tile sweeps (``plan_traj_sweeps``: gates
  whose sites fit one shared-memory tile of ``tile_bits`` bits); every CTA of
  the launch takes trajectories from a work counter and streams each through
  all sweeps, so a trajectory's state is read and written once per sweep
  instead of once per gate. Amplitude damping is unravelled exactly by the
  no-jump norm (the library's kernel: a uniform threshold per jump, the
  sweep run again from its input when a jump falls inside it).
* ``"per_gate"``: each gate is one ``qgb_traj_step`` call (a fused gate +
  noise kernel and a per-trajectory decision kernel drawing the damping
  branches site by site).

Both draw the same depolarising Paulis for the same seed. ``run(graph=True)``
captures the run in one CUDA graph and replays it.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from .statevector import _to_np, circuit_ops, pauli_expectations


TRAJ_SWEEP = np.dtype([("L", "<i4"), ("H", "<i4"), ("high_bits", "<i4", (10,)), ("op_begin", "<i4"),
                       ("op_end", "<i4")])
TRAJ_OP = np.dtype([("k", "<i4"), ("pos", "<i4", (2,)), ("gate", "<i4"), ("mat", "<i8"), ("flags", "<i4"),
                    ("run", "<i4"), ("run_pos", "<i4", (4,)), ("lpos", "<i4", (2,))])
TRAJ_MAX_OPS = 128


def plan_traj_sweeps(gate_bits, nbits, tile_bits, low_min, max_ops=TRAJ_MAX_OPS, max_high=10):
    """Cut a gate sequence (flat bits per gate, in order) into tile sweeps.

    Each sweep's tile is the low ``L`` bits times ``H = tile_bits - L`` high bits
    (``L >= low_min`` keeps every copied run at least 256 bytes). Gates are
    taken in order while their bits fit; a gate that does not fit is skipped,
    and so is every later gate sharing a bit with a skipped one, so gates only
    move past gates they commute with. Candidate tiles: the contiguous low
    ``tile_bits`` bits, or ``L`` in {low_min, 8} with high bits chosen greedily;
    the candidate taking the most gates wins. Returns ``[(L, high_bits, [gate
    indices])]``."""
    m = min(tile_bits, nbits)
    if m == nbits:
        shapes = [nbits]
    else:
        shapes = sorted({m, max(min(low_min, m), m - max_high), max(min(8, m), m - max_high)}, reverse=True)
    remaining = list(range(len(gate_bits)))
    sweeps = []
    while remaining:
        best = None
        # fallback shapes with fewer low bits (shorter copied runs) only when the others take nothing
        for L in shapes + [x for x in range(min(shapes) - 1, max(m - max_high, 1) - 1, -1)]:
            if best is not None and best[2] and L < min(shapes):
                break
            H = m - L
            high, taken, blocked = [], [], set()
            for j, gi in enumerate(remaining):
                bits = gate_bits[gi]
                if len(blocked) >= nbits:
                    break
                bset = set(bits)
                if bset & blocked or len(taken) >= max_ops:
                    blocked |= bset
                    continue
                need = [b for b in bits if b >= L and b not in high]
                if len(high) + len(need) <= H:
                    high.extend(need)
                    taken.append(gi)
                else:
                    blocked |= bset
            if best is None or len(taken) > len(best[2]):
                best = (L, high, taken)
        L, high, taken = best
        if not taken:
            raise RuntimeError("trajectory sweep planner made no progress (a gate wider than the tile)")
        for b in range(L, nbits):  # fill the tile to its full size (fewer, larger tiles; same traffic)
            if len(high) >= m - L:
                break
            if b not in high:
                high.append(b)
        sweeps.append((L, sorted(high), taken))
        done = set(taken)
        remaining = [g for g in remaining if g not in done]
    return sweeps


class _TileOp:
    def __init__(self, bits):
        self.bits = list(bits)


def plan_runs(tile_pos, m, rmax):
    """Group a sweep's gates (their tile positions, in order) into runs over
    ``R = min(rmax, m)`` tile bits that the kernel applies to register-resident
    groups of 2^R amplitudes: the fusion rule of the compiler (a gate joins the
    latest run it depends on while the union stays within R bits; earlier runs
    it covers and that nothing in between touches are absorbed), so gates move
    only past gates on other bits. Returns ``[(run bits padded to R, [gate
    positions in the list, application order])]``."""
    from .compiler import fuse_symbolic
    R = min(rmax, m)
    blocks = fuse_symbolic([_TileOp(p) for p in tile_pos], R)
    runs = []
    for b in blocks:
        bits = sorted(b.bits)
        for x in range(m):  # pad with unused tile bits: every run spans exactly R bits
            if len(bits) >= R:
                break
            if x not in bits:
                bits.append(x)
        runs.append((bits, list(b.ops)))
    return runs


class TrajectorySim:
    def __init__(self, circ, ntraj, p_dep=0.0, gamma=0.0, seed=0, dtype=torch.complex64, device="cuda",
                 log=False, mode="persistent", tile_bits=None, max_log=64):
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
        if mode not in ("persistent", "per_gate"):
            raise ValueError(f"trajectory mode {mode!r} (persistent, per_gate)")
        self.mode = mode
        self.max_log = int(max_log) if log else 0
        if tile_bits is None:
            from . import autotune
            tile_bits = autotune.choose_traj(self.n, dtype)
        self.tile_bits = int(tile_bits)
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
        if self.mode == "persistent":
            self._prepare_persistent()

    def _prepare_persistent(self):
        n, T = self.n, self.ntraj
        L = _lib.lib()
        if L.qgb_traj_sweep_bytes() != TRAJ_SWEEP.itemsize or L.qgb_traj_op_bytes() != TRAJ_OP.itemsize:
            raise _lib.QgbError("trajectory table layout mismatch with the library")
        isz = self.mats.element_size()
        low_min = 5 if isz == 8 else 4
        bits = [[n - 1 - int(q) for q in g.indices] for g in self.gates]
        plan = plan_traj_sweeps(bits, n, self.tile_bits, low_min) if self.gates else []
        sw = np.zeros(len(plan), dtype=TRAJ_SWEEP)
        ops = np.zeros(max(len(self.gates), 1), dtype=TRAJ_OP)
        rmax = 4 if isz == 8 else 3
        diag = [bool(np.all(np.asarray(_to_np(g.matrix)) == np.diag(np.diag(_to_np(g.matrix))))) for g in self.gates]
        o = 0
        for s_i, (Lb, high, taken) in enumerate(plan):
            tpos = {b: b for b in range(Lb)}
            for h, b in enumerate(high):
                tpos[b] = Lb + h
            m = Lb + len(high)
            sw[s_i]["L"], sw[s_i]["H"] = Lb, len(high)
            sw[s_i]["high_bits"][:len(high)] = high
            sw[s_i]["op_begin"] = o
            order = []
            for rbits, members in plan_runs([[tpos[b] for b in bits[gi]] for gi in taken], m, rmax):
                for q, mi in enumerate(members):
                    gi = taken[mi]
                    p = [tpos[b] for b in bits[gi]]
                    ops[o]["k"] = len(p)
                    ops[o]["pos"][:len(p)] = p
                    ops[o]["gate"] = gi
                    ops[o]["mat"] = self.offs[gi]
                    ops[o]["flags"] = 1 if diag[gi] else 0
                    if q == 0:
                        ops[o]["run"] = len(members)
                        ops[o]["run_pos"][:len(rbits)] = rbits
                    ops[o]["lpos"][:len(p)] = [rbits.index(x) for x in p]
                    order.append(gi)
                    o += 1
            sw[s_i]["op_end"] = o
            plan[s_i] = (Lb, high, order)  # the gates in the order the kernel applies them
        self.sweep_plan = plan
        self._sweeps_host = np.ascontiguousarray(sw)
        self._sweeps_dev = torch.from_numpy(sw.view(np.uint8).copy()).to(self.device)
        self._ops_host = np.ascontiguousarray(ops)
        self._ops_dev = torch.from_numpy(ops.view(np.uint8).copy()).to(self.device)
        self._nops = o
        code = _lib.dtype_code(self.dtype)
        mmax = max([p[0] + len(p[1]) for p in plan] + [1])
        nbytes = L.qgb_traj_run_scratch_bytes(code, n, mmax, T)
        if nbytes == 0:
            raise _lib.QgbError("trajectory scratch size query failed")
        self._scratch = torch.empty((nbytes + 15) // 16 * 2, dtype=torch.float64, device=self.device)
        self._scratch_bytes = self._scratch.numel() * 8
        self.jump_count = torch.zeros(T, dtype=torch.int32, device=self.device)
        self.jump_events = (torch.zeros(T, max(self.max_log, 1), 2, dtype=torch.int32, device=self.device)
                            if self.max_log else None)

    def _launch_all(self):
        if self.mode == "persistent":
            return self._launch_persistent()
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

    def _launch_persistent(self):
        L = _lib.lib()
        code = _lib.dtype_code(self.dtype)
        st = _lib.stream_ptr(self.device)
        jl = self.jump_events.data_ptr() if self.jump_events is not None else None
        _lib.check(L.qgb_traj_run(self.state.data_ptr(), code, self.n, self.ntraj, 2 ** self.n,
                                  self._sweeps_host.ctypes.data, self._sweeps_dev.data_ptr(),
                                  len(self.sweep_plan), self._ops_host.ctypes.data, self._ops_dev.data_ptr(),
                                  self._nops, self.mats.data_ptr(), self.mats.numel(), self.p_dep, self.gamma, self.seed, self.jump_count.data_ptr(), jl, self.max_log,
                                  self._scratch.data_ptr(), self._scratch_bytes, st), "traj_run")

    @property
    def launches(self):
        if self.mode == "persistent":
            return 2  # the work-counter reset and the persistent kernel
        return 1 + 2 * len(self.gates) + 1

    def jumps(self, t):
        """Persistent mode with ``log=True``: the amplitude-damping jumps of
        trajectory ``t`` as (gate index, site position in the gate) pairs."""
        cnt = int(self.jump_count[t].item())
        if cnt > self.max_log:
            raise _lib.QgbError(f"trajectory {t} jumped {cnt} times; the log holds {self.max_log}")
        return [tuple(int(x) for x in e) for e in self.jump_events[t, :cnt].cpu().numpy()]

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
