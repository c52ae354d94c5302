"""Adjoint-method gradients behind ``torch.autograd``.

The reference differentiates circuits by running its torch backend under
autograd (``core/param_gates.py:21-49`` builds gate matrices with
``torch.linalg.matrix_exp``; ``applications/compilation.py:73-133`` calls
``loss.backward()``), which keeps every intermediate state on the tape: one
state per gate. Here the forward pass runs the fused CUDA plan and keeps only
the final state; the backward pass walks the gates in reverse, uncomputing the
state (``phi <- U^dagger phi``) and carrying the co-state
(``lam <- U^dagger lam``) in one kernel pass per gate, which also reduces the
gate's gradient block ``sum_rest lam[r, rest] conj(phi[c, rest])`` in float64
(``qgb_adjoint_step``). Memory: three states, independent of depth.

Conventions: for a real loss L, torch's gradient of a complex tensor z is
``2 dL/d conj(z)``; the state function receives ``g = 2 dL/d conj(psi)`` and
returns ``dL/dM = sum g[r] conj(phi[c])`` (the factor 2 is already in ``g``);
the energy function starts from ``lam = H psi`` and returns
``2 sum lam[r] conj(phi[c])``.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib
from .compiler import Op, compile_ops
from .engine import Executor, Scratch


def _gate_list(sim):
    from .statevector import circuit_ops
    gates = [g for g in circuit_ops(sim.circ) if not (g.name == "ID" and getattr(g, "nm", None) is not None)]
    for g in gates:
        if len(g.indices) > 2:
            raise NotImplementedError("the adjoint sweep handles gates on one or two sites")
        if g.name == "Reset":
            raise NotImplementedError("Reset is not differentiable")
    return gates


class _Runner:
    """Forward plan + reverse sweep for a fixed gate structure."""

    def __init__(self, sim, gates):
        self.sim = sim
        self.gates = gates
        self.n = sim.num_sites
        self.dtype = sim.dtype
        self.device = sim.device
        self.code = _lib.dtype_code(self.dtype)
        self.scratch = Scratch(self.device)
        self._sites = [_lib.int_array(g.indices) for g in gates]

    def host_matrices(self, mats):
        """All gate matrices as complex128 NumPy arrays (one host transfer)."""
        flat = torch.cat([m.detach().reshape(-1).to("cpu", torch.complex128) for m in mats]).numpy()
        out, o = [], 0
        for m in mats:
            k = m.numel()
            d = int(round(k ** 0.5))
            out.append(flat[o:o + k].reshape(d, d))
            o += k
        return out, flat

    def forward_state(self, mats):
        n = self.n
        host, flat = self.host_matrices(mats)
        self._flat = flat
        ops = [Op([n - 1 - q for q in g.indices], m) for g, m in zip(self.gates, host)]
        kcap = 5 if self.dtype == torch.complex64 else 4
        isz = torch.empty(0, dtype=self.dtype).element_size()
        plan = compile_ops(ops, n, mode=self.sim.mode, width=self.sim.fusion_width, tile_bits=self.sim.tile_bits,
                           low_bits=self.sim.low_bits, max_sweep_k=kcap, itemsize=isz, device_fusion=True)
        psi = torch.empty(2 ** n, dtype=self.dtype, device=self.device)
        L = _lib.lib()
        _lib.check(L.qgb_init_basis(psi.data_ptr(), self.code, n, 0, 1, 0, _lib.stream_ptr(self.device)), "init")
        Executor(plan, self.dtype, self.device).run(psi)
        return psi

    def reverse(self, psi, lam, mats, need):
        """Reverse sweep from (psi, lam); returns per-gate sum_rest lam[r] conj(phi[c]) (complex128) or None."""
        L = _lib.lib()
        n = self.n
        st = _lib.stream_ptr(self.device)
        phi = psi.detach().clone()
        lam = lam.contiguous()
        # every gate matrix in one pinned upload; per-gate element offsets
        flat = getattr(self, "_flat", None)
        if flat is None:
            _, flat = self.host_matrices(mats)
        dev = torch.from_numpy(flat).to(self.dtype).pin_memory().to(self.device, non_blocking=True)
        isz = dev.element_size()
        offs = np.cumsum([0] + [m.numel() for m in mats])
        grads_dev = torch.empty(len(self.gates), 32, dtype=torch.float64, device=self.device)
        nbytes = L.qgb_reduce_scratch_bytes(n, 32, 1)
        scr = self.scratch.get(nbytes)
        base, gbase = dev.data_ptr(), grads_dev.data_ptr()
        for i in range(len(self.gates) - 1, -1, -1):
            g = self.gates[i]
            out = gbase + i * 32 * 8 if need[i] else None
            _lib.check(L.qgb_adjoint_step(phi.data_ptr(), lam.data_ptr(), self.code, n, self._sites[i],
                                          len(g.indices), base + int(offs[i]) * isz, out, scr.data_ptr(), nbytes, st),
                       "adjoint_step")
        host = grads_dev.cpu().numpy()
        out = []
        for i, g in enumerate(self.gates):
            if not need[i]:
                out.append(None)
                continue
            d = 2 ** len(g.indices)
            v = host[i, :2 * d * d]
            out.append((v[0::2] + 1j * v[1::2]).reshape(d, d))
        return out


def _grad_like(m, arr):
    return torch.from_numpy(arr).to(device=m.device, dtype=m.dtype if m.is_complex() else torch.complex128)


class _StateFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, runner, *mats):
        psi = runner.forward_state(mats)
        ctx.runner = runner
        ctx.mats = mats
        ctx.save_for_backward(psi)
        return psi

    @staticmethod
    def backward(ctx, g_psi):
        (psi,) = ctx.saved_tensors
        runner, mats = ctx.runner, ctx.mats
        need = [ctx.needs_input_grad[1 + i] for i in range(len(mats))]
        lam = g_psi.detach().to(runner.dtype).contiguous().clone()
        blocks = runner.reverse(psi, lam, mats, need)
        return (None, *[None if b is None else _grad_like(m, b) for m, b in zip(mats, blocks)])


class _EnergyFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, runner, terms, *mats):
        from .statevector import pauli_expectations
        psi = runner.forward_state(mats)
        e = pauli_expectations(psi, runner.n, terms).sum()
        ctx.runner, ctx.terms, ctx.mats = runner, terms, mats
        ctx.save_for_backward(psi)
        return e

    @staticmethod
    def backward(ctx, g_e):
        (psi,) = ctx.saved_tensors
        runner, terms, mats = ctx.runner, ctx.terms, ctx.mats
        L = _lib.lib()
        n = runner.n
        lam = torch.empty_like(psi)
        strings = "".join(s.lower() for _, s in terms).encode()
        coeff = _lib.double_array([c for c, _ in terms])
        _lib.check(L.qgb_pauli_apply(psi.data_ptr(), lam.data_ptr(), runner.code, n, strings, coeff, len(terms), 1, 0,
                                     _lib.stream_ptr(runner.device)), "pauli_apply")
        need = [ctx.needs_input_grad[2 + i] for i in range(len(mats))]
        blocks = runner.reverse(psi, lam, mats, need)
        scale = 2.0 * float(g_e)
        return (None, None, *[None if b is None else _grad_like(m, scale * b) for m, b in zip(mats, blocks)])


def _matrices(gates):
    return [g.matrix if torch.is_tensor(g.matrix) else torch.as_tensor(np.asarray(g.matrix, dtype=np.complex128))
            for g in gates]


def run_with_adjoint(sim):
    """Differentiable ``StatevectorSim.run``: the returned state carries an
    adjoint backward to every gate matrix that requires grad."""
    gates = _gate_list(sim)
    return _StateFn.apply(_Runner(sim, gates), *_matrices(gates))


def adjoint_energy(sim, terms):
    """Differentiable ``sum_t c_t <psi|P_t|psi>`` (float64) of ``sim``'s circuit."""
    gates = _gate_list(sim)
    return _EnergyFn.apply(_Runner(sim, gates), list(terms), *_matrices(gates))


# ------------------------------------------------------------ parameter-set batches

_KIND = {"RX": 1, "RY": 2, "RZ": 3, "RXX": 4, "RYY": 5, "RZZ": 6}


class BatchedAnsatz:
    """Energies and angle gradients of one parametrised circuit structure for
    many parameter sets at once (the reference differentiates one set at a time
    through torch autograd, ``applications/compilation.py:73-133``).

    ``gates``: ``(name, indices, p)`` per gate in execution order, ``name`` one of
    RX RY RZ RXX RYY RZZ with angle parameter index ``p``, or ``("fixed",
    indices, matrix)``. Gate matrices of every set are built on the device from
    the parameter tensor (``qgb_param_matrices``: ``expm(-i theta P)`` as in
    ``core/param_gates.py``); the forward pass applies each gate to all sets in
    one launch with per-set matrices; the reverse sweep (``lam = H psi``, then
    ``qgb_adjoint_step_batched`` per gate) carries all sets together and leaves
    each gate's matrix gradient, which ``qgb_param_grads`` maps to the angles.
    Memory: three states per set."""

    def __init__(self, n, gates, nparams=None, dtype=torch.complex64, device="cuda"):
        self.n = int(n)
        self.dtype, self.device = dtype, torch.device(device)
        if self.device.type != "cuda":
            raise _lib.QgbError("qaravan_gb300 runs on CUDA devices only")
        self.code = _lib.dtype_code(dtype)
        self.gates = [(g[0], [int(q) for q in g[1]], g[2]) for g in gates]
        kinds, pidx, fixed = [], [], []
        for i, (name, idx, p) in enumerate(self.gates):
            if len(idx) > 2:
                raise NotImplementedError("the adjoint sweep handles gates on one or two sites")
            if name == "fixed":
                kinds.append(0)
                pidx.append(0)
                fixed.append((i, np.asarray(p, dtype=np.complex128)))
            else:
                if _KIND[name] >= 4 and len(idx) != 2 or _KIND[name] < 4 and len(idx) != 1:
                    raise ValueError(f"{name} on {len(idx)} sites")
                kinds.append(_KIND[name])
                pidx.append(int(p))
        self.nparams = int(nparams) if nparams is not None else max([p for k, p in zip(kinds, pidx) if k] + [-1]) + 1
        self._kinds = torch.tensor(kinds, dtype=torch.int32, device=self.device)
        self._pidx = torch.tensor(pidx, dtype=torch.int32, device=self.device)
        self._fixed = fixed
        by_param = [[] for _ in range(self.nparams)]
        for g, (k, p) in enumerate(zip(kinds, pidx)):
            if k:
                by_param[p].append(g)
        ptr = np.cumsum([0] + [len(b) for b in by_param]).astype(np.int32)
        self._csr_ptr = torch.from_numpy(ptr).to(self.device)
        flat = np.array([g for b in by_param for g in b] or [0], dtype=np.int32)
        self._csr_gate = torch.from_numpy(flat).to(self.device)
        self._sites = [_lib.int_array(idx) for _, idx, _ in self.gates]
        self._need = [k != 0 for k in kinds]
        self.scratch = Scratch(self.device)

    @classmethod
    def hea(cls, n, layers, dtype=torch.complex64, device="cuda"):
        """The hardware-efficient ansatz of the adjoint benchmark: per layer RY(theta)
        then RZ(phi) on every qubit, then a CNOT ladder; parameter index
        2 * (l * n + q) + (0 theta, 1 phi), the flattening of ``workloads.hea_params``."""
        from .gates import CNOT
        gates = []
        for l in range(layers):
            for q in range(n):
                gates.append(("RY", [q], 2 * (l * n + q)))
                gates.append(("RZ", [q], 2 * (l * n + q) + 1))
            for q in range(n - 1):
                g = CNOT([q + 1, q], n)  # the gate object of workloads.hea_circuit (its own site order)
                gates.append(("fixed", list(g.indices), np.asarray(g.matrix, dtype=np.complex128)))
        return cls(n, gates, nparams=2 * layers * n, dtype=dtype, device=device)

    def _matrices(self, params, P):
        G = len(self.gates)
        mats = torch.zeros(P, G, 16, dtype=self.dtype, device=self.device)
        for i, m in self._fixed:
            mats[:, i, :m.size] = torch.as_tensor(m.reshape(-1)).to(self.dtype).to(self.device)
        _lib.check(_lib.lib().qgb_param_matrices(self._kinds.data_ptr(), self._pidx.data_ptr(), G, params.data_ptr(),
                                                 self.nparams, P, mats.data_ptr(), self.code, 16, 16 * G,
                                                 _lib.stream_ptr(self.device)), "param_matrices")
        return mats

    def energy_and_grad(self, params, terms):
        """``params``: (P, nparams) float64 (device or host). Returns float64 device
        tensors ``E`` (P,) = sum_t c_t <psi|P_t|psi> and ``dE/dparams`` (P, nparams)."""
        from .statevector import pauli_expectations
        L = _lib.lib()
        n, N = self.n, 2 ** self.n
        params = torch.as_tensor(params, dtype=torch.float64).to(self.device).contiguous()
        P = params.shape[0]
        if P < 1 or P > 65535:
            raise ValueError("1 to 65535 parameter sets")
        mats = self._matrices(params, P)
        st = _lib.stream_ptr(self.device)
        isz = mats.element_size()
        psi = torch.empty(P * N, dtype=self.dtype, device=self.device)
        _lib.check(L.qgb_init_basis(psi.data_ptr(), self.code, n, 0, P, N, st), "init")
        base = mats.data_ptr()
        set_stride = 16 * len(self.gates)
        for g, (_, idx, _) in enumerate(self.gates):
            _lib.check(L.qgb_op_action(psi.data_ptr(), self.code, n, self._sites[g], len(idx), base + g * 16 * isz,
                                       set_stride, P, N, st), "op_action")
        terms = list(terms)
        E = pauli_expectations(psi, n, terms, batch=P, stride=N).reshape(P, -1).sum(dim=1)
        lam = torch.empty_like(psi)
        strings = "".join(s.lower() for _, s in terms).encode()
        coeff = _lib.double_array([c for c, _ in terms])
        _lib.check(L.qgb_pauli_apply(psi.data_ptr(), lam.data_ptr(), self.code, n, strings, coeff, len(terms), P, N, st),
                   "pauli_apply")
        phi = psi  # uncomputed in place
        gblock = 32 * P  # doubles per gate: each set's 2 * d^2 back to back
        gmat = torch.zeros(len(self.gates) * gblock, dtype=torch.float64, device=self.device)
        nbytes = L.qgb_reduce_scratch_bytes(n, 32, P)
        scr = self.scratch.get(nbytes)
        for g in range(len(self.gates) - 1, -1, -1):
            idx = self.gates[g][1]
            out = gmat.data_ptr() + g * gblock * 8 if self._need[g] else None
            _lib.check(L.qgb_adjoint_step_batched(phi.data_ptr(), lam.data_ptr(), self.code, n, self._sites[g], len(idx),
                                                  base + g * 16 * isz, set_stride, P, N, out, scr.data_ptr(), nbytes,
                                                  st), "adjoint_step_batched")
        grad = torch.empty(P, self.nparams, dtype=torch.float64, device=self.device)
        gmat *= 2.0  # torch's convention: dE/dM = 2 sum lam conj(phi) for E = <psi|H|psi>
        _lib.check(L.qgb_param_grads(self._kinds.data_ptr(), self._csr_ptr.data_ptr(), self._csr_gate.data_ptr(),
                                     self.nparams, params.data_ptr(), P, gmat.data_ptr(), gblock // 2, grad.data_ptr(),
                                     st), "param_grads")
        return E, grad
