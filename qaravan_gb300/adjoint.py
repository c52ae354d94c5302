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
