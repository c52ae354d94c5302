"""The reference's ``qaravan.tensorQ`` surface for statevector and
density-matrix simulation, on the GPU.

``from qaravan_gb300.tensorQ import *`` replaces ``from qaravan.tensorQ import
*`` for the simulators (``StatevectorSim``, ``DensityMatrixSim``,
``MonteCarloSim``) and the free functions of ``tensorQ/statevector_sim.py``
(``:111-234``) and ``tensorQ/environments.py``, with the reference's names,
arguments and return types:

* NumPy inputs give NumPy results (computed in complex128 on the device);
  torch inputs give torch results on the input's device and dtype, and
  ``op_action`` carries torch autograd to both the state and the operator
  (the reference's torch backend differentiates through ``ncon``);
* every contraction runs in this package's CUDA kernels through the C ABI
  (``qgb_op_action``, ``qgb_partial_overlap``, ``qgb_pauli_expectation``,
  ``qgb_outcome_probs`` / ``qgb_sample_outcomes`` / ``qgb_collapse``);
  host-only helpers (``locs_to_indices``, ``all_zero_sv``, ``random_sv``)
  are restated in NumPy;
* measurements sample on the device from a seed drawn from NumPy's global
  random state (``numpy.random.seed`` makes them repeatable): the reference's
  distribution, not its ``numpy.random.choice`` stream.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib
from . import measure as _measure
from .density_matrix import DensityMatrixSim as _DensityMatrixSim
from .environments import environment_state_prep, environment_update, sv_environment
from .montecarlo import MonteCarloSim
from .paulis import pauli_masks
from .statevector import StatevectorSim as _StatevectorSim
from .statevector import inner_product

__all__ = ["StatevectorSim", "DensityMatrixSim", "MonteCarloSim", "locs_to_indices", "op_action", "all_zero_sv",
           "random_sv", "partial_overlap", "rdm_from_sv", "measure_sv", "measure_and_collapse_sv",
           "pauli_expectation_sv", "sv_environment", "environment_update", "environment_state_prep", "random_dm",
           "all_zero_dm", "partial_trace", "expectation"]


# --------------------------------------------------------------- simulators

class StatevectorSim(_StatevectorSim):
    """``StatevectorSim`` with the reference's constructor defaults
    (``tensorQ/statevector_sim.py:13-29``): ``backend="numpy"`` gives NumPy
    results in complex128 (the reference's NumPy path), ``backend="torch"``
    torch results in complex64 (its ``to_backend`` cast) on ``device``
    (default ``"cpu"``, differentiable when gate matrices require grad). The
    state itself lives and evolves on the GPU; ``dtype`` and the execution
    options of ``qaravan_gb300.StatevectorSim`` may be given as keywords."""

    def __init__(self, circ, init_state=None, backend="numpy", device="cpu", **kw):
        dtype = kw.pop("dtype", torch.complex128 if backend == "numpy" else torch.complex64)
        super().__init__(circ, init_state=init_state, backend=backend, device="cuda", dtype=dtype, **kw)
        self.result_device = torch.device(device)

    def _result(self, t):
        if self.backend == "numpy":
            return t.detach().cpu().numpy()
        return t.to(self.result_device) if t.device != self.result_device else t

    def run(self, progress_bar=True, debug=0):
        """Runs the circuit and returns the state as a rank-n array (``core/base_sim.py:30-53``)."""
        return self._result(super().run(progress_bar=progress_bar, debug=debug))

    def get_statevector(self):
        if not self.ran:
            super().run(progress_bar=False)
        return self._result(self.state.reshape(2 ** self.num_sites))


class DensityMatrixSim(_DensityMatrixSim):
    """``DensityMatrixSim(circ, init_state=None, nm=None)`` with the reference's
    NumPy results in complex128 (``tensorQ/density_matrix_sim.py:8-89``); the
    density matrix lives and evolves on the GPU."""

    def __init__(self, circ, init_state=None, nm=None, **kw):
        kw.setdefault("dtype", torch.complex128)
        super().__init__(circ, init_state=init_state, nm=nm, **kw)

    def run(self, progress_bar=True, debug=0):
        """Runs the circuit and returns rho as a rank-2n array (``core/base_sim.py:30-53``)."""
        out = super().run(progress_bar=progress_bar, debug=debug)
        return out.detach().cpu().numpy().reshape([2] * (2 * self.num_sites))

    def get_density_matrix(self):
        return super().get_density_matrix().detach().cpu().numpy()


# ----------------------------------------------------------------- helpers

def _device():
    if not torch.cuda.is_available():
        raise _lib.QgbError("qaravan_gb300 runs on CUDA devices only")
    return torch.device("cuda", torch.cuda.current_device())


def _qubits(sv, local_dim):
    if local_dim != 2:
        raise NotImplementedError("qaravan_gb300 supports qubits only (local_dim 2)")
    size = sv.numel() if torch.is_tensor(sv) else np.asarray(sv).size
    n = int(round(np.log2(size)))
    if 2 ** n != size:
        raise ValueError("state size is not a power of two")
    return n


def _on_device(x, dtype):
    """(flat device tensor of ``dtype``, how to give results back)."""
    if torch.is_tensor(x):
        dev = x.device if x.is_cuda else _device()
        t = x.reshape(-1).to(device=dev, dtype=dtype)
        return t, ("torch", x.device, x.dtype)
    t = torch.from_numpy(np.ascontiguousarray(np.asarray(x, dtype=np.complex128)).reshape(-1))
    return t.to(device=_device(), dtype=dtype), ("numpy", None, None)


def _give_back(t, how, shape):
    kind, device, dtype = how
    if kind == "numpy":
        return t.detach().cpu().numpy().reshape(shape)
    out = t.reshape(shape)
    return out.to(device=device, dtype=dtype) if (out.device != device or out.dtype != dtype) else out


def _state_dtype(sv):
    if torch.is_tensor(sv) and sv.dtype in (torch.complex64, torch.float32):
        return torch.complex64
    return torch.complex128


def _scratch(nbytes, device):
    return torch.empty(max(int(nbytes) // 8 + 1, 1), dtype=torch.float64, device=device)


def _apply(op2d, sites, state):
    """``state`` (flat, device) <- op on ``sites``, in place."""
    L = _lib.lib()
    m = op2d.contiguous()
    _lib.check(L.qgb_op_action(state.data_ptr(), _lib.dtype_code(state.dtype), _qubits(state, 2),
                               _lib.int_array(sites), len(sites), m.data_ptr(), 0, 1, 0,
                               _lib.stream_ptr(state.device)), "op_action")
    return state


def _overlap(a, b, sites):
    """Complex128 device tensor sum_rest a[r, rest] conj(b[c, rest]) on ``sites`` (as given)."""
    L = _lib.lib()
    n, k = _qubits(a, 2), len(sites)
    if k == 0:
        r = inner_product(b, a, n)  # sum conj(b) a
        return torch.complex(r[0], r[1]).reshape(1, 1)
    nbytes = max(L.qgb_partial_overlap_scratch_bytes(n, k, 1), L.qgb_reduce_scratch_bytes(n, 32, 1))
    scr = _scratch(nbytes, a.device)
    out = torch.empty(2 * 4 ** k, dtype=torch.float64, device=a.device)
    _lib.check(L.qgb_partial_overlap(a.data_ptr(), b.data_ptr(), _lib.dtype_code(a.dtype), n, _lib.int_array(sites),
                                     k, 1, 0, out.data_ptr(), scr.data_ptr(), scr.numel() * 8,
                                     _lib.stream_ptr(a.device)), "partial_overlap")
    return torch.complex(out[0::2], out[1::2]).reshape(2 ** k, 2 ** k)


class _OpActionFn(torch.autograd.Function):
    """out = U on ``sites`` applied to psi; backward: dL/dpsi* = U^H g and
    dL/dU = sum_rest g[r, rest] conj(psi[c, rest]) (torch's convention)."""

    @staticmethod
    def forward(ctx, op2d, psi, sites):
        ctx.sites = sites
        ctx.save_for_backward(op2d, psi)
        return _apply(op2d, sites, psi.detach().clone())

    @staticmethod
    def backward(ctx, g):
        op2d, psi = ctx.saved_tensors
        g = g.contiguous()
        g_psi = _apply(op2d.detach().conj().transpose(0, 1), ctx.sites, g.clone()) if ctx.needs_input_grad[1] else None
        g_op = None
        if ctx.needs_input_grad[0]:
            g_op = _overlap(g, psi.detach().contiguous(), ctx.sites).to(op2d.dtype)
        return g_op, g_psi, None


# ----------------------------------------------------------- free functions

def locs_to_indices(locs, n):
    """ncon labels for a gate on ascending sites ``locs`` of an n-site state
    (``tensorQ/statevector_sim.py:111-122``): (gate legs, state legs)."""
    shifted = [int(q) + 1 for q in locs]
    gate = [-q for q in shifted] + shifted
    bounds = [0] + shifted
    state = []
    for i, q in enumerate(shifted):
        state += [-j for j in range(bounds[i] + 1, q)]
        state.append(q)
    state += [-j for j in range(bounds[-1] + 1, n + 1)]
    return gate, state


def op_action(op, indices, sv, local_dim=2):
    """``op`` (2^k x 2^k, or rank-2k) on sites ``indices`` of ``sv`` (flat or
    rank-n), out of place (``tensorQ/statevector_sim.py:124-140``): the result
    has ``sv``'s shape; with torch inputs it is differentiable."""
    n = _qubits(sv, local_dim)
    indices = [int(q) for q in (indices if isinstance(indices, (list, tuple, np.ndarray)) else [indices])]
    k = len(indices)
    dtype = _state_dtype(sv)
    psi, how = _on_device(sv, dtype)
    if torch.is_tensor(op):
        m = op.reshape(2 ** k, 2 ** k).to(device=psi.device, dtype=dtype)
    else:
        m = torch.from_numpy(np.asarray(op, dtype=np.complex128).reshape(2 ** k, 2 ** k)).to(psi.device, dtype)
    shape = tuple(sv.shape)
    if torch.is_tensor(sv) or torch.is_tensor(op):
        out = _OpActionFn.apply(m, psi, indices)
        if how[0] == "numpy":  # torch operator, NumPy state: the state comes back as torch on the device
            return out.reshape(shape)
        return _give_back(out, how, shape)
    return _give_back(_apply(m, indices, psi.clone()), how, shape)


def all_zero_sv(num_sites, local_dim=2, dense=False, backend="numpy"):
    """|0...0> (``tensorQ/statevector_sim.py:142-148``): dense NumPy, or a
    SciPy CSC column."""
    if dense:
        sv = np.zeros(local_dim ** num_sites)
        sv[0] = 1.0
        return sv
    from scipy.sparse import csc_matrix
    return csc_matrix(([1], ([0], [0])), shape=(local_dim ** num_sites, 1))


def random_sv(num_sites, local_dim=2):
    """Normalised state with uniform [0, 1) real and imaginary parts from
    NumPy's global random state (``tensorQ/statevector_sim.py:150-153``)."""
    sv = np.random.rand(local_dim ** num_sites) + 1j * np.random.rand(local_dim ** num_sites)
    return sv / np.linalg.norm(sv)


def partial_overlap(sv1, sv2, local_dim=2, skip=None):
    """sum over the other sites of sv1 conj(sv2), a 2^k x 2^k matrix over the
    ``skip`` sites in ascending order (``tensorQ/statevector_sim.py:155-180``)."""
    _qubits(sv1, local_dim)
    sites = sorted(int(q) for q in skip) if skip is not None else []
    dtype = torch.complex128 if (_state_dtype(sv1) == torch.complex128 or _state_dtype(sv2) == torch.complex128) \
        else torch.complex64
    a, how = _on_device(sv1, dtype)
    b, _ = _on_device(sv2, dtype)
    out = _overlap(a.contiguous(), b.contiguous(), sites)
    if how[0] == "numpy":
        return out.cpu().numpy()
    return out.to(device=how[1])


def rdm_from_sv(sv, sites, local_dim=2):
    """Reduced density matrix of ``sites`` (ascending) (``:182-183``)."""
    return partial_overlap(sv, sv, local_dim=local_dim, skip=sites)


def random_dm(n):
    """a a^H / Tr with uniform [0, 1) real and imaginary parts of a from NumPy's
    global random state (``tensorQ/density_matrix_sim.py:108-111``)."""
    a = np.random.rand(2 ** n, 2 ** n) + 1.j * np.random.rand(2 ** n, 2 ** n)
    a = a @ a.conj().T
    return a / np.trace(a)


def all_zero_dm(n, local_dim=2):
    """|0..0><0..0| (``tensorQ/density_matrix_sim.py:113-116``)."""
    dm = np.zeros((local_dim ** n, local_dim ** n))
    dm[0, 0] = 1.0
    return dm


def partial_trace(dm, sites, local_dim=2):
    """Reduced density matrix of the kept ``sites`` (ascending) of a host
    density matrix (``tensorQ/density_matrix_sim.py:118-145``): the real trace
    for no site, ``dm`` itself for all sites."""
    size = int(round(np.log(dm.shape[0]) / np.log(local_dim)))
    sites = sorted(int(q) for q in sites)
    if not sites:
        return np.trace(dm).real
    if len(sites) == size:
        return dm
    t = np.asarray(dm).reshape([local_dim] * (2 * size))
    rest = [q for q in range(size) if q not in sites]
    t = t.transpose(sites + rest + [size + q for q in sites] + [size + q for q in rest])
    d, r = local_dim ** len(sites), local_dim ** len(rest)
    return np.einsum("arbr->ab", t.reshape(d, r, d, r))


def expectation(dm, op):
    """Re Tr(dm op) (``tensorQ/density_matrix_sim.py:147-148``)."""
    return np.trace(dm @ op).real


def _global_seed():
    return int(np.random.randint(0, 2 ** 62, dtype=np.int64))


def measure_sv(sv, meas_sites, shots=1):
    """Outcome string(s) of measuring ``meas_sites`` (``:185-193``): bits of
    the measured sites in ascending order; one string for ``shots=1``."""
    n = _qubits(sv, 2)
    psi, _ = _on_device(sv, _state_dtype(sv))
    probs = _measure.outcome_probs(psi, n, meas_sites)
    idx = _measure.sample_outcomes(probs, shots, _global_seed()).cpu().numpy()
    outs = [str(np.binary_repr(int(i), width=len(meas_sites))) for i in idx]
    return outs[0] if shots == 1 else outs


def measure_and_collapse_sv(sv, meas_sites, local_dim=2):
    """(outcome string, collapsed and renormalised state of the other sites)
    (``:195-215``; the projector reads the string in ``meas_sites`` order)."""
    n = _qubits(sv, local_dim)
    psi, how = _on_device(sv, _state_dtype(sv))
    meas_sites = [int(q) for q in meas_sites]
    probs = _measure.outcome_probs(psi, n, meas_sites)
    outcome = str(np.binary_repr(int(_measure.sample_outcomes(probs, 1, _global_seed()).cpu().item()),
                                 width=len(meas_sites)))
    out = _measure.collapse_sv(psi, n, meas_sites, outcome, probs)
    m = n - len(meas_sites)
    shape = (2 ** m,) if (not hasattr(sv, "ndim") or sv.ndim == 1) else (2,) * m
    return outcome, _give_back(out, how, shape)


def pauli_expectation_sv(sv, pauli_string):
    """Re <sv| P |sv> for a lower-case Pauli string over all sites (``:217-234``)."""
    n = _qubits(sv, 2)
    if len(pauli_string) != n:
        raise AssertionError("Pauli string length must match number of qubits in statevector")
    pauli_masks(pauli_string)  # validates the characters
    psi, how = _on_device(sv, _state_dtype(sv))
    L = _lib.lib()
    scr = _scratch(L.qgb_reduce_scratch_bytes(n, 1, 1), psi.device)
    out = torch.empty(1, dtype=torch.float64, device=psi.device)
    _lib.check(L.qgb_pauli_expectation(psi.data_ptr(), _lib.dtype_code(psi.dtype), n, pauli_string.lower().encode(),
                                       None, 1, 1, 0, out.data_ptr(), scr.data_ptr(), scr.numel() * 8,
                                       _lib.stream_ptr(psi.device)), "pauli_expectation")
    v = out.cpu()[0]
    return np.float64(v.item()) if how[0] == "numpy" else v
