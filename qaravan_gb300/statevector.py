"""``StatevectorSim`` on GB300: the reference's API, run by the CUDA engine.

Mirrors ``tensorQ/statevector_sim.py:13-109`` of the reference:
constructor ``(circ, init_state=None, backend=..., device=...)``, ``run``,
``apply_gate``, ``get_statevector``, ``local_expectation``,
``one_local_expectation``, ``pauli_expectation``, ``normalize_state``,
``measure`` / ``measure_and_collapse``. The state is a flat CUDA tensor of
``2^n`` complex64 (default, the reference torch backend's dtype) or
complex128 amplitudes with site ``q`` on flat bit ``n-1-q``.

``run`` compiles the circuit once (fusion + tile sweeps, see
``qaravan_gb300.compiler``) and replays the compiled plan; the result equals
applying the gates one by one in layer order as ``BaseSim.run`` does
(``core/base_sim.py:30-53``), Reset included (projector, then renormalise,
``:25-28``). Gates whose matrices require grad make ``run`` differentiable
through the adjoint method (``qaravan_gb300.adjoint``).
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib
from .compiler import Op, compile_ops
from .engine import Executor, Scratch


def _to_np(m):
    if torch.is_tensor(m):
        return m.detach().cpu().numpy().astype(np.complex128)
    return np.asarray(m, dtype=np.complex128)


def circuit_ops(circ, n=None, build=False, nm=None):
    """Flatten a (reference or local) Circuit into the op sequence run() applies:
    layers if the circuit is built (or after building it), Reset as projector
    plus a renormalisation marker, ID noise carriers as identities (skipped).
    ``build``: the caller owns ``circ`` (a simulator's own copy) and it is built
    in place as ``BaseSim.run`` does (``core/base_sim.py:37``,
    ``core/circuits.py:86-95``: decomposition when ``requires_decomp``, layers,
    noise); otherwise an unbuilt circuit is layered on a copy."""
    if build and hasattr(circ, "build") and not getattr(circ, "built", False):
        circ.build(nm)
        return [g for layer in circ.layers for g in layer]
    if getattr(circ, "layers", None) is None and hasattr(circ, "construct_layers"):
        layers = None
        try:
            c2 = circ.copy()
            c2.construct_layers()
            layers = c2.layers
        except Exception:
            layers = None
        seq = [g for layer in layers for g in layer] if layers is not None else list(circ.gate_list)
    elif getattr(circ, "layers", None) is not None:
        seq = [g for layer in circ.layers for g in layer]
    else:
        seq = list(circ.gate_list)
    return seq


def _gate_requires_grad(g):
    """Whether a gate's matrix carries an autograd graph, without building a
    parametrised gate's matrix that has not been read yet (its angles decide)."""
    if getattr(g, "matrix_pending", lambda: False)():
        return any(torch.is_tensor(a) and a.requires_grad for a in g.angles)
    return torch.is_tensor(g.matrix) and g.matrix.requires_grad


def gates_to_ops(seq, n):
    ops = []
    top = n - 1
    for g in seq:
        name = g.name
        if name == "ID" and getattr(g, "nm", None) is not None:
            continue  # identity on a statevector (ID.matrix = eye)
        m = g.matrix
        m = m if type(m) is np.ndarray and m.dtype == np.complex128 else _to_np(m)
        idx = g.indices
        if m.shape[0] != 1 << len(idx):
            raise NotImplementedError("qaravan_gb300 supports qubits only (local_dim 2)")
        ops.append(Op([top - int(q) for q in idx], m))
        if name == "Reset" and getattr(g, "normalize", True):
            ops.append(None)
    return ops


class StatevectorSim:
    def __init__(self, circ, init_state=None, backend="torch", device="cuda", dtype=torch.complex64,
                 mode="auto", fusion_width=None, tile_bits=None, low_bits=None, nm=None):
        self.circ = circ.copy() if hasattr(circ, "copy") else circ
        self.num_sites = circ.num_sites
        self.local_dim = getattr(circ, "local_dim", 2)
        if self.local_dim != 2:
            raise NotImplementedError("qaravan_gb300 supports qubits only (local_dim 2)")
        self.init_state = init_state
        self.backend = backend
        self.device = torch.device(device)
        if self.device.type != "cuda":
            raise _lib.QgbError("qaravan_gb300 runs on CUDA devices only")
        self.dtype = dtype
        # auto: the autotuner's choice for this size and dtype (a cached measurement, a
        # measurement now with QGB_AUTOTUNE=1, else the defaults measured on GB300:
        # complex64 -> dense fused blocks, one HBM pass each: 6-qubit blocks on the tensor
        # cores from 13 qubits up (half the passes of 4-qubit blocks at the same speed per
        # pass, fastest measured on the 28-qubit brickwork), 4-qubit blocks on the CUDA cores
        # below; complex128 -> 3-qubit blocks grouped into shared-memory tile sweeps (float64
        # arithmetic dominates, so fewer passes win))
        if mode == "auto":
            from . import autotune
            a_mode, a_width, a_tile = autotune.choose_sv(circ.num_sites, dtype)
            mode = a_mode
            fusion_width = a_width if fusion_width is None else fusion_width
            tile_bits = a_tile if tile_bits is None else tile_bits
        if fusion_width is None:
            if dtype == torch.complex64:
                fusion_width = 6 if circ.num_sites >= 13 and _lib.lib().qgb_get_dense_impl() >= 1 else 4
            else:
                fusion_width = 3
        if tile_bits is None:
            tile_bits = 14 if dtype == torch.complex64 else 13
        self.mode, self.fusion_width, self.tile_bits, self.low_bits = mode, fusion_width, tile_bits, low_bits
        self.state = None
        self.ran = False
        self.nm = nm
        self._exec = None
        self._scratch = Scratch(self.device)

    # ---------------------------------------------------------- state
    def initialize_state(self):
        n = self.num_sites
        L = _lib.lib()
        st = _lib.stream_ptr(self.device)
        if self.init_state is None or isinstance(self.init_state, str):
            idx = 0 if self.init_state is None else int(self.init_state, 2)
            self.state = torch.empty(2 ** n, dtype=self.dtype, device=self.device)
            _lib.check(L.qgb_init_basis(self.state.data_ptr(), _lib.dtype_code(self.dtype), n, idx, 1, 0, st),
                       "init_basis")
        elif isinstance(self.init_state, (np.ndarray, torch.Tensor)):
            t = self.init_state if torch.is_tensor(self.init_state) else torch.from_numpy(np.asarray(self.init_state))
            self.state = t.reshape(-1).to(dtype=self.dtype, device=self.device).contiguous().clone()
        else:
            raise ValueError("init_state must be a NumPy array, Torch tensor, or a bitstring")

    def compile(self):
        if self._exec is None:
            seq = circuit_ops(self.circ, build=True, nm=self.nm)
            ops = gates_to_ops(seq, self.num_sites)
            kcap = 5 if self.dtype == torch.complex64 else 4
            plan = compile_ops(ops, self.num_sites, mode=self.mode, width=self.fusion_width,
                               tile_bits=self.tile_bits, low_bits=self.low_bits, max_sweep_k=kcap,
                               itemsize=torch.empty(0, dtype=self.dtype).element_size(), device_fusion=True)
            self._exec = Executor(plan, self.dtype, self.device)
        return self._exec

    def _needs_grad(self):
        return torch.is_grad_enabled() and any(_gate_requires_grad(g) for g in self.circ.gate_list)

    def run(self, progress_bar=False, debug=0):
        """Apply the circuit to the initial state (``core/base_sim.py:30-53``)."""
        if self._needs_grad():
            from .adjoint import run_with_adjoint
            self.state = run_with_adjoint(self)
        else:
            self.initialize_state()
            self.compile().run(self.state)
        self.ran = True
        return self.state.reshape([2] * self.num_sites)

    def apply_gate(self, gate):
        """Single-gate apply (``StatevectorSim.apply_gate``, ``:50-52``)."""
        if self.state is None:
            self.initialize_state()
        n = self.num_sites
        m = torch.as_tensor(_to_np(gate.matrix)).to(dtype=self.dtype, device=self.device).contiguous()
        sites = _lib.int_array(gate.indices)
        _lib.check(_lib.lib().qgb_op_action(self.state.data_ptr(), _lib.dtype_code(self.dtype), n, sites,
                                            len(gate.indices), m.data_ptr(), 0, 1, 0,
                                            _lib.stream_ptr(self.device)), "op_action")
        self._keep = m

    def get_statevector(self):
        if not self.ran:
            self.run(progress_bar=False)
        sv = self.state.reshape(2 ** self.num_sites)
        return sv.detach().cpu().numpy() if self.backend == "numpy" else sv

    def normalize_state(self):
        Executor(compile_ops([], self.num_sites), self.dtype, self.device).normalize(self.state)

    # ---------------------------------------------------- expectations
    def _ensure_ran(self):
        if not self.ran:
            self.run(progress_bar=False)

    def pauli_sum_expectation(self, terms):
        """``sum_t c_t <psi|P_t|psi>`` for ``terms = [(c_t, 'ixyz..'), ...]`` (float64)."""
        self._ensure_ran()
        return float(pauli_expectations(self.state, self.num_sites, terms).sum())

    def pauli_expectation(self, pauli_string):
        """``pauli_expectation`` (``:75-79``, ``pauli_expectation_sv`` ``:217-234``)."""
        self._ensure_ran()
        return float(pauli_expectations(self.state, self.num_sites, [(1.0, pauli_string)])[0])

    def local_expectation(self, local_ops):
        """<psi| (x)_i O_i |psi> (``:63-73``)."""
        self._ensure_ran()
        return product_expectation(self.state, self.num_sites, {i: local_ops[i] for i in range(self.num_sites)})

    def one_local_expectation(self, op, site):
        """<psi| O_site |psi> (``:81-94``)."""
        self._ensure_ran()
        return product_expectation(self.state, self.num_sites, {site: op})

    def measure(self, meas_sites, shots=1, rng=None):
        from .measure import measure_sv
        self._ensure_ran()
        return measure_sv(self.state, self.num_sites, meas_sites, shots=shots, rng=rng)

    def measure_and_collapse(self, meas_sites, rng=None):
        from .measure import measure_and_collapse_sv
        self._ensure_ran()
        return measure_and_collapse_sv(self.state, self.num_sites, meas_sites, rng=rng)

    def __str__(self):
        from .measure import pretty_print_sv
        self._ensure_ran()
        return pretty_print_sv(self.state.detach().cpu().numpy())


# ------------------------------------------------------------------ helpers

def pauli_expectations(state, n, terms, batch=1, stride=0):
    """float64 tensor of ``c_t <psi|P_t|psi>`` per term (and per state for batch > 1)."""
    L = _lib.lib()
    terms = list(terms)
    strings = "".join(s.lower() for _, s in terms).encode()
    coeff = _lib.double_array([c for c, _ in terms])
    out = torch.empty(batch * len(terms), dtype=torch.float64, device=state.device)
    nbytes = L.qgb_reduce_scratch_bytes(n, len(terms), batch)
    scratch = torch.empty((nbytes + 7) // 8, dtype=torch.float64, device=state.device)
    _lib.check(L.qgb_pauli_expectation(state.data_ptr(), _lib.dtype_code(state.dtype), n, strings, coeff,
                                       len(terms), batch, stride, out.data_ptr(), scratch.data_ptr(), nbytes,
                                       _lib.stream_ptr(state.device)), "pauli_expectation")
    return out.reshape(batch, len(terms)) if batch > 1 else out


def inner_product(a, b, n, batch=1, stride=0):
    L = _lib.lib()
    out = torch.empty(2 * batch, dtype=torch.float64, device=a.device)
    nbytes = L.qgb_reduce_scratch_bytes(n, 2, batch)
    scratch = torch.empty((nbytes + 7) // 8, dtype=torch.float64, device=a.device)
    _lib.check(L.qgb_inner_product(a.data_ptr(), b.data_ptr(), _lib.dtype_code(a.dtype), n, batch, stride,
                                   out.data_ptr(), scratch.data_ptr(), nbytes, _lib.stream_ptr(a.device)),
               "inner_product")
    return out


def product_expectation(state, n, site_ops):
    """Re <psi| (x)_q O_q |psi> for ``site_ops = {site: 2x2}``: copy, apply the
    single-site operators with one fused sweep, inner product in float64."""
    ops = [Op([n - 1 - q], _to_np(o)) for q, o in sorted(site_ops.items())]
    kcap = 5 if state.dtype == torch.complex64 else 4
    plan = compile_ops(ops, n, mode="sweep", width=1, tile_bits=13, max_sweep_k=kcap, itemsize=state.element_size())
    phi = state.reshape(-1).clone()
    Executor(plan, state.dtype, state.device).run(phi)
    ip = inner_product(state.reshape(-1), phi, n)
    return float(ip[0].item())
