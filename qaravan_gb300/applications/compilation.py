"""State-preparation compilation of the reference (``applications/compilation.py``)
on the GPU: the circuit ansatzes, the infidelity of an ansatz over pairs of
input/output states, and its optimisation by automatic differentiation.

``msp_infidelity`` with ``backend="torch"`` runs each input state through
``qaravan_gb300.tensorQ.StatevectorSim`` (complex64 on the GPU, results on the
CPU as the reference's torch path gives them), whose backward is the adjoint
sweep; ``msp_via_autodiff`` is the reference's Adam loop around it. Qubits only.
"""
from __future__ import annotations

from itertools import combinations

import numpy as np
import scipy.linalg
import torch

from ..circuits import Circuit, brickwall_skeleton
from ..environments import RunContext
from ..gates import CNOT, RZ, U, Gate, embed_operator
from ..paulis import pauli_Z

__all__ = ["dressed_cnot_circ", "random_circ", "k_body_z", "rz_ansatz", "msp_infidelity", "msp_via_autodiff",
           "construct_unitary", "string_to_sv"]


def string_to_sv(string, local_dim=2):
    """Basis state of a digit string (``core/utils.py:46-50``)."""
    sv = np.zeros(local_dim ** len(string))
    sv[int(string, local_dim)] = 1.0
    return sv


def dressed_cnot_circ(skeleton, num_qubits, params, local_dim=2):
    """U gates on both sites of every skeleton pair followed by its CNOT, then a
    final U on every site; 3 angles per U (``applications/compilation.py:21-38``)."""
    if local_dim != 2:
        raise NotImplementedError("qaravan_gb300 supports qubits only (local_dim 2)")
    counter = 0
    gates = []
    for pair in skeleton:
        gates.append(U(pair[0], *params[3 * counter:3 * (counter + 1)]))
        counter += 1
        gates.append(U(pair[1], *params[3 * counter:3 * (counter + 1)]))
        counter += 1
        gates.append(CNOT(pair, num_qubits))
    for i in range(num_qubits):
        gates.append(U(i, *params[3 * counter:3 * (counter + 1)]))
        counter += 1
    return Circuit(gates, num_qubits)


def random_circ(n, depth):
    """``dressed_cnot_circ`` on ``brickwall_skeleton(n, depth)`` with uniform
    angles from NumPy's global random state (``:40-44``; the skeleton call is the
    reference's, a lattice of n x depth sites)."""
    skeleton = brickwall_skeleton(n, depth)
    num_params = len(skeleton) * 6 + n * 3
    return dressed_cnot_circ(skeleton, n, np.random.rand(num_params))


def k_body_z(n, k):
    """(name, dense operator) of every k-body Z string on n sites (``:46-51``)."""
    ops = []
    for indices in combinations(range(n), k):
        name = "".join("Z" if i in indices else "I" for i in range(n))
        ops.append((name, embed_operator(n, list(indices), [pauli_Z] * k, dense=True)))
    return ops


def rz_ansatz(n, params, body=1):
    """RZ on every site, then exp(-i theta Z..Z) for every k-body Z string up to
    ``body`` (``:53-64``)."""
    gates = [RZ(i, params[i]) for i in range(n)]
    for k in range(2, body + 1):
        extra = []
        for i, (name, mat) in enumerate(k_body_z(n, k)):
            extra.append(Gate("R" + name, np.arange(n), scipy.linalg.expm(-1.j * params[len(gates) + i] * mat)))
        gates += extra
    return Circuit(gates, n)


def msp_infidelity(params, skeleton, in_states, out_states, backend="numpy"):
    """Mean of 1 - |<out|C(params)|in>|^2 over the pairs (``:73-90``); with
    ``backend="torch"`` differentiable in ``params``."""
    from ..tensorQ import StatevectorSim
    num_qubits = int(np.log2(len(in_states[0])))
    ansatz = dressed_cnot_circ(skeleton, num_qubits, params, local_dim=2)
    infid = 0
    for in_state, out_state in zip(in_states, out_states):
        sim = StatevectorSim(ansatz, backend=backend, init_state=in_state)
        sim.run(progress_bar=False)
        sv = sim.get_statevector()
        if backend == "torch":
            target = torch.tensor(out_state, dtype=torch.complex128)
            infid += 1 - torch.abs(torch.dot(sv.to(torch.complex128).conj(), target)) ** 2
        else:
            infid += 1 - np.abs(np.dot(sv.conj(), out_state)) ** 2
    return infid / len(in_states)


def msp_via_autodiff(in_states, out_states, cnot_skeleton, init_params=None, lr=0.05, num_sweeps=100,
                     threshold=2e-8, context=None):
    """Adam on ``msp_infidelity`` (``:92-131``); returns (params, run_state).
    The run context keeps the reference's stop rules (plateau 1e-8, absolute
    ``threshold``) without checkpoint files."""
    if init_params is None:
        num_qubits = int(np.log2(len(in_states[0])))
        init_params = torch.nn.Parameter(torch.randn(len(cnot_skeleton) * 6 + num_qubits * 3))
    elif not isinstance(init_params, torch.nn.Parameter):
        init_params = torch.nn.Parameter(torch.tensor(init_params, dtype=torch.float64))
    optimizer = torch.optim.Adam([init_params], lr=lr)
    context = context if context is not None else RunContext(
        progress_interval=10, max_iter=num_sweeps, convergence_check=True, stop_ratio=1e-8,
        stop_absolute=threshold, quiet=True)
    cost_list = []
    run_state = {"cost_list": cost_list, "step": context.step}
    while True:
        cost = msp_infidelity(init_params, cnot_skeleton, in_states, out_states, backend="torch")
        cost_list.append(cost.item())
        optimizer.zero_grad()
        cost.backward()
        optimizer.step()
        run_state["step"] += 1
        run_state["cost_list"] = cost_list
        if context.step_update(run_state):
            break
    return init_params, run_state


def construct_unitary(in_strings, out_states, local_dim=2):
    """A unitary taking each basis state of ``in_strings`` to its output state
    (QR of out^T in, the given columns kept) (``:202-212``)."""
    in_mat = np.array([string_to_sv(s, local_dim) for s in in_strings])
    out_mat = np.array(out_states)
    a = out_mat.T @ in_mat
    q, _ = np.linalg.qr(a, mode="reduced")
    for col in [int(s, local_dim) for s in in_strings]:
        q[:, col] = a[:, col]
    return q
