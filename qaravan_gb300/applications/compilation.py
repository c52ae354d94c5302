"""State-preparation compilation of the reference (``applications/compilation.py``)
on the GPU: the circuit ansatzes, the infidelity of an ansatz over pairs of
input/output states, and its optimisation by automatic differentiation.

``msp_infidelity`` with ``backend="torch"`` runs each input state through
``qaravan_gb300.tensorQ.StatevectorSim`` (complex64 on the GPU, results on the
CPU as the reference's torch path gives them), whose backward is the adjoint
sweep; ``msp_via_autodiff`` is the reference's Adam loop around it.

``msp_environment`` / ``msp_via_environments`` replace the reference's d^2
dense circuit unitaries per gate (``circ_to_mat`` with the gate set to each
matrix unit) by the equivalent partial overlap of the input state run up to
the gate and the output state pulled back through the rest of the circuit:
<out|S E_ij P|in> = sum_rest conj(lam[i, rest]) phi[j, rest]. The sweep keeps
the forward states and the pulled-back states of all pairs on the device as
one batch and moves both by one gate per step, so each gate costs two batched
gate applications and one batched partial overlap instead of a full circuit
unitary per matrix entry. Qubits only.
"""
from __future__ import annotations

from itertools import combinations

import numpy as np
import scipy.linalg
import torch

from ..circuits import Circuit, brickwall_skeleton
from ..environments import RunContext, _Dev
from ..gates import CNOT, RZ, U, Gate, embed_operator
from ..paulis import pauli_Z

__all__ = ["dressed_cnot_circ", "random_circ", "k_body_z", "rz_ansatz", "msp_infidelity", "msp_via_autodiff",
           "msp_environment", "msp_via_environments", "msp_job", "construct_unitary", "unitary_embedding",
           "msp_cost", "msp_optimize", "string_to_sv"]


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


def _pulled_back(dev, gates, states, batch):
    """``states`` <- (g_last ... g_first)^dagger ``states``: the last gate is undone first."""
    for g in reversed(gates):
        dev.op_action(np.asarray(g.matrix).conj().T, g.indices, states, batch)
    return states


def _run_forward(dev, gates, states, batch):
    for g in gates:
        dev.op_action(g.matrix, g.indices, states, batch)
    return states


def msp_environment(in_state, ansatz, out_state, gate_idx, dtype=torch.complex128, device="cuda"):
    """Environment of gate ``gate_idx`` for one input/output pair
    (``applications/compilation.py:135-146``): ``env[a, b]`` is <out| ansatz with
    the gate replaced by |b><a| |in>, i.e. the reference's matrix of
    <out|A(E_ij)|in> over (i, j), transposed. For a gate on k sites the result
    is 2^k x 2^k (the reference's d x d covers one site)."""
    dev = _Dev(ansatz.num_sites, dtype, device)
    gates = ansatz.gate_list
    phi = _run_forward(dev, gates[:gate_idx], dev.vec(in_state), 1)
    lam = _pulled_back(dev, gates[gate_idx + 1:], dev.vec(out_state), 1)
    return dev.partial_overlap(phi, lam, gates[gate_idx].indices)


def msp_via_environments(in_states, ansatz, out_states, num_sweeps=100, quiet=True, threshold=2e-8,
                         dtype=torch.complex128, device="cuda"):
    """Sweeps over the ansatz replacing every gate whose name starts with 'U' by
    the unitary that maximises Re tr(env U) for the summed environment of all
    pairs (``applications/compilation.py:148-187``); returns
    ``(ansatz, cost_list, term_cond)`` with the reference's stop rules (plateau
    of the relative decrease below 1e-4 after the second sweep, cost below
    ``threshold``) and its printed termination message."""
    n = ansatz.num_sites
    dev = _Dev(n, dtype, device)
    npairs = len(in_states)
    ins = torch.stack([dev.vec(s) for s in in_states])
    outs = torch.stack([dev.vec(s) for s in out_states])
    gates = ansatz.gate_list
    term_cond = None
    cost_list = []
    new_cost = None
    for sweep in range(num_sweeps):
        # phi: the inputs after the gates before the current one (already updated in
        # this sweep); lam: the outputs pulled back through the gates after it
        phi = ins.clone()
        lam = _pulled_back(dev, gates[1:], outs.clone(), npairs)
        for gate_idx, gate in enumerate(gates):
            if gate.name[0] == "U":
                env_list = dev.partial_overlap(phi, lam, gate.indices, batch=npairs)
                env = sum(env_list[p] for p in range(npairs))
                x, _, yh = np.linalg.svd(env)
                new_gate = yh.conj().T @ x.conj().T
                ansatz.update_gate(gate_idx, new_gate)
                new_cost = npairs - np.trace(env @ new_gate).real
                if new_cost < 0:
                    if np.abs(new_cost) < 1e-6:
                        new_cost = 1e-16
                    else:
                        print("Cost has become negative somehow")
            if gate_idx + 1 < len(gates):
                dev.op_action(gate.matrix, gate.indices, phi, npairs)
                nxt = gates[gate_idx + 1]
                dev.op_action(nxt.matrix, nxt.indices, lam, npairs)
        if new_cost is None:
            raise ValueError("the ansatz has no gate named U*")
        cost_list.append(np.sqrt(new_cost))
        if sweep > 1 and (cost_list[-2] - cost_list[-1]) / cost_list[-2] < 1e-4:
            term_cond = "cost function has plateaued"
            break
        if cost_list[-1] < threshold:
            term_cond = "cost function has converged"
            break
        if not quiet and sweep % 10 == 0:
            print(cost_list[-1])
    term_cond = "reached maximum number of sweeps" if term_cond is None else term_cond
    print(term_cond)
    return ansatz, cost_list, term_cond


def msp_job(in_states, out_states, skeleton, local_dim=2, max_sweeps=500, max_instances=50, threshold=2e-8,
            dtype=torch.complex128, device="cuda"):
    """Restarts of ``msp_via_environments`` from uniform random angles (NumPy's
    global random state) until one converges below ``threshold``
    (``applications/compilation.py:189-208``); returns ``(sols, data)``."""
    num_cnots = len(skeleton)
    num_sites = int(np.ceil(np.log(len(in_states[0])) / np.log(local_dim)))
    num_params = num_cnots * 6 + num_sites * 3
    sols, data = [], []
    for _ in range(max_instances):
        params = np.random.rand(num_params)
        ansatz = dressed_cnot_circ(skeleton, num_sites, params, local_dim)
        new_ansatz, cost_list, term_cond = msp_via_environments(in_states, ansatz, out_states, num_sweeps=max_sweeps,
                                                                threshold=threshold, dtype=dtype, device=device)
        sols.append(new_ansatz)
        data.append({"sol": new_ansatz, "cost_list": cost_list, "term_cond": term_cond})
        print(f"After optimization: {cost_list[-1]}")
        if cost_list[-1] < threshold:
            break
    return sols, data


def unitary_embedding(in_strings, out_states, local_dim=2):
    """Deprecated embedding of the map in_strings -> out_states into a square
    matrix: the columns of the given inputs are kept and the others are filled,
    in order, with a basis of the null space of (out^T in)^T
    (``applications/compilation.py:221-246``). The reference's own function
    raises NameError (its module does not import scipy); this one computes what
    its body describes."""
    print("This function is deprecated. Use construct_unitary instead.")
    dim = len(out_states[0])
    in_mat = np.array([string_to_sv(s, local_dim) for s in in_strings])
    a = np.array(out_states).T @ in_mat
    kept = {int(s, local_dim) for s in in_strings}
    space = scipy.linalg.null_space(a.T)
    fill = [c for c in range(dim) if c not in kept][:dim - len(in_strings)]
    for j, col in enumerate(fill):
        a[:, col] = space[:, j]
    return a


def msp_cost(params, skeleton, vecs, target, dtype=torch.complex128, device="cuda"):
    """Mean over ``vecs`` of ||C(params) v - t||, t = ``target @ v`` for a matrix
    target or the paired output state (``applications/compilation.py:248-260``);
    the inputs run through the circuit on the device as one batch."""
    num_qubits = int(np.log2(len(vecs[0])))
    ansatz = dressed_cnot_circ(skeleton, num_qubits, params)
    dev = _Dev(num_qubits, dtype, device)
    states = _run_forward(dev, ansatz.gate_list, torch.stack([dev.vec(v) for v in vecs]), len(vecs))
    out = states.cpu().numpy().astype(np.complex128)
    c = 0.0
    if type(target) == np.ndarray:
        for v, o in zip(vecs, out):
            c += np.linalg.norm(o - target @ v)
    else:
        for o, t in zip(out, target):
            c += np.linalg.norm(o - t)
    return c / len(vecs)


def msp_optimize(vecs, target, skeleton, num_reps=10, quiet=True, dtype=torch.complex128, device="cuda"):
    """Deprecated L-BFGS-B restarts on ``msp_cost`` from uniform random angles
    (``applications/compilation.py:262-287``); returns ``(results, vals)``."""
    from scipy.optimize import minimize
    print("SciPy optimizers are horrible. Use msp_via_autodiff or msp_via_environments instead.")
    num_cnots = len(skeleton)
    num_qubits = int(np.log2(len(vecs[0])))
    num_params = num_cnots * 6 + num_qubits * 3
    results, vals = [], []
    for _ in range(num_reps):
        params = np.random.rand(num_params)
        result = minimize(msp_cost, x0=params, args=(skeleton, vecs, target, dtype, device), method="L-BFGS-B",
                          options={"maxfun": 5000, "maxiter": 5000, "disp": False})
        results.append(result)
        vals.append(result.fun)
        if not quiet:
            print(result.fun)
    print(f"Best cost with {num_cnots} CNOTs is: {min(vals)}")
    return results, vals
