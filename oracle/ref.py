"""NumPy complex128 restatement of the reference's hot-path algorithms.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).

Every function follows the reference file and lines in its docstring, using
the same contraction labels through ``oracle.ncon`` (tensordot + transpose),
so it is also the reference's CPU algorithm when timed as the CPU baseline.
Gate objects are duck-typed: ``.name``, ``.indices``, ``.matrix``, plus
``.nm/.time/.dd`` for noise carriers and ``.normalize`` for resets.
"""
from __future__ import annotations

import numpy as np

from .ncon import ncon, permute

PAULI = {
    'i': np.eye(2, dtype=complex),
    'x': np.array([[0, 1], [1, 0]], dtype=complex),
    'y': np.array([[0, -1j], [1j, 0]], dtype=complex),
    'z': np.array([[1, 0], [0, -1]], dtype=complex),
}


def _np(m):
    try:
        import torch
        if torch.is_tensor(m):
            return m.detach().cpu().numpy()
    except Exception:  # pragma: no cover
        pass
    return np.asarray(m)


# ------------------------------------------------------------- statevector

def locs_to_indices(locs, n):
    """``tensorQ/statevector_sim.py:111-122``."""
    shifted = [loc + 1 for loc in locs]
    gate_indices = [-i for i in shifted] + shifted
    bounds = [0] + shifted
    tensor_indices = []
    for i in range(len(shifted)):
        tensor_indices += [-j for j in range(bounds[i] + 1, bounds[i + 1])]
        tensor_indices.append(shifted[i])
    tensor_indices += [-j for j in range(bounds[-1] + 1, n + 1)]
    return gate_indices, tensor_indices


def op_action(op, indices, sv, local_dim=2):
    """``tensorQ/statevector_sim.py:124-140``: sort the indices, permute the
    operator's legs to match, one ncon contraction."""
    op = _np(op)
    k = len(indices)
    if op.ndim != 2 * k:
        op = op.reshape(*[local_dim] * 2 * k)
    n = sv.ndim if sv.ndim > 1 else int(round(np.log(len(sv)) / np.log(local_dim)))
    state = sv.reshape(*[local_dim] * n) if sv.ndim == 1 else sv
    sorted_idx = sorted(indices)
    order = [list(indices).index(i) for i in sorted_idx]
    op = permute(op, order + [i + k for i in order])
    gi, si = locs_to_indices(sorted_idx, n)
    out = ncon((op, state), (gi, si))
    return out.reshape(local_dim ** n) if sv.ndim == 1 else out


def op_action_torch(op, indices, state):
    """The torch-backend form of ``op_action`` (``tensorQ/statevector_sim.py:124-140``
    with ``ncon_torch`` on torch tensors): differentiable by torch autograd.
    ``state`` is the rank-n tensor ``[2]*n``."""
    k = len(indices)
    n = state.ndim
    op = op.reshape(*[2] * 2 * k)
    sorted_idx = sorted(indices)
    order = [list(indices).index(i) for i in sorted_idx]
    op = permute(op, order + [i + k for i in order])
    gi, si = locs_to_indices(sorted_idx, n)
    return ncon((op, state), (gi, si))


def construct_layers(gates):
    """Greedy ASAP layering, ``core/circuits.py:42-63``."""
    layers = []
    for g in gates:
        li = len(layers) - 1
        gi = set(g.indices)
        while li >= 0 and not (gi & {i for h in layers[li] for i in h.indices}):
            li -= 1
        if li < len(layers) - 1:
            layers[li + 1].append(g)
        else:
            layers.append([g])
    return layers


def initial_sv(n, init_state=None):
    """``tensorQ/statevector_sim.py:31-48`` (bitstring or array or |0...0>)."""
    if init_state is None:
        sv = np.zeros(2 ** n, dtype=np.complex128)
        sv[0] = 1.0
    elif isinstance(init_state, str):
        sv = np.zeros(2 ** n, dtype=np.complex128)
        sv[int(init_state, 2)] = 1.0
    else:
        sv = np.asarray(init_state, dtype=np.complex128).reshape(-1).copy()
    return sv.reshape([2] * n)


def normalize_sv(state):
    """``tensorQ/statevector_sim.py:107-109``."""
    return state / np.linalg.norm(state.reshape(-1))


def run_sv(gates, n, init_state=None, layered=True):
    """``core/base_sim.py:30-53``: layer loop; Reset = projector + renormalise
    (``:25-28``); ``apply_gate`` = ``op_action`` (``statevector_sim.py:50-52``)."""
    state = initial_sv(n, init_state)
    seq = [g for layer in construct_layers(gates) for g in layer] if layered else list(gates)
    for g in seq:
        state = op_action(g.matrix, g.indices, state)
        if g.name == "Reset" and getattr(g, "normalize", True):
            state = normalize_sv(state)
    return state.reshape(2 ** n)


def local_expectation(sv, local_ops):
    """``tensorQ/statevector_sim.py:63-73``: <psi| (x)_i O_i |psi>."""
    n = int(round(np.log2(sv.size)))
    state = sv.reshape([2] * n)
    right = state.copy()
    for i in range(n):
        si = [-(j + 1) for j in range(n)]
        si[i] = 1
        right = ncon((_np(local_ops[i]), right), ([-(i + 1), 1], si))
    lab = list(range(1, n + 1))
    return ncon((state.conj(), right), (lab, lab)).real


def one_local_expectation(sv, op, site):
    """``tensorQ/statevector_sim.py:81-94``."""
    n = int(round(np.log2(sv.size)))
    state = sv.reshape([2] * n)
    si = [-(j + 1) for j in range(n)]
    si[site] = 1
    right = ncon((_np(op), state), ([-(site + 1), 1], si))
    lab = list(range(1, n + 1))
    return ncon((state.conj(), right), (lab, lab)).real


def pauli_expectation_sv(sv, pauli_string):
    """``tensorQ/statevector_sim.py:217-234``."""
    n = int(round(np.log2(sv.size)))
    assert len(pauli_string) == n
    t = sv.reshape([2] * n)
    right = t.copy()
    for i in range(n):
        if pauli_string[i] == 'i':
            continue
        si = [-(j + 1) for j in range(n)]
        si[i] = 1
        right = ncon((PAULI[pauli_string[i]], right), ([-(i + 1), 1], si))
    lab = list(range(1, n + 1))
    return ncon((t.conj(), right), (lab, lab)).real


def pauli_sum_expectation(sv, terms):
    return float(sum(c * pauli_expectation_sv(sv, s) for c, s in terms))


def pauli_sum_apply(sv, terms):
    """H|psi> for ``terms = [(coeff, pstr)]`` by per-site contractions."""
    n = int(round(np.log2(sv.size)))
    out = np.zeros_like(sv)
    for c, s in terms:
        t = sv.reshape([2] * n)
        for i, ch in enumerate(s):
            if ch != 'i':
                t = op_action(PAULI[ch], [i], t)
        out = out + c * t.reshape(-1)
    return out


def partial_overlap(sv1, sv2, skip=None, local_dim=2):
    """``tensorQ/statevector_sim.py:155-180``: M[a, b] = sum_rest sv1[a, rest] conj(sv2[b, rest])."""
    n = int(round(np.log(len(sv1)) / np.log(local_dim)))
    sites = sorted(skip) if skip is not None else []
    psi = sv1.reshape([local_dim] * n)
    phic = sv2.reshape([local_dim] * n).conj()
    pl, ql = [0] * n, [0] * n
    nc, nf = 1, -1
    for i in range(n):
        if i in sites:
            pl[i] = nf
            ql[i] = nf - len(sites)
            nf -= 1
        else:
            pl[i] = ql[i] = nc
            nc += 1
    out = ncon([psi, phic], [pl, ql])
    kd = local_dim ** len(sites)
    return np.asarray(out).reshape((kd, kd))


def measure_probs(sv, meas_sites):
    """Outcome probabilities of ``measure_sv`` (``tensorQ/statevector_sim.py:185-193``)."""
    return np.real(np.diag(partial_overlap(sv, sv, skip=meas_sites)))


def collapse_sv(sv, meas_sites, outcome):
    """Post-measurement state of ``measure_and_collapse_sv`` for a given outcome
    (``tensorQ/statevector_sim.py:195-215``); measured sites are removed."""
    from functools import reduce
    n = int(round(np.log2(sv.size)))
    bras = [np.array([1, 0]) if b == '0' else np.array([0, 1]) for b in outcome]
    bra = reduce(np.kron, bras).reshape([2] * len(bras))
    state = sv.reshape([2] * n)
    sidx = sorted(meas_sites)
    order = [list(meas_sites).index(i) for i in sidx]
    bra = permute(bra, order)
    gi, si = locs_to_indices(sidx, n)
    out = ncon((bra, state), (gi[len(gi) // 2:], si))
    out = out / np.linalg.norm(out)
    return out.reshape(2 ** (n - len(meas_sites)))


# ------------------------------------------------------------ density matrix

def generate_gate_indices(locs, n):
    """``tensorQ/density_matrix_sim.py:91-99``."""
    numbers = list(range(1, 2 * len(locs) + 1))
    contracted = sorted(numbers)[-len(numbers) // 2:] + sorted(numbers)[:len(numbers) // 2]
    numbers = [int(l) + 1 for l in locs] + [int(l) + n + 1 for l in locs]
    largest, smallest = sorted(numbers)[-len(numbers) // 2:], sorted(numbers)[:len(numbers) // 2]
    return [-i for i in largest + smallest] + contracted


def generate_state_indices(locs, n):
    """``tensorQ/density_matrix_sim.py:101-107``."""
    si = [-i for i in range(1, 2 * n + 1)]
    pos = 1
    for loc in locs:
        si[loc] = pos
        si[loc + n] = pos + len(locs)
        pos += 1
    return si


def to_superop(matrix):
    """``core/gates.py:43-44``: ``kron(conj M, M)``."""
    m = _np(matrix)
    return np.kron(m.conj(), m)


def channel_superop(kraus):
    """``core/noise.py:10-13``: sum of ``kron(conj K, K)``."""
    return sum(np.kron(_np(k).conj(), _np(k)) for k in kraus)


def dm_apply_superop(rho, superop, locs, n):
    """``tensorQ/density_matrix_sim.py:38-42``: one ncon of the superoperator
    (reshaped to ``[2]*4k``) with the rank-2n state."""
    k = len(locs)
    s = _np(superop).reshape([2] * 4 * k)
    return ncon((s, rho), (generate_gate_indices(locs, n), generate_state_indices(locs, n)))


def initial_dm(n, init_state=None):
    """``tensorQ/density_matrix_sim.py:12-36``."""
    if init_state is None:
        dm = np.zeros((2 ** n, 2 ** n), dtype=np.complex128)
        dm[0, 0] = 1.0
    elif isinstance(init_state, str):
        sv = np.zeros(2 ** n)
        sv[int(init_state, 2)] = 1.0
        dm = np.outer(sv, sv.conj()).astype(np.complex128)
    else:
        dm = np.asarray(init_state, dtype=np.complex128).reshape(2 ** n, 2 ** n)
    return dm.reshape([2] * 2 * n)


def dm_normalize(rho, n):
    """``tensorQ/density_matrix_sim.py:85-89``: divide by the real trace."""
    dm = rho.reshape(2 ** n, 2 ** n)
    return (dm / np.trace(dm).real).reshape([2] * 2 * n)


def gate_superop(g):
    if g.name == "ID" and getattr(g, "nm", None) is not None:
        return _np(g.nm.get_superop(g.time, getattr(g, "dd", False)))
    return to_superop(g.matrix)


def run_dm(ops, n, init_state=None, layered=True):
    """``DensityMatrixSim.run`` (``core/base_sim.py:30-53`` with
    ``density_matrix_sim.py:38-42``) over an explicit op sequence; noise
    carriers (``ID`` with ``.nm``) contribute their channel superoperator."""
    rho = initial_dm(n, init_state)
    seq = [g for layer in construct_layers(ops) for g in layer] if layered else list(ops)
    for g in seq:
        rho = dm_apply_superop(rho, gate_superop(g), g.indices, n)
        if g.name == "Reset" and getattr(g, "normalize", True):
            rho = dm_normalize(rho, n)
    return rho.reshape(2 ** n, 2 ** n)


def dm_apply_gate_then_channels(rho, n, g, channel_kraus_per_qubit):
    """Oracle recipe for per-gate noise: apply ``g``, then for each qubit of
    the gate apply each listed single-qubit channel in order."""
    rho = dm_apply_superop(rho, to_superop(g.matrix), g.indices, n)
    for q in g.indices:
        for kraus in channel_kraus_per_qubit:
            rho = dm_apply_superop(rho, channel_superop(kraus), [q], n)
    return rho


def dm_one_local_expectation(dm, op, site):
    """``tensorQ/density_matrix_sim.py:60-70``: Tr(O_site rho)."""
    n = int(round(np.log2(dm.shape[0])))
    rho = dm.reshape([2] * 2 * n)
    si = [-(j + 1) for j in range(2 * n)]
    si[site] = 1
    mod = ncon((_np(op), rho), ([-(site + 1), 1], si))
    return np.trace(mod.reshape(2 ** n, 2 ** n)).real


def dm_local_expectation(dm, local_ops):
    """``tensorQ/density_matrix_sim.py:49-58``: Tr((x)_i O_i rho)."""
    n = int(round(np.log2(dm.shape[0])))
    rho = dm.reshape([2] * 2 * n)
    for i in range(n):
        si = [-(j + 1) for j in range(2 * n)]
        si[i] = 1
        rho = ncon((_np(local_ops[i]), rho), ([-(i + 1), 1], si))
    return np.trace(rho.reshape(2 ** n, 2 ** n)).real


def dm_global_expectation(dm, op):
    """``tensorQ/density_matrix_sim.py:72-76``."""
    return np.trace(dm @ _np(op)).real


def dm_pauli_expectation(dm, pstr):
    from functools import reduce
    P = reduce(np.kron, [PAULI[c] for c in pstr])
    return np.trace(dm @ P).real


def purity(dm):
    return float(np.real(np.trace(dm @ dm)))


# ------------------------------------------------------------- trajectories

def mc_expectation_sample(gates, n, nm, obs, rng):
    """One ``MonteCarloSim.expectation_sample`` (``tensorQ/monte_carlo_sim.py:14-35``):
    layer the circuit, interleave one sampled Pauli layer after every layer,
    run a statevector, return <psi|obs|psi>. ``nm.sample_string(rng)`` gives
    the n-site Pauli string."""
    layers = construct_layers(gates)
    state = initial_sv(n)
    for layer in layers:
        for g in layer:
            state = op_action(g.matrix, g.indices, state)
        s = nm.sample_string(rng)
        for i, ch in enumerate(s):
            if ch != 'i':
                state = op_action(PAULI[ch], [i], state)
    sv = state.reshape(-1)
    return np.vdot(sv, _np(obs) @ sv).real


# --------------------------------------------------------------- gradients

def energy(gates, n, terms):
    return pauli_sum_expectation(run_sv(gates, n), terms)


def matrix_gradients(gates, n, terms):
    """Exact dL/dM for L = <psi|H|psi>, returned in torch's convention for a
    real loss (2 * dL/d conj(M)), by the reverse sweep written with ``op_action``
    and ``partial_overlap`` only: grad_g = 2 * partial_overlap(lam_g, phi_{g-1}) on
    the gate's sites, with lam_g = U_{>g}^dagger H psi and phi_{g-1} the state
    before gate g."""
    phi = run_sv(gates, n, layered=False)
    lam = pauli_sum_apply(phi, terms)
    grads = [None] * len(gates)
    for gi in range(len(gates) - 1, -1, -1):
        g = gates[gi]
        m = _np(g.matrix)
        phi = op_action(m.conj().T, g.indices, phi)
        sites = list(g.indices)
        ov = partial_overlap(lam, phi, skip=sites)
        # partial_overlap orders kept sites ascending; re-index to g.indices order
        k = len(sites)
        srt = sorted(sites)
        perm = [srt.index(s) for s in sites]
        ov = ov.reshape([2] * 2 * k).transpose(perm + [p + k for p in perm]).reshape(2 ** k, 2 ** k)
        grads[gi] = 2.0 * ov
        lam = op_action(m.conj().T, g.indices, lam)
    return grads
