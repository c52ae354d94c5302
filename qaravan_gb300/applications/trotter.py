"""Trotter applications of the reference on the GPU (``applications/trotter.py``).

Same functions, arguments and results as the reference; the state (or
vec(rho)) stays on the device for the whole run: one Trotter step is compiled
once and applied ``max_steps`` times, and the observable is evaluated on the
device after each step (a dense operator as a matrix-vector product, a Pauli
sum ``[(coeff, 'ixyz..'), ...]`` through ``qgb_pauli_expectation``; for
vec(rho), a dense operator as ``<vec(op^dagger)|vec(rho)>`` through
``qgb_inner_product``). The
reference rebuilds a simulator per step and copies the state through the host.
Results are complex128 by default (the reference's NumPy precision).
"""
from __future__ import annotations

import numpy as np
import torch

from ..density_matrix import DensityMatrixSim
from ..gates import embed_operator
from ..montecarlo import MonteCarloSim, trotter_mc_sim
from ..paulis import pauli_Z
from ..statevector import StatevectorSim, inner_product, pauli_expectations

__all__ = ["magnetization", "trotter_sv_sim", "trotter_dm_sim", "trotter_dm_sim_uncached", "trotter_mc_sim",
           "trotter_mc_sim_uncached"]


def magnetization(n):
    """Total Z magnetisation on n qubits divided by sqrt(n 2^n) (``applications/trotter.py:5-8``)."""
    mz = sum(embed_operator(n, [i], [pauli_Z], dense=True) for i in range(n))
    return mz / np.sqrt(n * 2 ** n)


def _is_pauli_sum(op):
    return isinstance(op, (list, tuple)) and len(op) > 0 and isinstance(op[0], (list, tuple))


def _dense(op, device, dtype):
    return torch.as_tensor(np.asarray(op, dtype=np.complex128)).to(device=device, dtype=dtype)


def _sv_expectation(state, n, op, dense):
    if dense is None:
        return float(pauli_expectations(state, n, list(op)).sum())
    return float(torch.vdot(state, dense @ state).real)


def trotter_sv_sim(ham, step_size, max_steps, op, dtype=torch.complex128):
    """<op> after each of ``max_steps`` first-order Trotter steps from |0...0>
    (``applications/trotter.py:10-22``)."""
    circ = ham.trotter_circ(step_size, 1)
    n = ham.num_sites
    sim = StatevectorSim(circ, dtype=dtype)
    ex = sim.compile()
    sim.initialize_state()
    state = sim.state
    dense = None if _is_pauli_sum(op) else _dense(op, state.device, dtype)
    out = []
    for _ in range(int(max_steps)):
        ex.run(state)
        out.append(_sv_expectation(state, n, op, dense))
    return out


def _dm_observable(op, n, device, dtype):
    """None for a Pauli sum, else vec(op^dagger) on the device: Tr(op rho) = <vec(op^dagger)|vec(rho)>."""
    if _is_pauli_sum(op):
        return None
    od = np.ascontiguousarray(np.asarray(op, dtype=np.complex128).conj().T)
    return torch.as_tensor(od).to(device=device, dtype=dtype).reshape(-1)


def _dm_expectation(sim, op, od):
    if od is None:
        return float(sim.pauli_expectations(list(op)).sum())
    return float(inner_product(od, sim.state, 2 * sim.num_sites)[0].item())


def trotter_dm_sim(ham, step_size, max_steps, channel, op, dtype=torch.complex128):
    """Tr(op rho) after each noisy Trotter step (``channel`` after every layer,
    ``applications/trotter.py:24-36``)."""
    circ = ham.trotter_circ(step_size, 1)
    sim = DensityMatrixSim(circ, nm=channel, dtype=dtype)
    ex = sim.compile()
    sim.initialize_state()
    od = _dm_observable(op, sim.num_sites, sim.state.device, dtype)
    out = []
    for _ in range(int(max_steps)):
        ex.run(sim.state)
        out.append(_dm_expectation(sim, op, od))
    return out


def trotter_dm_sim_uncached(ham, step_size, max_steps, channel, op, dtype=torch.complex128):
    """The same from scratch for every step count (``applications/trotter.py:38-48``)."""
    out = []
    od = None
    for num_steps in range(1, int(max_steps) + 1):
        sim = DensityMatrixSim(ham.trotter_circ(step_size, num_steps), nm=channel, dtype=dtype)
        sim.run()
        if od is None:
            od = _dm_observable(op, sim.num_sites, sim.state.device, dtype)
        out.append(_dm_expectation(sim, op, od))
    return out


def trotter_mc_sim_uncached(ham, step_size, max_steps, channel, op, num_samples=1000, rng=None,
                            dtype=torch.complex64):
    """Monte-Carlo estimate from scratch for every step count, all samples of a
    step count as one batch (``applications/trotter.py:50-59``)."""
    out = []
    for num_steps in range(1, int(max_steps) + 1):
        sim = MonteCarloSim(ham.trotter_circ(step_size, num_steps), nm=channel, dtype=dtype)
        out.append(float(np.mean(sim.expectation_samples(op, num_samples, rng=rng))))
    return out
