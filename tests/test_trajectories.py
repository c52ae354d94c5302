"""Noisy trajectories: Philox pinned to its published known answer (CPU),
exact replay of logged branches against the oracle (GPU), and the trajectory
average against the reference's density-matrix run (GPU)."""
import numpy as np
import pytest
import torch

from conftest import golden
from gateio import unpack_gates
from oracle import ref


def _philox_np(ctr, key):
    """Philox4x32-10 restated in NumPy (Salmon et al., SC'11)."""
    c = [np.uint64(x) for x in ctr]
    k0, k1 = np.uint64(key[0]), np.uint64(key[1])
    M = np.uint64(0xFFFFFFFF)
    for _ in range(10):
        p0 = np.uint64(0xD2511F53) * c[0]
        p1 = np.uint64(0xCD9E8D57) * c[2]
        hi0, lo0 = p0 >> np.uint64(32), p0 & M
        hi1, lo1 = p1 >> np.uint64(32), p1 & M
        c = [(hi1 ^ c[1] ^ k0) & M, lo1, (hi0 ^ c[3] ^ k1) & M, lo0]
        k0 = (k0 + np.uint64(0x9E3779B9)) & M
        k1 = (k1 + np.uint64(0xBB67AE85)) & M
    return [int(x) for x in c]


def _uniform_np(event, traj, stream, seed):
    c = _philox_np([event, traj, stream, 0], [seed & 0xFFFFFFFF, seed >> 32])
    bits = ((c[0] << 21) ^ (c[1] >> 11)) & ((1 << 53) - 1)
    return bits / 9007199254740992.0


def test_philox_known_answer_and_library_match():
    # Random123 known-answer vector for philox4x32-10 with zero counter and key
    assert _philox_np([0, 0, 0, 0], [0, 0]) == [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]
    from qaravan_gb300 import build
    build.build()
    from qaravan_gb300.trajectories import philox_uniform
    for ev, t, s, seed in [(0, 0, 0, 0), (5, 17, 1, 1234), (1559, 1023, 3, 2 ** 40 + 7)]:
        assert philox_uniform(ev, t, s, seed) == _uniform_np(ev, t, s, seed)


PAULI = [np.eye(2), np.array([[0, 1], [1, 0]]), np.array([[0, -1j], [1j, 0]]), np.diag([1, -1])]


def _replay(gates, n, t, seed, p_dep, gamma, plog, jlog):
    psi = ref.initial_sv(n).reshape(-1)
    for i, g in enumerate(gates):
        psi = ref.op_action(np.asarray(g.matrix), g.indices, psi)
        if p_dep > 0:
            for j, q in enumerate(g.indices):
                u = _uniform_np(i, t, 2 * j, seed)
                pk = 0 if u < 1 - p_dep else 1 + min(2, int((u - (1 - p_dep)) / (p_dep / 3)))
                assert pk == plog[i, t, j]
                psi = ref.op_action(PAULI[pk], [q], psi)
        for j, q in enumerate(g.indices):
            probs = np.abs(psi.reshape([2] * n)) ** 2
            p1 = probs.take(1, axis=q).sum() / probs.sum()
            pj = gamma * p1
            u = _uniform_np(i, t, 2 * j + 1, seed)
            jump = u < pj
            assert int(jump) == jlog[i, t, j]
            if jump:
                psi = ref.op_action(np.array([[0, np.sqrt(gamma)], [0, 0]]) / np.sqrt(pj), [q], psi)
            else:
                psi = ref.op_action(np.diag([1, np.sqrt(1 - gamma)]) / np.sqrt(1 - pj), [q], psi)
    return psi


@pytest.mark.gpu
@pytest.mark.parametrize("dtype,n", [(torch.complex64, 6), (torch.complex128, 6), (torch.complex64, 10),
                                     (torch.complex128, 10)])
def test_trajectory_replay_matches_oracle(dtype, n, cuda_ok):
    """Gate-by-gate mode: every trajectory replayed branch by branch through the oracle. At 10
    qubits the unions of 2 to 4 bits that reach bits 0..4 take the warp-staged
    access path (complex64)."""
    from qaravan_gb300 import workloads
    from qaravan_gb300.circuits import Circuit
    from qaravan_gb300.trajectories import TrajectorySim
    T, seed, p, gamma = 12, 77, 0.3, 0.35
    gates = workloads.brickwork_gates(n, 3, 4)
    sim = TrajectorySim(Circuit(gates, n=n), T, p_dep=p, gamma=gamma, seed=seed, dtype=dtype, log=True,
                        mode="per_gate")
    states = sim.run().cpu().numpy()
    plog, jlog = sim.pauli_log.cpu().numpy(), sim.jump_log.cpu().numpy()
    assert jlog.sum() > 0 and plog.sum() > 0  # the noise is strong enough to branch
    tol = 1e-5 if dtype == torch.complex64 else 1e-12
    for t in range(T):
        exp = _replay(sim.gates, n, t, seed, p, gamma, plog, jlog)  # the simulator's (layer) order
        assert np.max(np.abs(states[t] - exp)) < tol


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["persistent", "per_gate"])
def test_graph_replay_is_deterministic(mode, cuda_ok):
    from qaravan_gb300 import workloads
    from qaravan_gb300.trajectories import TrajectorySim
    circ = workloads.tfi_trotter_circuit(8, 0.05, 3)
    a = TrajectorySim(circ, 64, p_dep=0.05, gamma=0.05, seed=3, mode=mode, tile_bits=6).run().clone()
    sim = TrajectorySim(circ, 64, p_dep=0.05, gamma=0.05, seed=3, mode=mode, tile_bits=6)
    b = sim.run(graph=True).clone()
    c = sim.run(graph=True).clone()
    assert torch.equal(a, b) and torch.equal(b, c)


@pytest.mark.gpu
@pytest.mark.parametrize("fixture,ntraj", [("traj_dm10_strong.npz", 8192), ("traj_dm10.npz", 1024)])
def test_trajectory_average_matches_reference_dm(fixture, ntraj, cuda_ok):
    """Mean <Z_i>, <Z_i Z_i+1> over trajectories (the persistent launch, the
    default) vs the reference DensityMatrixSim with the same per-gate channels,
    within 5 standard errors."""
    from qaravan_gb300.circuits import Circuit
    from qaravan_gb300.trajectories import TrajectorySim, z_terms
    z = golden(fixture)
    n = int(z["n"])
    gates = unpack_gates(z)
    sim = TrajectorySim(Circuit(gates, n=n), ntraj, p_dep=float(z["p"]), gamma=float(z["gamma"]), seed=11)
    sim.run(graph=True)
    mean, std = sim.mean_expectations(z_terms(n))
    mean, std = mean.cpu().numpy(), std.cpu().numpy()
    exp = np.concatenate([z["z"], z["zz"]])
    se = np.maximum(std, 1e-3) / np.sqrt(ntraj)
    assert np.all(np.abs(mean - exp) < 5 * se + 1e-5), (mean - exp, se)


def _replay_jumps(gates, n, t, seed, p_dep, gamma, jumps):
    """Oracle replay of one persistent-mode trajectory: the Paulis from the same
    Philox counters, and amplitude damping K1 (renormalised) exactly at the
    logged (gate, site) jumps, K0 (renormalised) elsewhere."""
    psi = ref.initial_sv(n).reshape(-1)
    jset = set(jumps)
    for i, g in enumerate(gates):
        psi = ref.op_action(np.asarray(g.matrix), g.indices, psi)
        for j, q in enumerate(g.indices):
            if p_dep > 0:
                u = _uniform_np(i, t, 2 * j, seed)
                pk = 0 if u < 1 - p_dep else 1 + min(2, int((u - (1 - p_dep)) / (p_dep / 3)))
                psi = ref.op_action(PAULI[pk], [q], psi)
            if gamma > 0:
                k = np.array([[0, np.sqrt(gamma)], [0, 0]]) if (i, j) in jset else np.diag([1, np.sqrt(1 - gamma)])
                psi = ref.op_action(k, [q], psi)
                psi = psi / np.linalg.norm(psi)
    return psi


@pytest.mark.gpu
@pytest.mark.parametrize("dtype,n,tile", [(torch.complex64, 6, 13), (torch.complex128, 6, 12),
                                          (torch.complex64, 10, 6), (torch.complex128, 10, 5),
                                          (torch.complex64, 12, 7)])
def test_persistent_trajectories_replay_matches_oracle(dtype, n, tile, cuda_ok):
    """Persistent launch (tiles smaller than the state at 10 and 12 qubits, so
    each trajectory crosses several sweeps): every trajectory replayed through
    the oracle with its logged jumps and its Philox Paulis."""
    from qaravan_gb300 import workloads
    from qaravan_gb300.circuits import Circuit
    from qaravan_gb300.trajectories import TrajectorySim
    T, seed, p, gamma = 12, 77, 0.3, 0.35
    gates = workloads.brickwork_gates(n, 3, 4)
    sim = TrajectorySim(Circuit(gates, n=n), T, p_dep=p, gamma=gamma, seed=seed, dtype=dtype, log=True,
                        tile_bits=tile)
    assert sim.mode == "persistent" and sim.launches == 2
    if n > tile:
        assert len(sim.sweep_plan) > 1
    states = sim.run().cpu().numpy()
    counts = sim.jump_count.cpu().numpy()
    assert counts.sum() > 0  # the damping is strong enough to jump
    tol = 1e-5 if dtype == torch.complex64 else 1e-12
    for t in range(T):
        exp = _replay_jumps(sim.gates, n, t, seed, p, gamma, sim.jumps(t))
        assert np.max(np.abs(states[t] - exp)) < tol


@pytest.mark.gpu
@pytest.mark.parametrize("dtype", [torch.complex64, torch.complex128])
def test_persistent_and_per_gate_draw_the_same_paulis(dtype, cuda_ok):
    """Without damping both modes are the same exact computation with the same
    Philox draws: equal states."""
    from qaravan_gb300 import workloads
    from qaravan_gb300.trajectories import TrajectorySim
    circ = workloads.tfi_trotter_circuit(11, 0.05, 4)
    a = TrajectorySim(circ, 40, p_dep=0.1, seed=9, dtype=dtype, mode="persistent", tile_bits=7).run()
    b = TrajectorySim(circ, 40, p_dep=0.1, seed=9, dtype=dtype, mode="per_gate").run()
    tol = 1e-5 if dtype == torch.complex64 else 1e-12
    assert torch.max(torch.abs(a - b)).item() < tol


@pytest.mark.gpu
@pytest.mark.parametrize("fixture,ntraj", [("traj_dm10_strong.npz", 8192)])
def test_per_gate_trajectory_average_matches_reference_dm(fixture, ntraj, cuda_ok):
    """The gate-by-gate path (sequential damping decisions) against the reference DM."""
    from qaravan_gb300.circuits import Circuit
    from qaravan_gb300.trajectories import TrajectorySim, z_terms
    z = golden(fixture)
    n = int(z["n"])
    gates = unpack_gates(z)
    sim = TrajectorySim(Circuit(gates, n=n), ntraj, p_dep=float(z["p"]), gamma=float(z["gamma"]), seed=11,
                        mode="per_gate")
    sim.run(graph=True)
    mean, std = sim.mean_expectations(z_terms(n))
    mean, std = mean.cpu().numpy(), std.cpu().numpy()
    exp = np.concatenate([z["z"], z["zz"]])
    se = np.maximum(std, 1e-3) / np.sqrt(ntraj)
    assert np.all(np.abs(mean - exp) < 5 * se + 1e-5), (mean - exp, se)
