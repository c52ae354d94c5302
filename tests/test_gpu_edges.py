"""Edge cases of the simulators against the oracle: an empty circuit, one
qubit, a gate whose block covers the whole state, descending and
non-adjacent sites, bitstring initial states, and the smallest state the
tensor-core kernel takes (13 qubits). Tolerances: complex64 1e-5, complex128
1e-12 (max absolute amplitude error)."""
import numpy as np
import pytest
import torch

from oracle import ref

pytestmark = pytest.mark.gpu

TOL = {torch.complex64: 1e-5, torch.complex128: 1e-12}
DTYPES = [torch.complex64, torch.complex128]


@pytest.fixture(scope="module", autouse=True)
def built(cuda_ok):
    from qaravan_gb300 import build
    build.build()


def _sv(circ, dtype, **kw):
    from qaravan_gb300 import StatevectorSim
    sim = StatevectorSim(circ, dtype=dtype, **kw)
    sim.run()
    return sim.get_statevector().reshape(-1).to(torch.complex128).cpu().numpy()


@pytest.mark.parametrize("dtype", DTYPES)
def test_empty_circuit_leaves_the_initial_state(dtype):
    from qaravan_gb300 import DensityMatrixSim
    from qaravan_gb300.circuits import Circuit
    sv = _sv(Circuit([], n=5), dtype)
    want = np.zeros(32)
    want[0] = 1
    assert np.max(np.abs(sv - want)) == 0
    sv = _sv(Circuit([], n=4), dtype, init_state="0110")
    assert abs(sv[int("0110", 2)] - 1) == 0 and np.count_nonzero(sv) == 1
    dm = DensityMatrixSim(Circuit([], n=3), dtype=dtype)
    dm.run()
    rho = dm.get_density_matrix().reshape(8, 8).to(torch.complex128).cpu().numpy()
    assert abs(rho[0, 0] - 1) == 0 and np.count_nonzero(rho) == 1


@pytest.mark.parametrize("dtype", DTYPES)
def test_one_qubit(dtype):
    from qaravan_gb300.circuits import Circuit
    from qaravan_gb300.gates import H, RY
    gates = [H(0), RY(0, 0.3), H(0)]
    sv = _sv(Circuit(gates, n=1), dtype)
    assert np.max(np.abs(sv - ref.run_sv(gates, 1))) < TOL[dtype]


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("mode,width", [("gate", 2), ("fused", 6), ("sweep", 4)])
def test_descending_and_distant_sites_and_whole_state_blocks(dtype, mode, width):
    """Two-qubit Haar gates on descending, non-adjacent site pairs of a 6-qubit
    state; fused width 6 makes one block cover the whole state."""
    from qaravan_gb300 import workloads
    from qaravan_gb300.circuits import Circuit
    from qaravan_gb300.gates import Gate
    rng = np.random.default_rng(41)
    n = 6
    gates = []
    for a, b in [(5, 0), (3, 1), (0, 4), (2, 5), (4, 3), (1, 2), (5, 0)]:
        gates.append(Gate("U2", [a, b], workloads.haar_unitary(4, rng)))
        gates.append(Gate("U1", [b], workloads.haar_unitary(2, rng)))
    sv = _sv(Circuit(gates, n=n), dtype, mode=mode, fusion_width=width)
    assert np.max(np.abs(sv - ref.run_sv(gates, n))) < TOL[dtype]


def test_smallest_tensor_core_state_matches_oracle():
    """13 qubits (one 8192-amplitude tile, the tensor-core kernel's smallest
    state), complex64 brickwork fused into 6-qubit tensor-core blocks, from a
    bitstring initial state."""
    from qaravan_gb300 import _lib, workloads
    from qaravan_gb300.circuits import Circuit
    assert _lib.lib().qgb_get_dense_impl() >= 1
    n = 13
    gates = workloads.brickwork_gates(n, 6, 91)
    init = "1011001110001"
    sv = _sv(Circuit(gates, n=n), torch.complex64, mode="fused", fusion_width=6, init_state=init)
    assert np.max(np.abs(sv - ref.run_sv(gates, n, init_state=init))) < 1e-5
    assert abs(np.linalg.norm(sv) - 1) < 1e-6


def test_noise_free_trajectories_equal_the_statevector():
    """With no noise every trajectory is the ideal state: 64 trajectories of the
    20-qubit TFI Trotter circuit against StatevectorSim (complex64), and each
    trajectory's norm stays 1 with amplitude damping alone."""
    from qaravan_gb300 import workloads
    from qaravan_gb300.trajectories import TrajectorySim
    n = 20
    circ = workloads.tfi_trotter_circuit(n, 0.05, 2)
    ideal = _sv(circ, torch.complex64)
    states = TrajectorySim(circ, 64, p_dep=0.0, gamma=0.0, seed=5).run()
    err = (states.to(torch.complex128).cpu() - torch.from_numpy(ideal)).abs().max().item()
    assert err < 1e-5
    damped = TrajectorySim(circ, 64, p_dep=0.0, gamma=0.05, seed=5).run()
    norms = torch.linalg.vector_norm(damped.to(torch.complex128), dim=1).cpu().numpy()
    assert np.max(np.abs(norms - 1)) < 1e-5


@pytest.mark.parametrize("dtype", DTYPES)
def test_unitary_density_matrix_is_the_pure_state(dtype):
    """A noise-free density-matrix run equals |psi><psi| of the statevector run
    of the same circuit (10 qubits, brickwork)."""
    from qaravan_gb300 import DensityMatrixSim, workloads
    from qaravan_gb300.circuits import Circuit
    n = 10
    gates = workloads.brickwork_gates(n, 4, 17)
    psi = _sv(Circuit(gates, n=n), dtype)
    dm = DensityMatrixSim(Circuit(gates, n=n), dtype=dtype)
    dm.run()
    rho = dm.get_density_matrix().reshape(2 ** n, 2 ** n).to(torch.complex128).cpu().numpy()
    assert np.max(np.abs(rho - np.outer(psi, psi.conj()))) < TOL[dtype]
