"""Density matrices at the sizes of the uneven noisy batch (6-14 qubits, depth
up to 40, depolarising 1e-3 after every two-qubit gate) on the default
complex64 path: 6-qubit fused blocks on the tensor cores with the trace chain.

Tolerances: the complex64 bar of 1e-5 on the trace, purity, every Tr(rho Z_i)
and every entry of rho. References: the oracle at 9 qubits, the complex128
path (itself pinned to the oracle at 1e-12) at 10 and 13 qubits, and at 14
qubits the complex64 CUDA-core path (no tensor cores, round-to-nearest FMA)."""
import numpy as np
import pytest
import torch

from oracle import ref

pytestmark = pytest.mark.gpu

TOL = 1e-5


@pytest.fixture(scope="module", autouse=True)
def built(cuda_ok):
    from qaravan_gb300 import build
    build.build()


def _run(circ, dtype):
    from qaravan_gb300 import DensityMatrixSim
    sim = DensityMatrixSim(circ, dtype=dtype)
    sim.run()
    n = circ.num_sites
    z = sim.pauli_expectations([(1.0, 'i' * q + 'z' + 'i' * (n - q - 1)) for q in range(n)]).cpu().numpy()
    return sim, sim.trace(), sim.purity(), z


def _check(a, b, tol=TOL):
    sa, ta, pa, za = a
    sb, tb, pb, zb = b
    assert abs(ta - 1) < tol, ta
    assert abs(pa - pb) < tol, (pa, pb)
    assert np.max(np.abs(za - zb)) < tol
    da = sa.get_density_matrix()
    db = sb.get_density_matrix().to(da.dtype)
    assert torch.max(torch.abs(da - db)).item() < tol


def test_tensor_core_dm_depth40_9_qubits_vs_oracle():
    from qaravan_gb300 import workloads
    n = 9
    c = workloads.noisy_brickwork_circuit(n, 40, 21, p=1e-3)
    sim, tr, pur, z = _run(c, torch.complex64)
    assert sim.mode == "fused" and sim.fusion_width == 6  # the tensor-core path
    seq = [g for layer in c.layers for g in layer]
    dm = ref.run_dm(seq, n, layered=False)
    assert abs(tr - 1) < TOL
    assert abs(pur - ref.purity(dm)) < TOL
    zref = [ref.dm_pauli_expectation(dm, 'i' * q + 'z' + 'i' * (n - q - 1)) for q in range(n)]
    assert np.max(np.abs(z - zref)) < TOL
    assert np.max(np.abs(sim.get_density_matrix().cpu().numpy() - dm)) < TOL


@pytest.mark.parametrize("n,seed", [(10, 5), (13, 8)])
def test_tensor_core_dm_depth40_vs_complex128(n, seed):
    from qaravan_gb300 import workloads
    c = workloads.noisy_brickwork_circuit(n, 40, seed, p=1e-3)
    _check(_run(c, torch.complex64), _run(c, torch.complex128))


def test_tensor_core_dm_depth40_14_qubits_vs_cuda_cores():
    from qaravan_gb300 import _lib, workloads
    c = workloads.noisy_brickwork_circuit(14, 40, 13, p=1e-3)
    tc = _run(c, torch.complex64)
    L = _lib.lib()
    prev = L.qgb_get_dense_impl()
    _lib.check(L.qgb_set_dense_impl(0), "set_dense_impl")
    try:
        cc = _run(c, torch.complex64)
    finally:
        L.qgb_set_dense_impl(prev)
    _check(tc, cc)


def test_trace_chain_removes_the_tensor_core_drift():
    # the same 13-qubit depth-40 circuit without the chain drifts well beyond the chain's
    # residual (one epoch of passes); with it the trace stays within 2e-6 of 1
    from qaravan_gb300 import engine, workloads
    c = workloads.noisy_brickwork_circuit(13, 40, 8, p=1e-3)
    with_chain = _run(c, torch.complex64)[1]
    engine.set_trace_chain(False)
    try:
        without = _run(c, torch.complex64)[1]
    finally:
        engine.set_trace_chain(True)
    assert abs(with_chain - 1) < 2e-6
    assert abs(without - 1) > 2 * abs(with_chain - 1)
