"""Uneven density-matrix batches vs the oracle and complex128: one batched
launch for the small circuits, one persistent tensor-core launch for the
complex64 circuits of 8-14 qubits (parallel streams for complex128), in one
CUDA graph; the persistent launch's results are bitwise reproducible."""
import numpy as np
import pytest
import torch

from oracle import ref

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built(cuda_ok):
    from qaravan_gb300 import build
    build.build()


def _oracle(circ, n):
    seq = [g for layer in circ.layers for g in layer]
    return ref.run_dm(seq, n, layered=False)


@pytest.mark.parametrize("dtype", [torch.complex64, torch.complex128])
def test_uneven_batch_matches_oracle(dtype):
    from qaravan_gb300 import DensityMatrixSim, workloads
    from qaravan_gb300.batch import DensityMatrixBatch
    rng = np.random.default_rng(3)
    specs = [(int(rng.integers(2, 10)), int(rng.integers(1, 4)), int(rng.integers(1 << 30))) for _ in range(14)]
    specs += [(7, 2, 5), (8, 2, 6), (6, 3, 7)]
    circs = [workloads.noisy_brickwork_circuit(n, d, s, p=0.05) for n, d, s in specs]
    sims = [DensityMatrixSim(c, dtype=dtype) for c in circs]
    batch = DensityMatrixBatch(sims, dtype=dtype)
    assert batch.small and (batch.pers if dtype == torch.complex64 else batch.large)  # both paths exercised
    batch.run(graph=True)
    res = batch.results()
    tol = 1e-5 if dtype == torch.complex64 else 1e-12
    for (n, d, s), c, r, i in zip(specs, circs, res, range(len(specs))):
        dm = _oracle(c, n)
        assert abs(r["trace"] - 1) < tol
        assert abs(r["purity"] - ref.purity(dm)) < 10 * tol
        z = [ref.dm_pauli_expectation(dm, 'i' * q + 'z' + 'i' * (n - q - 1)) for q in range(n)]
        assert np.max(np.abs(r["z"] - z)) < 10 * tol
        assert np.max(np.abs(batch.density_matrix(i).cpu().numpy() - dm)) < tol
    # replaying the graph reproduces the results exactly
    first = batch.out.clone()
    batch.run(graph=True)
    assert torch.equal(first, batch.out)


def test_persistent_batch_at_config_sizes_against_complex128():
    """Circuits of 8-14 qubits, depth 10-40, depolarising 1e-3 (the uneven
    batch's generator) in one persistent launch: trace, purity, Tr(rho Z_i) and
    every entry of rho against each circuit run alone in complex128 (the
    oracle-pinned path), at the complex64 bar of 1e-5; the 9-qubit circuit also
    against the oracle."""
    from qaravan_gb300 import DensityMatrixSim, workloads
    from qaravan_gb300.batch import DensityMatrixBatch
    specs = [(8, 40, 1), (9, 12, 2), (10, 25, 3), (11, 40, 4), (12, 18, 5), (13, 30, 6), (14, 10, 7), (6, 20, 8)]
    circs = [workloads.noisy_brickwork_circuit(n, d, s, p=1e-3) for n, d, s in specs]
    batch = DensityMatrixBatch([DensityMatrixSim(c, dtype=torch.complex64) for c in circs], dtype=torch.complex64)
    assert len(batch.pers) == 7 and not batch.large and len(batch.small) == 1
    batch.run(graph=True)
    res = batch.results()
    for i, ((n, d, sd), c) in enumerate(zip(specs, circs)):
        s128 = DensityMatrixSim(c, dtype=torch.complex128)
        s128.run()
        z = s128.pauli_expectations([(1.0, 'i' * q + 'z' + 'i' * (n - q - 1)) for q in range(n)]).cpu().numpy()
        assert abs(res[i]["trace"] - 1) < 1e-5, (n, res[i]["trace"])
        assert abs(res[i]["purity"] - s128.purity()) < 1e-5
        assert np.max(np.abs(res[i]["z"] - z)) < 1e-5
        rho = batch.density_matrix(i).to(torch.complex128)
        assert float((rho - s128.get_density_matrix()).abs().max()) < 1e-5
        if n == 9:
            seq = [g for layer in c.layers for g in layer]
            dm = ref.run_dm(seq, n, layered=False)
            assert np.max(np.abs(rho.cpu().numpy() - dm)) < 1e-5
            assert abs(res[i]["purity"] - ref.purity(dm)) < 1e-5
        del s128, rho
    # bitwise reproducible: a second replay gives the same results and states
    first = batch.out.clone()
    st = batch.density_matrix(5).clone()
    batch.run(graph=True)
    assert torch.equal(first, batch.out)
    assert torch.equal(st, batch.density_matrix(5))
    torch.cuda.empty_cache()
