"""Uneven density-matrix batches (one batched launch for the small circuits,
parallel streams for the large ones, one CUDA graph) vs the oracle."""
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
    assert batch.small and batch.large  # both paths exercised
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
