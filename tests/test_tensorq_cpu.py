"""Host-only helpers of ``qaravan_gb300.tensorQ`` against the oracle's
restatement of ``tensorQ/statevector_sim.py:111-153``."""
import numpy as np

from oracle import ref


def test_locs_to_indices_matches_oracle():
    from qaravan_gb300.tensorQ import locs_to_indices
    for locs, n in [([0], 1), ([2], 5), ([0, 3], 6), ([1, 2, 7], 9), ([4, 5], 6)]:
        assert locs_to_indices(locs, n) == ref.locs_to_indices(locs, n)


def test_all_zero_and_random_sv():
    from qaravan_gb300.tensorQ import all_zero_sv, random_sv
    d = all_zero_sv(5, dense=True)
    assert d.shape == (32,) and d[0] == 1 and d.sum() == 1
    s = all_zero_sv(5)
    assert s.shape == (32, 1) and s.toarray()[0, 0] == 1
    np.random.seed(4)
    a = random_sv(6)
    np.random.seed(4)
    b = random_sv(6)
    assert np.array_equal(a, b) and abs(np.linalg.norm(a) - 1) < 1e-12
    np.random.seed(4)
    raw = np.random.rand(64) + 1j * np.random.rand(64)
    assert np.max(np.abs(a - raw / np.linalg.norm(raw))) < 1e-15


def test_reference_host_scenarios():
    """Host-only cases of the reference's tests/test_core.py: construct_unitary,
    a copied circuit keeping a gate's autograd graph, lattice skeletons."""
    import torch
    from qaravan_gb300.applications import construct_unitary
    from qaravan_gb300.core import (Circuit, Gate, all_skeletons, brickwall_skeleton, coords_from_index, even_filter,
                                    horiz_filter, index_from_coords, nn_edges, random_unitary, string_to_sv)
    u = random_unitary(4)
    ins = ["00", "01", "10"]
    q = construct_unitary(ins, [u @ string_to_sv(s) for s in ins])
    assert np.allclose(q.conj().T @ q, np.eye(4), atol=1e-7) and np.allclose(q @ q.conj().T, np.eye(4), atol=1e-7)
    for s in ins:
        assert np.allclose(q @ string_to_sv(s), u @ string_to_sv(s), atol=1e-7)
    theta = torch.randn(1, dtype=torch.float64, requires_grad=True)
    mat = torch.matrix_exp(-1j * theta * torch.tensor([[0., 1.], [1., 0.]], dtype=torch.complex128))
    gate = Gate("Rx", [0], mat)
    Circuit([gate], n=1).copy()
    out = gate.matrix @ torch.tensor([1.0, 0.0], dtype=torch.complex128)
    torch.real(torch.dot(out.conj(), out)).backward()
    assert theta.grad is not None
    Lx = 4
    assert index_from_coords(2, 1, Lx) == 6 and index_from_coords(1, 2, Lx) == 9
    assert coords_from_index(6, Lx) == (2, 1) and coords_from_index(9, Lx) == (1, 2)
    assert horiz_filter((1, 2)) and not horiz_filter((1, 4))
    assert even_filter((0, 1), vert=False, Lx=Lx) and not even_filter((1, 2), vert=False, Lx=Lx)
    assert even_filter((0, 4), vert=True, Lx=Lx) and even_filter((1, 5), vert=True, Lx=Lx)
    assert not even_filter((4, 8), vert=True, Lx=Lx) and not even_filter((5, 9), vert=True, Lx=Lx)
    assert len(nn_edges(Lx, 3)) == 2 * Lx * 3 - Lx - 3
    assert brickwall_skeleton(Lx=4, Ly=2, depth=1) == [(0, 1), (2, 3), (4, 5), (6, 7), (1, 2), (5, 6), (0, 4),
                                                       (1, 5), (2, 6), (3, 7)]
    assert len(all_skeletons(4, Lx=Lx, Ly=3)) == (2 * Lx * 3 - Lx - 3) ** 4
