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
