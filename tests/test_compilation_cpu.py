"""Host-side parts of the compilation application (applications/compilation.py)
that need no GPU: the deprecated unitary embedding and the unitary
construction from basis strings."""
import numpy as np


def test_unitary_embedding_keeps_the_given_columns():
    """The deprecated embedding: the given input columns map to their outputs,
    the other columns are an orthonormal basis of the null space of (out^T in)^T."""
    from qaravan_gb300.applications import unitary_embedding
    rng = np.random.default_rng(4)
    outs = []
    for _ in range(2):
        v = rng.normal(size=8) + 1j * rng.normal(size=8)
        outs.append(v / np.linalg.norm(v))
    a = unitary_embedding(["010", "111"], outs)
    assert np.max(np.abs(a[:, 2] - outs[0])) < 1e-15 and np.max(np.abs(a[:, 7] - outs[1])) < 1e-15
    rest = a[:, [0, 1, 3, 4, 5, 6]]
    assert np.max(np.abs(rest.conj().T @ rest - np.eye(6))) < 1e-12
    assert np.max(np.abs(a[:, [2, 7]].T @ rest)) < 1e-12


def test_construct_unitary_maps_the_given_basis_states():
    """``construct_unitary`` (QR of out^T in with the given columns kept): column
    int(s, 2) is the output state paired with input string s."""
    from qaravan_gb300.applications import construct_unitary
    rng = np.random.default_rng(12)
    outs = []
    for _ in range(3):
        v = rng.normal(size=8) + 1j * rng.normal(size=8)
        outs.append(v / np.linalg.norm(v))
    q = construct_unitary(["000", "011", "110"], outs)
    for s, o in zip(["000", "011", "110"], outs):
        assert np.max(np.abs(q[:, int(s, 2)] - o)) < 1e-15
