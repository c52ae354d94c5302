"""Noise-model additions used by the Monte-Carlo path (CPU): the inverse Pauli
channel (core/noise.py:131-135) undoes the channel in the Pauli transfer matrix;
Pauli-Lindblad sampling multiplies the fired generators and its inverse sample
carries gamma * (-1)^(non-empty) (core/noise.py:194-210)."""
import numpy as np

from qaravan_gb300.noise import PauliLindbladNoise, PauliNoise
from qaravan_gb300.paulis import pauli_multiply


def test_pauli_noise_pinv_inverts_the_transfer_matrix():
    nm = PauliNoise(["ii", "xi", "zz", "yx"], [0.9, 0.05, 0.03, 0.02])
    inv = nm.pinv()
    assert np.allclose(np.diag(inv.ptm()) * np.diag(nm.ptm()), 1.0)
    assert abs(sum(inv.probs) - 1) < 1e-9


def test_lindblad_samples_and_inverse_prefactors():
    nm = PauliLindbladNoise(["xi", "zz", "iy"], [0.2, 0.3, 0.1], dense=False)
    rng = np.random.default_rng(3)
    seen_empty = seen_full = False
    for _ in range(400):
        s = nm.sample_string(rng)
        assert len(s) == 2 and set(s) <= set("ixyz")
        layer, pref = nm.inv_sample(rng)
        if layer:
            assert pref == -nm.gamma
            seen_full = True
        else:
            assert pref == nm.gamma
            seen_empty = True
    assert seen_empty and seen_full
    # the product of the fired generators, phases dropped
    r = np.random.default_rng(11)
    flags = [r.random() < rate for rate in nm.rates]
    want = "ii"
    for st, f in zip(nm.strings, flags):
        if f:
            want, _ = pauli_multiply(want, st)
    assert nm.sample_string(np.random.default_rng(11)) == want
