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


def test_random_pauli_channel_and_lindblad_superops_match_the_reference():
    """Fixture from the reference (make_golden.py gen_noise_misc)."""
    import numpy as np
    from conftest import golden
    from qaravan_gb300.noise import PauliLindbladNoise, random_pauli_channel
    z = golden("noise_misc.npz")
    np.random.seed(3)
    ch = random_pauli_channel(3, 5, 0.2)
    assert list(ch.strings) == [str(x) for x in z["strings"]]
    assert np.max(np.abs(np.array(ch.probs) - z["probs"])) < 1e-15
    assert str(ch) == str(z["text"])
    lb = PauliLindbladNoise(['xi', 'zz', 'yx'], [0.05, 0.1, 0.02])
    assert np.max(np.abs(lb.make_superop() - z["lb_superop"])) < 1e-14
    assert np.max(np.abs(lb.get_superop_for_string(1) - z["lb_superop_1"])) < 1e-15
