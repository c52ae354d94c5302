"""The reference's own test scenarios (tests/test_core.py, tests/test_resets.py:
the statevector and measurement cases) restated against this package's
reference-named namespaces, as a user switching imports would run them:
``from qaravan_gb300.tensorQ import *`` and ``from qaravan_gb300.core import *``."""
from collections import Counter

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built(cuda_ok):
    from qaravan_gb300 import build
    build.build()


def _ghz_sim():
    from qaravan_gb300.core import CNOT, Circuit, H
    from qaravan_gb300.tensorQ import StatevectorSim
    return StatevectorSim(Circuit([H(0), CNOT([1, 0], 3), CNOT([2, 1], 3)], 3))


def test_ghz_state_and_expectations():
    from qaravan_gb300.core import pauli_Z
    sim = _ghz_sim()
    sim.run()
    sv = sim.get_statevector()
    want = np.zeros(8, dtype=complex)
    want[0] = want[-1] = 1 / np.sqrt(2)
    assert np.allclose(sv, want, atol=1e-7)
    assert abs(_ghz_sim().pauli_expectation("izz") - 1.0) < 1e-7
    assert abs(_ghz_sim().pauli_expectation("izi")) < 1e-7
    assert abs(_ghz_sim().one_local_expectation(pauli_Z, 2)) < 1e-7


def _three_outcome_state():
    from qaravan_gb300.core import string_to_sv
    return (np.sqrt(0.3) * string_to_sv("0001") + np.sqrt(0.45) * string_to_sv("1110")
            + np.sqrt(0.25) * string_to_sv("1011"))


def test_measurement_frequencies():
    from qaravan_gb300.tensorQ import measure_sv
    sv = _three_outcome_state()
    counts = Counter(measure_sv(sv, [0, 1]) for _ in range(2000))
    for outcome, p in (("00", 0.3), ("11", 0.45), ("10", 0.25)):
        assert abs(counts[outcome] / 2000 - p) < 0.05


def test_measure_and_collapse():
    from qaravan_gb300.core import string_to_sv
    from qaravan_gb300.tensorQ import measure_and_collapse_sv
    sv = _three_outcome_state()
    for _ in range(50):
        outcome, post = measure_and_collapse_sv(sv, [0, 2])
        if outcome == "00":
            assert np.allclose(post, string_to_sv("01"))
        else:
            assert outcome == "11"
            want = np.sqrt(0.45 / 0.7) * string_to_sv("10") + np.sqrt(0.25 / 0.7) * string_to_sv("01")
            assert np.allclose(post, want, atol=1e-7)


def _run(gates, n=None):
    from qaravan_gb300.core import Circuit
    from qaravan_gb300.tensorQ import StatevectorSim
    sim = StatevectorSim(Circuit(gates, n=n))
    sim.run(progress_bar=False)
    return sim.get_statevector()


def test_resets():
    from qaravan_gb300.core import CNOT, H, Reset, X, string_to_sv
    assert np.allclose(_run([H(0), Reset(0, "0")]), [1, 0])
    assert np.allclose(_run([H(0), Reset(0, "1")]), [0, 1])
    assert np.allclose(_run([H(0), X(1), Reset(0, "1")], n=2), [0, 0, 0, 1])
    assert np.allclose(_run([H(0), CNOT([1, 0]), Reset(0, "0")], n=2), [1, 0, 0, 0])
    assert np.allclose(_run([H(0), H(1), Reset([0, 1], "10")], n=2), [0, 0, 1, 0])
    assert np.allclose(_run([H(0), Reset(0, "1"), H(0), Reset(0, "1")]), [0, -1])
    want = (string_to_sv("100") - string_to_sv("111")) / np.sqrt(2)
    assert np.allclose(_run([H(0), CNOT([1, 0]), Reset(1, "1"), H(1), CNOT([2, 1])], n=3), want)
