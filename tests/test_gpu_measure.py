"""Measurement on the device against the oracle (the reference's
rdm_from_sv / measure_sv / measure_and_collapse_sv, restated): outcome
probabilities for sorted, unsorted, single and all-site measurements; shot
sampling replayed exactly with a NumPy restatement of the Philox stream and the
inverse-CDF search, and its distribution; collapse for sorted and unsorted
sites."""
import numpy as np
import pytest
import torch

from oracle import ref
from test_trajectories import _philox_np

pytestmark = pytest.mark.gpu

TOL = {torch.complex64: 1e-6, torch.complex128: 1e-12}


@pytest.fixture(scope="module", autouse=True)
def built(cuda_ok):
    from qaravan_gb300 import build
    build.build()


def _state(n, seed):
    rng = np.random.default_rng(seed)
    v = rng.normal(size=2 ** n) + 1j * rng.normal(size=2 ** n)
    return v / np.linalg.norm(v)


SITE_SETS = [[3], [0, 2, 5], [5, 2, 0], [9, 1, 4, 7], [0, 1, 2, 3, 4, 5, 6, 7, 8, 9], [8, 9]]


@pytest.mark.parametrize("dtype", [torch.complex64, torch.complex128])
@pytest.mark.parametrize("sites", SITE_SETS)
def test_outcome_probs_match_oracle(dtype, sites):
    from qaravan_gb300.measure import outcome_probs
    n = 10
    sv = _state(n, len(sites) + 7 * sites[0])
    got = outcome_probs(torch.as_tensor(sv).to(dtype).cuda(), n, sites).cpu().numpy()
    want = ref.measure_probs(sv, sites)
    assert np.max(np.abs(got - want)) < TOL[dtype]


@pytest.mark.parametrize("n,sites", [(14, [2, 11]), (20, [0, 7, 13, 19]), (20, list(range(14))), (16, list(range(16)))])
def test_outcome_probs_large_sum_to_one(n, sites):
    """Size-independent check at sizes the oracle would be slow on: the probabilities
    are the marginals of |psi|^2 (total 1; each equals the direct marginal sum)."""
    from qaravan_gb300.measure import outcome_probs
    sv = _state(n, n)
    got = outcome_probs(torch.as_tensor(sv).to(torch.complex128).cuda(), n, sites).cpu().numpy()
    p = np.abs(sv.reshape([2] * n)) ** 2
    rest = tuple(q for q in range(n) if q not in sites)
    want = p.sum(axis=rest).reshape(-1)  # remaining axes are the sites ascending
    assert abs(got.sum() - 1) < 1e-12
    assert np.max(np.abs(got - want)) < 1e-12


def _replay(probs, shots, seed):
    cdf = np.cumsum(probs)
    total = cdf[-1]
    out = []
    for s in range(shots):
        c = _philox_np([s & 0xFFFFFFFF, s >> 32, 0, 1], [seed & 0xFFFFFFFF, seed >> 32])
        u = (((c[0] << 21) ^ (c[1] >> 11)) & ((1 << 53) - 1)) / 9007199254740992.0 * total
        out.append(min(int(np.searchsorted(cdf, u, side="right")), len(probs) - 1))
    return np.array(out)


@pytest.mark.parametrize("m", [1, 4, 13])
def test_sampling_replays_exactly(m):
    from qaravan_gb300.measure import sample_outcomes
    rng = np.random.default_rng(m)
    p = rng.random(2 ** m) ** 3
    p[rng.random(2 ** m) < 0.2] = 0.0  # zero-probability outcomes are never drawn
    seed = 0x1234_5678_9ABC + m
    got = sample_outcomes(torch.as_tensor(p).cuda(), 3000, seed).cpu().numpy()
    want = _replay(p, 3000, seed)
    assert np.sum(got != want) <= 1  # a float64 prefix-sum ulp can move a draw at a bin edge
    assert np.all(p[got] > 0)


def test_sampling_distribution():
    from qaravan_gb300.measure import outcome_probs, sample_outcomes
    n, sites = 12, [1, 4, 6, 10]
    sv = _state(n, 5)
    probs = outcome_probs(torch.as_tensor(sv).to(torch.complex64).cuda(), n, sites)
    shots = 400000
    idx = sample_outcomes(probs, shots, 99).cpu().numpy()
    freq = np.bincount(idx, minlength=16) / shots
    p = ref.measure_probs(sv, sites)
    sigma = np.sqrt(p * (1 - p) / shots)
    assert np.all(np.abs(freq - p) < 5 * sigma + 1e-12)


@pytest.mark.parametrize("dtype", [torch.complex64, torch.complex128])
@pytest.mark.parametrize("sites,outcome", [([2, 5], "10"), ([5, 2], "10"), ([7, 0, 3], "011"), ([3, 7, 0], "011"),
                                           ([9], "1")])
def test_collapse_matches_oracle(dtype, sites, outcome):
    from qaravan_gb300.measure import collapse_sv
    n = 10
    sv = _state(n, 17)
    got = collapse_sv(torch.as_tensor(sv).to(dtype).cuda(), n, sites, outcome).cpu().numpy()
    want = ref.collapse_sv(sv, sites, outcome)
    assert np.max(np.abs(got - want)) < 10 * TOL[dtype]


def test_simulator_measure_and_collapse():
    from qaravan_gb300 import StatevectorSim, workloads
    from qaravan_gb300.circuits import Circuit
    n = 14
    sim = StatevectorSim(Circuit(workloads.brickwork_gates(n, 3, 8), n=n))
    shots = sim.measure([0, 5, 9], shots=64, rng=np.random.default_rng(1))
    assert len(shots) == 64 and all(len(s) == 3 and set(s) <= {"0", "1"} for s in shots)
    outcome, post = sim.measure_and_collapse([4, 1], rng=np.random.default_rng(2))
    assert post.numel() == 2 ** (n - 2)
    assert abs(torch.linalg.vector_norm(post.to(torch.complex128)).item() - 1) < 1e-5
