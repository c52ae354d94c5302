"""Monte-Carlo Pauli-channel trajectories in a batch: the per-state Pauli-layer
kernel against the oracle's gate-by-gate application; every sample of a batch
replayed exactly through the oracle (same noise strings); batch means against
the exact mixture (all noise patterns enumerated, weighted by their
probabilities), plain and with the quasi-probability prefactors of the inverse
channel; and trotter_mc_sim replayed step by step."""
import itertools

import numpy as np
import pytest
import torch

from oracle import ref

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built(cuda_ok):
    from qaravan_gb300 import build
    build.build()


def _vdot_obs(sv, obs):
    return float(sum(c * ref.pauli_expectation_sv(sv, s) for c, s in obs))


@pytest.mark.parametrize("dtype", [torch.complex64, torch.complex128])
def test_pauli_layer_kernel_matches_oracle(dtype):
    from qaravan_gb300 import _lib
    from qaravan_gb300.gates import pauli_string_to_gates
    from qaravan_gb300.paulis import pauli_masks
    n, S = 9, 6
    rng = np.random.default_rng(4)
    states = rng.normal(size=(S, 2 ** n)) + 1j * rng.normal(size=(S, 2 ** n))
    strings = ["".join(rng.choice(list("ixyz"), size=n)) for _ in range(S)]
    strings[0] = "i" * n
    strings[1] = "z" * 3 + "i" * (n - 3)
    masks = np.array([pauli_masks(s) for s in strings], dtype=np.int64)
    dev = torch.as_tensor(states.reshape(-1)).to(dtype).cuda()
    xm, zm = torch.as_tensor(masks[:, 0]).cuda(), torch.as_tensor(masks[:, 1]).cuda()
    ny = torch.as_tensor(masks[:, 2].astype(np.int32)).cuda()
    _lib.check(_lib.lib().qgb_pauli_layer(dev.data_ptr(), _lib.dtype_code(dtype), n, xm.data_ptr(), zm.data_ptr(),
                                          ny.data_ptr(), S, 2 ** n, _lib.stream_ptr()))
    got = dev.cpu().numpy().reshape(S, -1)
    tol = 1e-5 if dtype == torch.complex64 else 1e-12
    for b in range(S):
        want = states[b].reshape([2] * n)
        for g in pauli_string_to_gates(strings[b]):
            want = ref.op_action(g.matrix, g.indices, want)
        assert np.max(np.abs(got[b] - want.reshape(-1))) < tol


def _circuit(n, depth, seed):
    from qaravan_gb300 import workloads
    from qaravan_gb300.circuits import Circuit
    return Circuit(workloads.brickwork_gates(n, depth, seed), n=n)


def _replay(circ, strings_s, obs):
    from qaravan_gb300.gates import pauli_string_to_gates
    n = circ.num_sites
    c = circ.copy()
    c.construct_layers()
    state = ref.initial_sv(n)
    for layer, s in zip(c.layers, strings_s):
        for g in layer:
            state = ref.op_action(g.matrix, g.indices, state)
        for g in pauli_string_to_gates(s):
            state = ref.op_action(g.matrix, g.indices, state)
    return _vdot_obs(state.reshape(-1), obs)


OBS6 = [(1.0, "zziiii"), (0.5, "ixiixi"), (-0.3, "yiiiiy")]


@pytest.mark.parametrize("kind", ["pauli", "lindblad"])
def test_every_sample_replays_through_the_oracle(kind):
    from qaravan_gb300.montecarlo import MonteCarloSim
    from qaravan_gb300.noise import PauliLindbladNoise, PauliNoise
    n = 6
    circ = _circuit(n, 2, 11)
    nm = (PauliNoise(["ii", "xi", "iz", "yy"], [0.7, 0.1, 0.15, 0.05]) if kind == "pauli"
          else PauliLindbladNoise(["xi", "zz", "iy"], [0.05, 0.1, 0.02]))
    sim = MonteCarloSim(circ, nm=nm)
    S = 24
    vals = sim.expectation_samples(OBS6, S, rng=np.random.default_rng(5))
    nlay = len(sim._layers())
    strings, _ = sim.sample_noise(S, nlay, rng=np.random.default_rng(5))
    for s in range(S):
        assert abs(vals[s] - _replay(circ, strings[s], OBS6)) < 1e-5
    # a dense observable (the reference's form) gives the same numbers
    from functools import reduce
    from qaravan_gb300.paulis import pauli_mapping
    dense = sum(c * reduce(np.kron, [pauli_mapping[ch] for ch in p]) for c, p in OBS6)
    vals2 = sim.expectation_samples(dense, S, rng=np.random.default_rng(5))
    assert np.max(np.abs(vals2 - vals)) < 1e-5


def _exact_mixture(circ, nm, obs, inverse=False):
    """Sum over every noise pattern of every layer, weighted by its probability
    (times the inverse-channel prefactor product for ``inverse``)."""
    from qaravan_gb300.noise import PauliLindbladNoise
    from qaravan_gb300.paulis import pauli_multiply
    c = circ.copy()
    c.construct_layers()
    L = len(c.layers)
    n = circ.num_sites
    if isinstance(nm, PauliLindbladNoise):
        outcomes = []
        for fired in itertools.product([0, 1], repeat=len(nm.strings)):
            p, s = 1.0, "i" * nm.num_sites
            for f, r, st in zip(fired, nm.rates, nm.strings):
                p *= r if f else 1 - r
                if f:
                    s, _ = pauli_multiply(s, st)
            w = nm.gamma * (-1) ** (s != "i" * nm.num_sites) if inverse else 1.0
            outcomes.append((p * w, s))
    else:
        outcomes = list(zip(nm.probs, nm.strings))
    total = 0.0
    for combo in itertools.product(outcomes, repeat=L):
        w = np.prod([x[0] for x in combo])
        total += w * _replay(circ, [x[1] + "i" * (n - len(x[1])) for x in combo], obs)
    return total


@pytest.mark.parametrize("kind,inverse", [("pauli", False), ("lindblad", False), ("lindblad", True)])
def test_batch_mean_matches_the_exact_mixture(kind, inverse):
    from qaravan_gb300.montecarlo import MonteCarloSim
    from qaravan_gb300.noise import PauliLindbladNoise, PauliNoise
    n = 4
    circ = _circuit(n, 1, 3)  # 3 layers
    nm = (PauliNoise(["ii", "xi", "zz"], [0.8, 0.12, 0.08]) if kind == "pauli"
          else PauliLindbladNoise(["xi", "zz"], [0.04, 0.06]))
    obs = [(1.0, "zzii"), (0.7, "ixxi")]
    exact = _exact_mixture(circ, nm, obs, inverse)
    sim = MonteCarloSim(circ, nm=nm)
    S = 60000
    out = sim.expectation_samples(obs, S, rng=np.random.default_rng(9), inverse=inverse)
    est = out[0] * out[1] if inverse else out
    assert abs(est.mean() - exact) < 5 * est.std() / np.sqrt(S) + 1e-6


def test_trotter_mc_sim_replays_step_by_step():
    from qaravan_gb300.hamiltonians import TFI
    from qaravan_gb300.montecarlo import MonteCarloSim, trotter_mc_sim
    from qaravan_gb300.noise import PauliNoise
    from qaravan_gb300.gates import pauli_string_to_gates
    ham = TFI(5, jz=1.0, h=0.7)
    nm = PauliNoise(["iiiii", "xiiii", "iizii"], [0.85, 0.1, 0.05])
    obs = [(1.0, "ziiii"), (1.0, "iziii")]
    S, steps = 8, 3
    got = trotter_mc_sim(ham, 0.1, steps, nm, obs, num_samples=S, rng=np.random.default_rng(2))
    circ = ham.trotter_circ(0.1, 1)
    sim = MonteCarloSim(circ, nm=nm)
    layers = sim._layers()
    rng = np.random.default_rng(2)
    states = [ref.initial_sv(5) for _ in range(S)]
    for step in range(steps):
        strings, _ = sim.sample_noise(S, len(layers), rng)
        vals = []
        for s in range(S):
            st = states[s]
            for layer, ps in zip(layers, strings[s]):
                for g in layer:
                    st = ref.op_action(g.matrix, g.indices, st)
                for g in pauli_string_to_gates(ps):
                    st = ref.op_action(g.matrix, g.indices, st)
            states[s] = st
            vals.append(_vdot_obs(st.reshape(-1), obs))
        assert abs(got[step] - np.mean(vals)) < 1e-5
