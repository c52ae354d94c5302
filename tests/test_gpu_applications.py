"""Trotter applications (applications/trotter.py) on the GPU against the
oracle's restatement: the statevector run step by step (dense magnetisation
and a Pauli sum), the noisy density-matrix run step by step and from scratch,
and the host helpers of tensorQ/density_matrix_sim.py."""
import numpy as np
import pytest
import torch

from oracle import ref

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built(cuda_ok):
    from qaravan_gb300 import build
    build.build()


def test_trotter_sv_sim_matches_oracle():
    from qaravan_gb300.applications import magnetization, trotter_sv_sim
    from qaravan_gb300.hamiltonians import TFI
    n, dt, steps = 6, 0.1, 5
    ham = TFI(n, jz=1.0, h=0.7)
    op = magnetization(n)
    got = trotter_sv_sim(ham, dt, steps, op)
    gates = ham.trotter_circ(dt, 1).gate_list
    cur = ref.initial_sv(n)
    want = []
    for _ in range(steps):
        cur = ref.run_sv(gates, n, init_state=cur).reshape(-1)
        want.append(np.vdot(cur, op @ cur).real)
    assert np.max(np.abs(np.array(got) - want)) < 1e-12
    terms = [(1.0, "z" + "i" * (n - 1)), (0.5, "i" * (n - 2) + "xx")]
    got_p = trotter_sv_sim(ham, dt, 3, terms)
    cur = ref.initial_sv(n)
    for s in range(3):
        cur = ref.run_sv(gates, n, init_state=cur).reshape(-1)
        assert abs(got_p[s] - sum(c * ref.pauli_expectation_sv(cur, p) for c, p in terms)) < 1e-12


def test_trotter_dm_sim_cached_and_uncached_match_oracle():
    from qaravan_gb300.applications import magnetization, trotter_dm_sim, trotter_dm_sim_uncached
    from qaravan_gb300.hamiltonians import TFI
    from qaravan_gb300.noise import PauliNoise
    n, dt, steps = 4, 0.1, 4
    ham = TFI(n, jz=1.0, h=0.9)
    # circuit-level Pauli noise is one channel over all sites after each layer (core/circuits.py:64-84)
    ch = PauliNoise(["iiii", "xiii", "iziz", "yyii", "iixx"], [0.92, 0.02, 0.03, 0.01, 0.02])
    op = magnetization(n)
    got = trotter_dm_sim(ham, dt, steps, ch, op)
    got_u = trotter_dm_sim_uncached(ham, dt, steps, ch, op)
    # cached: one step's layers (each followed by the channel) applied again and again
    c = ham.trotter_circ(dt, 1)
    c.build(ch)
    seq = [g for layer in c.layers for g in layer]
    rho = None
    want = []
    for _ in range(steps):
        rho = ref.run_dm(seq, n, init_state=rho, layered=False)
        want.append(np.trace(op @ rho.reshape(2 ** n, 2 ** n)).real)
    assert np.max(np.abs(np.array(got) - want)) < 1e-12
    # uncached: the layers of the whole num_steps circuit (the greedy layering may merge steps)
    want_u = []
    for k in range(1, steps + 1):
        c = ham.trotter_circ(dt, k)
        c.build(ch)
        r = ref.run_dm([g for layer in c.layers for g in layer], n, layered=False)
        want_u.append(np.trace(op @ r.reshape(2 ** n, 2 ** n)).real)
    assert np.max(np.abs(np.array(got_u) - want_u)) < 1e-12


def test_dm_host_helpers():
    from qaravan_gb300.tensorQ import all_zero_dm, expectation, partial_trace, random_dm, rdm_from_sv
    np.random.seed(3)
    rho = random_dm(4)
    assert abs(np.trace(rho) - 1) < 1e-12 and np.max(np.abs(rho - rho.conj().T)) < 1e-12
    assert all_zero_dm(3)[0, 0] == 1 and all_zero_dm(3).sum() == 1
    v = np.random.default_rng(1).normal(size=16) + 1j * np.random.default_rng(2).normal(size=16)
    v /= np.linalg.norm(v)
    full = np.outer(v, v.conj())
    for sites in ([2], [3, 0], [1, 2, 3]):
        assert np.max(np.abs(partial_trace(full, sites) - rdm_from_sv(v, sites))) < 1e-12
    assert abs(partial_trace(full, []) - 1) < 1e-12
    z = np.kron(np.diag([1, -1]), np.eye(8))
    assert abs(expectation(full, z) - np.vdot(v, z @ v).real) < 1e-12


def test_msp_infidelity_gradient_and_autodiff_loop():
    """The compilation loss (applications/compilation.py:73-90) with the torch
    backend: value and gradient against the oracle's autograd through the same
    dressed-CNOT circuit; a few Adam steps lower it."""
    from qaravan_gb300.applications import dressed_cnot_circ, msp_infidelity, msp_via_autodiff
    from qaravan_gb300.circuits import brickwall_skeleton
    from qaravan_gb300.environments import RunContext
    n = 3
    sk = brickwall_skeleton(n, 1, 2)
    rng = np.random.default_rng(51)
    in_states = [np.eye(2 ** n)[i] for i in (0, 5)]
    out_states = []
    for _ in range(2):
        v = rng.normal(size=2 ** n) + 1j * rng.normal(size=2 ** n)
        out_states.append(v / np.linalg.norm(v))
    p0 = rng.uniform(0, 2 * np.pi, size=len(sk) * 6 + n * 3)
    th = torch.tensor(p0, requires_grad=True)
    loss = msp_infidelity(th, sk, in_states, out_states, backend="torch")
    loss.backward()
    th2 = torch.tensor(p0, requires_grad=True)
    circ = dressed_cnot_circ(sk, n, th2)
    want = 0
    for a, b in zip(in_states, out_states):
        st = torch.tensor(a, dtype=torch.complex128).reshape([2] * n)
        for layer in ref.construct_layers(circ.gate_list):
            for g in layer:
                m = g.matrix if torch.is_tensor(g.matrix) else torch.tensor(np.asarray(g.matrix), dtype=torch.complex128)
                st = ref.op_action_torch(m, g.indices, st)
        want = want + 1 - torch.abs(torch.dot(st.reshape(-1).conj(), torch.tensor(b))) ** 2
    want = want / 2
    want.backward()
    assert abs(loss.item() - want.item()) < 1e-5  # complex64 statevector, as the reference's torch path
    assert torch.max(torch.abs(th.grad - th2.grad)).item() < 1e-4
    params, state = msp_via_autodiff(in_states, out_states, sk, init_params=p0, lr=0.05,
                                     context=RunContext(max_iter=15, quiet=True))
    assert state["cost_list"][-1] < state["cost_list"][0]


def test_trotter_applications_match_the_reference_outputs():
    """Fixture produced by the reference's own applications/trotter.py
    (make_golden.py gen_trotter_apps)."""
    from conftest import golden
    from qaravan_gb300.applications import magnetization, trotter_dm_sim, trotter_dm_sim_uncached, trotter_sv_sim
    from qaravan_gb300.hamiltonians import TFI
    from qaravan_gb300.noise import PauliNoise
    z = golden("trotter_apps.npz")
    assert np.max(np.abs(np.array(trotter_sv_sim(TFI(6, jz=1.0, h=0.7), 0.1, 5, magnetization(6))) - z["sv"])) < 1e-12
    ch = PauliNoise(["iiii", "xiii", "iziz", "yyii", "iixx"], [0.92, 0.02, 0.03, 0.01, 0.02])
    ham = TFI(4, jz=1.0, h=0.9)
    assert np.max(np.abs(np.array(trotter_dm_sim(ham, 0.1, 4, ch, magnetization(4))) - z["dm"])) < 1e-12
    assert np.max(np.abs(np.array(trotter_dm_sim_uncached(ham, 0.1, 4, ch, magnetization(4))) - z["dm_uncached"])) < 1e-12


def _msp_problem(n, sk, npairs, seed):
    rng = np.random.default_rng(seed)
    ins = [np.eye(2 ** n)[i] for i in rng.choice(2 ** n, size=npairs, replace=False)]
    outs = []
    for _ in range(npairs):
        v = rng.normal(size=2 ** n) + 1j * rng.normal(size=2 ** n)
        outs.append(v / np.linalg.norm(v))
    return ins, outs, rng.uniform(0, 2 * np.pi, size=len(sk) * 6 + n * 3)


def test_msp_environments_match_the_reference_outputs():
    """Fixture produced by the reference's own applications/compilation.py
    (make_golden.py gen_msp_env): single-gate environments, three sweeps of
    msp_via_environments (costs and every final gate matrix) and msp_cost."""
    from conftest import golden
    from qaravan_gb300.applications import (dressed_cnot_circ, msp_cost, msp_environment, msp_via_environments,
                                            string_to_sv)
    z = golden("msp_env.npz")
    n, sk, params = int(z["n"]), z["skeleton"].tolist(), z["params"]
    ins = [string_to_sv(str(s)) for s in z["in_strings"]]
    outs = list(z["outs"])
    ansatz = dressed_cnot_circ(sk, n, params)
    for i, want in zip(z["env_idx"], z["envs"]):
        assert np.max(np.abs(msp_environment(ins[1], ansatz, outs[1], int(i)) - want)) < 1e-12
    new, costs, term = msp_via_environments(ins, dressed_cnot_circ(sk, n, params), outs, num_sweeps=3)
    assert term == str(z["term"])
    assert np.max(np.abs(np.array(costs) - z["costs"])) < 1e-10
    for g, m, size in zip(new.gate_list, z["mats"], z["sizes"]):
        assert np.asarray(g.matrix).size == size
        assert np.max(np.abs(np.asarray(g.matrix).reshape(-1) - m[:size])) < 1e-10
    assert abs(msp_cost(params, sk, ins, z["target"]) - float(z["cost_mat"])) < 1e-12
    assert abs(msp_cost(params, sk, ins, outs) - float(z["cost_states"])) < 1e-12


def test_msp_environment_general_sites_against_oracle():
    """Environments on 9 qubits with pairs that are neither adjacent nor
    ascending, for one-site and two-site gates: env[a, b] equals the oracle's
    <out| ansatz with the gate set to |b><a| |in>, each matrix unit run through
    the whole circuit."""
    from qaravan_gb300.applications import dressed_cnot_circ, msp_environment
    n, sk = 9, [[0, 5], [7, 2], [3, 4], [8, 1], [6, 0]]
    ins, outs, params = _msp_problem(n, sk, 1, 3)
    ansatz = dressed_cnot_circ(sk, n, params)
    for gate_idx in (0, 3, 5, 11, len(ansatz.gate_list) - 2):
        g = ansatz.gate_list[gate_idx]
        d = 2 ** len(g.indices)
        env = msp_environment(ins[0], ansatz, outs[0], gate_idx)
        want = np.zeros((d, d), dtype=np.complex128)
        for a in range(d):
            for b in range(d):
                unit = np.zeros((d, d))
                unit[b, a] = 1.0
                gates = [type("G", (), {"name": h.name, "indices": list(h.indices),
                                        "matrix": unit if j == gate_idx else np.asarray(h.matrix)})()
                         for j, h in enumerate(ansatz.gate_list)]
                want[a, b] = np.vdot(outs[0], ref.run_sv(gates, n, init_state=ins[0]))
        if len(g.indices) == 1:
            assert np.max(np.abs(env - want)) < 1e-12
        else:  # the environment's rows and columns follow the sites in ascending order
            perm = [0, 2, 1, 3] if g.indices[0] > g.indices[1] else [0, 1, 2, 3]
            assert np.max(np.abs(env - want[np.ix_(perm, perm)])) < 1e-12


def test_msp_via_environments_cost_is_the_final_overlap():
    """Nine qubits, four pairs: every sweep's cost is non-increasing (each update
    is the optimal unitary for its environment) and the last cost squared is
    npairs - Re sum_p <out_p|A|in_p> of the final ansatz, run by the oracle."""
    from qaravan_gb300.applications import dressed_cnot_circ, msp_via_environments
    n, sk = 9, [[0, 1], [2, 3], [4, 5], [6, 7], [1, 2], [3, 4], [5, 6], [7, 8], [8, 0]]
    ins, outs, params = _msp_problem(n, sk, 4, 9)
    new, costs, term = msp_via_environments(ins, dressed_cnot_circ(sk, n, params), outs, num_sweeps=6)
    assert all(b <= a + 1e-12 for a, b in zip(costs, costs[1:]))
    gates = [type("G", (), {"name": g.name, "indices": list(g.indices), "matrix": np.asarray(g.matrix)})()
             for g in new.gate_list]
    amp = sum(np.vdot(o, ref.run_sv(gates, n, init_state=i)) for i, o in zip(ins, outs))
    assert abs(costs[-1] ** 2 - (len(ins) - amp.real)) < 1e-10
    for g in new.gate_list:
        if g.name[0] == "U":
            m = np.asarray(g.matrix)
            assert np.max(np.abs(m @ m.conj().T - np.eye(2))) < 1e-12

