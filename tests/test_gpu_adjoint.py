"""Adjoint gradients vs the reference's torch autograd (fixture), the oracle's
exact reverse sweep, and central finite differences (complex128)."""
import numpy as np
import pytest
import torch

from conftest import golden
from oracle import ref

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built(cuda_ok):
    from qaravan_gb300 import build
    build.build()


def _hea_grad(n, layers, params, dtype, terms, mode="sweep"):
    from qaravan_gb300 import StatevectorSim, workloads
    from qaravan_gb300.adjoint import adjoint_energy
    th = torch.tensor(params, dtype=torch.float64, requires_grad=True)
    sim = StatevectorSim(workloads.hea_circuit(n, layers, th), dtype=dtype, mode=mode)
    e = adjoint_energy(sim, terms)
    e.backward()
    return float(e.item()), th.grad.numpy().copy()


@pytest.mark.parametrize("dtype", [torch.complex64, torch.complex128])
def test_energy_gradient_matches_reference_autograd(dtype):
    from qaravan_gb300.hamiltonians import TFI
    z = golden("grad_hea6.npz")
    n, layers = int(z["n"]), int(z["layers"])
    e, g = _hea_grad(n, layers, z["params"], dtype, TFI(n, 1, 1).pauli_sum())
    assert abs(e - float(z["energy"])) < 1e-5
    rel = np.max(np.abs(g - z["grad"])) / np.max(np.abs(z["grad"]))
    assert rel < 1e-5 if dtype == torch.complex128 else rel < 2e-5


def test_energy_gradient_central_differences_c128():
    from qaravan_gb300 import workloads
    from qaravan_gb300.hamiltonians import TFI
    n, layers = 8, 3
    params = workloads.hea_params(n, layers, 21)
    terms = TFI(n, 1, 1).pauli_sum()
    e, g = _hea_grad(n, layers, params, torch.complex128, terms)
    rng = np.random.default_rng(0)
    eps = 1e-5
    for _ in range(12):
        idx = (rng.integers(layers), rng.integers(n), rng.integers(2))
        pp, pm = params.copy(), params.copy()
        pp[idx] += eps
        pm[idx] -= eps
        fd = (ref.energy(workloads.hea_circuit(n, layers, pp).gate_list, n, terms)
              - ref.energy(workloads.hea_circuit(n, layers, pm).gate_list, n, terms)) / (2 * eps)
        assert abs(fd - g[idx]) < 1e-7


def test_matrix_gradients_match_oracle_reverse_sweep():
    """Raw dL/dM for every gate (fixed and parametrised) against the oracle."""
    from qaravan_gb300 import StatevectorSim, workloads
    from qaravan_gb300.adjoint import adjoint_energy
    from qaravan_gb300.circuits import Circuit
    from qaravan_gb300.gates import Gate
    from qaravan_gb300.hamiltonians import TFI
    n = 9
    gates = workloads.brickwork_gates(n, 2, 8)
    tg = [Gate(g.name, g.indices, torch.tensor(np.asarray(g.matrix), dtype=torch.complex128, requires_grad=True))
          for g in gates]
    terms = TFI(n, 1, 1).pauli_sum()
    sim = StatevectorSim(Circuit(tg, n=n), dtype=torch.complex128)
    adjoint_energy(sim, terms).backward()
    seq = [g for layer in ref.construct_layers(gates) for g in layer]
    exp = ref.matrix_gradients(seq, n, terms)
    by_id = {id(g): e for g, e in zip(seq, exp)}
    for g, t in zip(gates, tg):
        assert np.max(np.abs(t.matrix.grad.numpy() - by_id[id(g)])) < 1e-10


def test_state_function_with_arbitrary_loss():
    """run() returns a differentiable state; any torch loss on it back-propagates
    through the adjoint sweep (the reference's compilation loop pattern)."""
    from qaravan_gb300 import StatevectorSim, workloads
    n, layers = 7, 2
    params = workloads.hea_params(n, layers, 5)
    th = torch.tensor(params, dtype=torch.float64, requires_grad=True)
    sim = StatevectorSim(workloads.hea_circuit(n, layers, th), dtype=torch.complex128)
    sv = sim.get_statevector()
    target = torch.zeros(2 ** n, dtype=torch.complex128, device=sv.device)
    target[5] = 1
    loss = 1 - torch.abs(torch.vdot(target, sv)) ** 2 + torch.real(sv[0] * sv[1].conj())
    loss.backward()
    g = th.grad.numpy().copy()
    # same loss through the oracle's op_action on CPU torch tensors with torch autograd
    th2 = torch.tensor(params, dtype=torch.float64, requires_grad=True)
    circ = workloads.hea_circuit(n, layers, th2)
    st = torch.zeros([2] * n, dtype=torch.complex128)
    st.view(-1)[0] = 1
    for layer in ref.construct_layers(circ.gate_list):
        for gate in layer:
            m = gate.matrix if torch.is_tensor(gate.matrix) else torch.tensor(np.asarray(gate.matrix), dtype=torch.complex128)
            st = ref.op_action_torch(m, gate.indices, st)
    sv2 = st.reshape(-1)
    loss2 = 1 - torch.abs(sv2[5]) ** 2 + torch.real(sv2[0] * sv2[1].conj())
    loss2.backward()
    assert abs(loss.item() - loss2.item()) < 1e-12
    assert np.max(np.abs(g - th2.grad.numpy())) < 1e-10


def test_adjoint_memory_is_state_sized():
    from qaravan_gb300 import StatevectorSim, workloads
    from qaravan_gb300.adjoint import adjoint_energy
    from qaravan_gb300.hamiltonians import TFI
    n, layers = 22, 6
    th = torch.tensor(workloads.hea_params(n, layers, 1), dtype=torch.float64, requires_grad=True)
    sim = StatevectorSim(workloads.hea_circuit(n, layers, th), dtype=torch.complex64)
    torch.cuda.synchronize()
    torch.cuda.reset_peak_memory_stats()
    base = torch.cuda.memory_allocated()
    e = adjoint_energy(sim, TFI(n, 1, 1).pauli_sum())
    e.backward()
    torch.cuda.synchronize()
    peak = torch.cuda.max_memory_allocated() - base
    state = 2 ** n * 8
    assert peak < 5 * state, peak / state
    assert np.all(np.isfinite(th.grad.numpy()))
