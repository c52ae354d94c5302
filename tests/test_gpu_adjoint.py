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


@pytest.mark.parametrize("n,layers,count", [(14, 2, None), (24, 4, 64)])
def test_energy_gradient_parameter_shift_c128(n, layers, count):
    """The complex128 adjoint gradient of the TFI energy of the hardware-efficient
    ansatz against the exact parameter-shift rule: every angle enters one
    exp(-i theta P) gate, so dE/dtheta = E(theta + pi/4) - E(theta - pi/4). All
    angles at 14 qubits; 64 seeded angles at 24 qubits. Shifted energies by the
    complex128 simulator (itself pinned to the oracle)."""
    from qaravan_gb300 import StatevectorSim, workloads
    from qaravan_gb300.hamiltonians import TFI
    params = workloads.hea_params(n, layers, 5)
    terms = TFI(n, 1, 1).pauli_sum()
    _, g = _hea_grad(n, layers, params, torch.complex128, terms)
    flat = np.arange(params.size)
    if count is not None:
        flat = np.random.default_rng(8).choice(params.size, size=count, replace=False)
    worst = 0.0
    for f in flat:
        idx = np.unravel_index(f, params.shape)
        e = []
        for sgn in (1, -1):
            p = params.copy()
            p[idx] += sgn * np.pi / 4
            e.append(StatevectorSim(workloads.hea_circuit(n, layers, p), dtype=torch.complex128)
                     .pauli_sum_expectation(terms))
        worst = max(worst, abs((e[0] - e[1]) - g[idx]))
    assert worst < 1e-10


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
    assert peak < 3.5 * state, peak / state  # state, co-state and the uncomputed copy
    assert np.all(np.isfinite(th.grad.numpy()))


def _oracle_loss_grad(gates, n, terms, leaves):
    """sum_t c_t <psi|P_t|psi> through the oracle's torch op_action with torch
    autograd (matrix_exp included), and the gradients of ``leaves``."""
    st = torch.zeros([2] * n, dtype=torch.complex128)
    st.view(-1)[0] = 1
    for layer in ref.construct_layers(gates):
        for gate in layer:
            m = gate.matrix if torch.is_tensor(gate.matrix) else torch.tensor(np.asarray(gate.matrix), dtype=torch.complex128)
            st = ref.op_action_torch(m, gate.indices, st)
    pauli = {"x": [[0, 1], [1, 0]], "y": [[0, -1j], [1j, 0]], "z": [[1, 0], [0, -1]]}
    e = 0
    for c, s in terms:
        v = st
        for q, ch in enumerate(s):
            if ch != "i":
                v = ref.op_action_torch(torch.tensor(pauli[ch], dtype=torch.complex128), [q], v)
        e = e + c * torch.vdot(st.reshape(-1), v.reshape(-1)).real
    e.backward()
    return float(e), [l.grad.numpy().copy() for l in leaves]


def _mixed_circuit(th, free):
    """Rotations on angles of ``th`` (one angle used twice) and a dense gate whose
    matrix ``free`` is itself a leaf."""
    from qaravan_gb300.circuits import Circuit
    from qaravan_gb300.gates import CNOT, Gate, RX, RXX, RY, RYY, RZ, RZZ
    n = 5
    gates = [RX([0], th[0]), RY([1], th[1]), RZ([2], th[2]), RXX([0, 1], th[3]), RYY([2, 3], th[4]),
             RZZ([3, 4], th[5]), Gate("free", [1, 2], free), CNOT([2, 1], n), RX([4], th[0]), RY([3], th[6])]
    return Circuit(gates, n=n), n


@pytest.mark.parametrize("when", ["before_sim", "inside_sim"])
def test_rotation_angles_mixed_with_matrix_leaves_and_replaced_gates(when):
    """Angles and matrix leaves get the oracle's autograd gradients. A rotation
    whose matrix is replaced (update_gate) before the simulator is built comes
    back from the angles, as the reference's simulator copies the circuit
    (core/base_sim.py:11, core/param_gates.py:48-49); one replaced in the
    simulator's own built circuit keeps the new matrix and its angle gets no
    gradient from it."""
    from qaravan_gb300 import StatevectorSim
    from qaravan_gb300.adjoint import adjoint_energy
    from qaravan_gb300.hamiltonians import TFI
    rng = np.random.default_rng(3)
    p = rng.uniform(-2, 2, size=7)
    q, _ = np.linalg.qr(rng.normal(size=(4, 4)) + 1j * rng.normal(size=(4, 4)))
    rep = np.linalg.qr(rng.normal(size=(2, 2)) + 1j * rng.normal(size=(2, 2)))[0]
    terms = TFI(5, 1, 0.7).pauli_sum()
    th = torch.tensor(p, requires_grad=True)
    fr = torch.tensor(q, requires_grad=True)
    c, n = _mixed_circuit(th, fr)
    last = len(c.gate_list) - 1
    if when == "before_sim":
        c.update_gate(last, rep)
        sim = StatevectorSim(c, dtype=torch.complex128)
    else:
        sim = StatevectorSim(c, dtype=torch.complex128)
        sim.circ.construct_layers()
        sim.circ.update_gate(last, rep)
    e = adjoint_energy(sim, terms)
    e.backward()
    th2 = torch.tensor(p, requires_grad=True)
    fr2 = torch.tensor(q, requires_grad=True)
    c2, _ = _mixed_circuit(th2, fr2)
    if when == "inside_sim":
        c2.update_gate(last, rep)
    e2, (g_th, g_fr) = _oracle_loss_grad(c2.gate_list, n, terms, [th2, fr2])
    assert abs(float(e) - e2) < 1e-12
    assert np.max(np.abs(th.grad.numpy() - g_th)) < 1e-9  # matrix_exp's own derivative error is ~1e-10
    if when == "inside_sim":
        assert g_th[6] == 0 and th.grad[6] == 0
    else:
        assert abs(g_th[6]) > 1e-3
    assert np.max(np.abs(fr.grad.numpy() - g_fr)) < 1e-10


@pytest.mark.parametrize("init", ["bitstring", "array"])
def test_adjoint_energy_starts_from_the_initial_state(init):
    """The differentiable run starts where StatevectorSim.initialize_state does
    (core/base_sim.py:30-53 with tensorQ/statevector_sim.py:31-48): energy and
    gradients against the oracle's autograd from the same initial state."""
    from qaravan_gb300 import StatevectorSim, workloads
    from qaravan_gb300.adjoint import adjoint_energy
    from qaravan_gb300.hamiltonians import TFI
    n, layers = 6, 2
    params = workloads.hea_params(n, layers, 31)
    rng = np.random.default_rng(32)
    if init == "bitstring":
        init_state = "011010"
    else:
        v = rng.normal(size=2 ** n) + 1j * rng.normal(size=2 ** n)
        init_state = v / np.linalg.norm(v)
    terms = TFI(n, 1, 0.6).pauli_sum()
    th = torch.tensor(params, dtype=torch.float64, requires_grad=True)
    e = adjoint_energy(StatevectorSim(workloads.hea_circuit(n, layers, th), init_state=init_state,
                                      dtype=torch.complex128), terms)
    e.backward()
    th2 = torch.tensor(params, dtype=torch.float64, requires_grad=True)
    circ = workloads.hea_circuit(n, layers, th2)
    st = torch.tensor(ref.initial_sv(n, init_state), dtype=torch.complex128).reshape([2] * n)
    for layer in ref.construct_layers(circ.gate_list):
        for g in layer:
            m = g.matrix if torch.is_tensor(g.matrix) else torch.tensor(np.asarray(g.matrix), dtype=torch.complex128)
            st = ref.op_action_torch(m, g.indices, st)
    pauli = {"x": [[0, 1], [1, 0]], "y": [[0, -1j], [1j, 0]], "z": [[1, 0], [0, -1]]}
    e2 = 0
    for c, s in terms:
        v = st
        for q, ch in enumerate(s):
            if ch != "i":
                v = ref.op_action_torch(torch.tensor(pauli[ch], dtype=torch.complex128), [q], v)
        e2 = e2 + c * torch.vdot(st.reshape(-1), v.reshape(-1)).real
    e2.backward()
    assert abs(float(e) - float(e2)) < 1e-12
    assert torch.max(torch.abs(th.grad - th2.grad)).item() < 1e-9


def test_parameters_on_the_device():
    """Angles living on the GPU (one parameter tensor, and separate scalars): the
    same energy and gradient as host angles, the gradient on the angles' device."""
    from qaravan_gb300 import StatevectorSim, workloads
    from qaravan_gb300.adjoint import adjoint_energy
    from qaravan_gb300.hamiltonians import TFI
    n, layers = 8, 3
    params = workloads.hea_params(n, layers, 12)
    terms = TFI(n, 1, 1).pauli_sum()
    e_host, g_host = _hea_grad(n, layers, params, torch.complex64, terms)
    th = torch.tensor(params, dtype=torch.float64, device="cuda", requires_grad=True)
    e = adjoint_energy(StatevectorSim(workloads.hea_circuit(n, layers, th), dtype=torch.complex64), terms)
    e.backward()
    assert th.grad.is_cuda
    assert abs(float(e.item()) - e_host) < 1e-12
    assert np.max(np.abs(th.grad.cpu().numpy() - g_host)) < 1e-12
    scalars = [torch.tensor(float(v), dtype=torch.float64, device="cuda", requires_grad=True) for v in params.reshape(-1)]
    th2 = torch.stack(scalars).reshape(params.shape)  # not a view of one leaf: the stacked path
    e2 = adjoint_energy(StatevectorSim(workloads.hea_circuit(n, layers, th2), dtype=torch.complex64), terms)
    e2.backward()
    got = np.array([s.grad.item() for s in scalars]).reshape(params.shape)
    assert abs(float(e2.item()) - e_host) < 1e-12 and np.max(np.abs(got - g_host)) < 1e-12
