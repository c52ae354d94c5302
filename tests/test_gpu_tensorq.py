"""The reference-named free functions of ``qaravan_gb300.tensorQ`` against the
oracle's restatement of ``tensorQ/statevector_sim.py``: op_action (NumPy and
torch, shapes, autograd to state and operator), partial_overlap and
rdm_from_sv for 0 to 5 sites, pauli_expectation_sv, measurements (repeatable
under numpy.random.seed, distribution, collapse)."""
import numpy as np
import pytest
import torch

from oracle import ref

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built(cuda_ok):
    from qaravan_gb300 import build
    build.build()


def _sv(n, seed):
    rng = np.random.default_rng(seed)
    v = rng.normal(size=2 ** n) + 1j * rng.normal(size=2 ** n)
    return v / np.linalg.norm(v)


def _haar(d, rng):
    q, r = np.linalg.qr(rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d)))
    return q * (np.diag(r) / np.abs(np.diag(r)))


@pytest.mark.parametrize("indices", [[3], [4, 1], [0, 6, 2], [5, 2, 7, 0]])
def test_op_action_numpy_matches_oracle(indices):
    from qaravan_gb300.tensorQ import op_action
    n = 8
    rng = np.random.default_rng(len(indices))
    sv = _sv(n, 1)
    op = _haar(2 ** len(indices), rng)
    got = op_action(op, indices, sv)
    assert isinstance(got, np.ndarray) and got.shape == sv.shape
    assert np.max(np.abs(got - ref.op_action(op, indices, sv))) < 1e-12
    t = sv.reshape([2] * n)
    got_t = op_action(op.reshape([2] * 2 * len(indices)), indices, t)
    assert got_t.shape == t.shape
    assert np.max(np.abs(got_t.reshape(-1) - got)) < 1e-12


def test_op_action_torch_autograd_matches_oracle_autograd():
    from qaravan_gb300.tensorQ import op_action
    n = 7
    rng = np.random.default_rng(3)
    u1, u2 = _haar(4, rng), _haar(8, rng)
    target = torch.tensor(_sv(n, 9))

    def loss_of(fn, sv, a, b):
        s = fn(b, [5, 1, 3], fn(a, [2, 0], sv))
        return 1 - torch.abs(torch.vdot(target.to(s.device), s)) ** 2 + torch.real(s[0] * s[3].conj())

    sv0 = torch.tensor(_sv(n, 4), requires_grad=True)
    a0 = torch.tensor(u1, requires_grad=True)
    b0 = torch.tensor(u2, requires_grad=True)
    l0 = loss_of(op_action, sv0.cuda(), a0, b0)
    l0.backward()
    sv1 = torch.tensor(_sv(n, 4), requires_grad=True)
    a1 = torch.tensor(u1, requires_grad=True)
    b1 = torch.tensor(u2, requires_grad=True)

    def oracle_fn(op, idx, s):
        return ref.op_action_torch(op, idx, s.reshape([2] * n)).reshape(-1)

    l1 = loss_of(oracle_fn, sv1, a1, b1)
    l1.backward()
    assert abs(l0.item() - l1.item()) < 1e-12
    for x, y in ((sv0, sv1), (a0, a1), (b0, b1)):
        assert torch.max(torch.abs(x.grad - y.grad)).item() < 1e-10


@pytest.mark.parametrize("skip", [None, [4], [6, 1], [5, 0, 3], [7, 2, 4, 0, 6]])
@pytest.mark.parametrize("dtype", [np.complex128, np.complex64])
def test_partial_overlap_and_rdm_match_oracle(skip, dtype):
    from qaravan_gb300.tensorQ import partial_overlap, rdm_from_sv
    n = 9
    a, b = _sv(n, 5).astype(dtype), _sv(n, 6).astype(dtype)
    tol = 1e-12 if dtype == np.complex128 else 1e-6
    got = partial_overlap(a, b, skip=skip)
    want = ref.partial_overlap(a.astype(np.complex128), b.astype(np.complex128), skip=skip)
    assert got.shape == want.shape
    assert np.max(np.abs(got - want)) < tol
    if skip:
        rho = rdm_from_sv(a, skip)
        assert abs(np.trace(rho) - 1) < tol * 10 and np.max(np.abs(rho - rho.conj().T)) < tol


def test_partial_overlap_torch_inputs_and_batchless_inner_product():
    from qaravan_gb300.tensorQ import partial_overlap
    n = 10
    a, b = _sv(n, 7), _sv(n, 8)
    got = partial_overlap(torch.tensor(a).cuda(), torch.tensor(b).cuda(), skip=[9, 3, 0])
    assert torch.is_tensor(got) and got.is_cuda
    assert np.max(np.abs(got.cpu().numpy() - ref.partial_overlap(a, b, skip=[9, 3, 0]))) < 1e-12
    assert abs(partial_overlap(a, b)[0, 0] - np.vdot(b, a)) < 1e-12


def test_pauli_expectation_sv_matches_oracle():
    from qaravan_gb300.tensorQ import pauli_expectation_sv
    n = 8
    sv = _sv(n, 11)
    for s in ["zzixiiyi", "xxxxxxxx", "iiiiiiii", "yzyzyzyz"]:
        assert abs(pauli_expectation_sv(sv, s) - ref.pauli_expectation_sv(sv, s)) < 1e-12


def test_measurements_repeatable_distributed_and_collapsed():
    from qaravan_gb300.tensorQ import measure_and_collapse_sv, measure_sv, rdm_from_sv
    n = 8
    sv = _sv(n, 12)
    np.random.seed(5)
    a = measure_sv(sv, [6, 1, 3], shots=2000)
    np.random.seed(5)
    b = measure_sv(sv, [6, 1, 3], shots=2000)
    assert a == b and all(len(x) == 3 for x in a)
    p = np.real(np.diag(rdm_from_sv(sv, [6, 1, 3])))
    freq = np.bincount([int(x, 2) for x in a], minlength=8) / 2000
    assert np.all(np.abs(freq - p) < 5 * np.sqrt(p * (1 - p) / 2000) + 1e-3)
    assert isinstance(measure_sv(sv, [2]), str)
    out, post = measure_and_collapse_sv(sv, [4, 0])
    assert post.shape == (2 ** (n - 2),) and abs(np.linalg.norm(post) - 1) < 1e-12
    want = ref.collapse_sv(sv, [4, 0], out) if hasattr(ref, "collapse_sv") else None
    if want is not None:
        assert np.max(np.abs(post - want.reshape(-1))) < 1e-12


def test_reference_default_simulators_return_numpy_complex128():
    """tensorQ.StatevectorSim(circ) / DensityMatrixSim(circ, nm=...) with the
    reference's defaults: NumPy results in complex128, against the reference's
    own outputs (fixtures)."""
    from conftest import golden
    from gateio import unpack_gates
    from qaravan_gb300.circuits import Circuit
    from qaravan_gb300.gates import CNOT, H
    from qaravan_gb300.noise import QubitNoise
    from qaravan_gb300.paulis import pauli_Z
    from qaravan_gb300.tensorQ import DensityMatrixSim, StatevectorSim
    z = golden("sv_brickwork12.npz")
    sim = StatevectorSim(Circuit(unpack_gates(z), n=int(z["n"])))
    sv = sim.get_statevector()
    assert isinstance(sv, np.ndarray) and sv.dtype == np.complex128
    assert np.max(np.abs(sv - z["sv"])) < 1e-12
    state = sim.run(progress_bar=False)
    assert isinstance(state, np.ndarray) and state.shape == (2,) * int(z["n"])
    k = golden("dm_kats.npz")
    dm = DensityMatrixSim(Circuit([H(0), CNOT([1, 0], 3), CNOT([2, 1], 3)], 3), nm=QubitNoise(1000, 1000, 1, 5))
    rho = dm.get_density_matrix()
    assert isinstance(rho, np.ndarray) and np.max(np.abs(rho - k["thermal_dm"])) < 1e-12
    assert abs(dm.local_expectation([pauli_Z] * 3) - 0.020609303627304454) < 1e-12


def test_reference_torch_backend_compilation_pattern():
    """The reference's compilation loss (applications/compilation.py:73-90):
    StatevectorSim(ansatz, backend="torch", init_state=...) on the default CPU
    device, torch.dot against a CPU target, backward to the angles -- against
    the same loss through the oracle's torch op_action (complex64 results)."""
    from qaravan_gb300 import workloads
    from qaravan_gb300.tensorQ import StatevectorSim
    n, layers = 6, 2
    params = workloads.hea_params(n, layers, 13)
    rng = np.random.default_rng(14)
    in_state, out_state = _sv(n, 15), _sv(n, 16)
    th = torch.tensor(params, dtype=torch.float64, requires_grad=True)
    sim = StatevectorSim(workloads.hea_circuit(n, layers, th), backend="torch", init_state=in_state)
    sim.run(progress_bar=False)
    ansatz_sv = sim.get_statevector()
    assert ansatz_sv.device.type == "cpu" and ansatz_sv.dtype == torch.complex64
    target = torch.tensor(out_state, dtype=torch.complex128)
    loss = 1 - torch.abs(torch.dot(ansatz_sv.to(torch.complex128).conj(), target)) ** 2
    loss.backward()
    th2 = torch.tensor(params, dtype=torch.float64, requires_grad=True)
    circ = workloads.hea_circuit(n, layers, th2)
    st = torch.tensor(in_state, dtype=torch.complex128).reshape([2] * n)
    for layer in ref.construct_layers(circ.gate_list):
        for g in layer:
            m = g.matrix if torch.is_tensor(g.matrix) else torch.tensor(np.asarray(g.matrix), dtype=torch.complex128)
            st = ref.op_action_torch(m, g.indices, st)
    loss2 = 1 - torch.abs(torch.dot(st.reshape(-1).conj(), target)) ** 2
    loss2.backward()
    assert abs(loss.item() - loss2.item()) < 1e-5
    assert torch.max(torch.abs(th.grad - th2.grad)).item() < 1e-4
