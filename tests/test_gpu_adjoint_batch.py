"""Batched adjoint gradients for many parameter sets at once: energies and
angle gradients of every set against the single-set adjoint path (itself
checked against the reference autograd gradient and finite differences), the
device-built gate matrices against the host ParamGate matrices, and one set
against the exact parameter-shift rule in complex128."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built(cuda_ok):
    from qaravan_gb300 import build
    build.build()


def _tfi_terms(n):
    return [(1.0, "i" * q + "zz" + "i" * (n - q - 2)) for q in range(n - 1)] + \
           [(1.0, "i" * q + "x" + "i" * (n - q - 1)) for q in range(n)]


def test_device_param_matrices_match_param_gates():
    from qaravan_gb300.adjoint import BatchedAnsatz
    from qaravan_gb300.gates import RX, RXX, RY, RYY, RZ, RZZ
    gates = [("RX", [0], 0), ("RY", [1], 1), ("RZ", [2], 2), ("RXX", [0, 1], 3), ("RYY", [1, 2], 4), ("RZZ", [2, 0], 5)]
    ba = BatchedAnsatz(3, gates, dtype=torch.complex128)
    params = torch.tensor(np.random.default_rng(1).uniform(-3, 3, size=(4, 6)), dtype=torch.float64, device="cuda")
    mats = ba._matrices(params, 4).cpu().numpy()
    cls = {"RX": RX, "RY": RY, "RZ": RZ, "RXX": RXX, "RYY": RYY, "RZZ": RZZ}
    for s in range(4):
        for g, (name, idx, p) in enumerate(gates):
            want = np.asarray(cls[name](idx, float(params[s, p])).matrix)
            d = want.shape[0]
            assert np.max(np.abs(mats[s, g, :d * d].reshape(d, d) - want)) < 1e-12


@pytest.mark.parametrize("dtype,tol", [(torch.complex64, 2e-5), (torch.complex128, 1e-10)])
def test_batched_gradients_match_single_set_adjoint(dtype, tol):
    from qaravan_gb300 import StatevectorSim, workloads
    from qaravan_gb300.adjoint import BatchedAnsatz, adjoint_energy
    n, layers, P = 8, 3, 5
    terms = _tfi_terms(n)
    ba = BatchedAnsatz.hea(n, layers, dtype=dtype)
    sets = np.stack([workloads.hea_params(n, layers, 10 + s) for s in range(P)])  # (P, layers, n, 2)
    E, grad = ba.energy_and_grad(sets.reshape(P, -1), terms)
    E, grad = E.cpu().numpy(), grad.cpu().numpy()
    for s in range(P):
        t = torch.tensor(sets[s], dtype=torch.float64, requires_grad=True)
        sim = StatevectorSim(workloads.hea_circuit(n, layers, t), dtype=dtype)
        e = adjoint_energy(sim, terms)
        e.backward()
        g1 = t.grad.numpy().reshape(-1)
        assert abs(float(e) - E[s]) < tol * max(1.0, abs(E[s])) * 10
        assert np.max(np.abs(grad[s] - g1)) / max(np.max(np.abs(g1)), 1e-12) < tol


def test_batched_gradient_matches_parameter_shift():
    """Each angle enters one gate exp(-i theta P), so the energy is
    a + b cos(2 theta) + c sin(2 theta) in it and dE/dtheta = E(theta + pi/4)
    - E(theta - pi/4) exactly; the shifted sets run as one batch."""
    from qaravan_gb300 import workloads
    from qaravan_gb300.adjoint import BatchedAnsatz
    n, layers = 6, 2
    terms = _tfi_terms(n)
    ba = BatchedAnsatz.hea(n, layers, dtype=torch.complex128)
    x0 = workloads.hea_params(n, layers, 3).reshape(-1)
    _, grad = ba.energy_and_grad(x0[None, :], terms)
    P = len(x0)
    shifts = np.concatenate([np.tile(x0, (P, 1)) + np.pi / 4 * np.eye(P), np.tile(x0, (P, 1)) - np.pi / 4 * np.eye(P)])
    e, _ = ba.energy_and_grad(shifts, terms)
    e = e.cpu().numpy()
    assert np.max(np.abs(grad.cpu().numpy()[0] - (e[:P] - e[P:]))) < 1e-10


@pytest.mark.parametrize("dtype,tol", [(torch.complex64, 2e-5), (torch.complex128, 1e-10)])
def test_all_rotation_kinds_and_shared_parameters(dtype, tol):
    """RX..RZZ, a fixed gate and a parameter used by two gates: batched gradients
    against the parameter-shift rule, evaluated by shifting one gate's angle at a
    time (a shared parameter's derivative is the sum over its gates)."""
    from qaravan_gb300.adjoint import BatchedAnsatz
    from qaravan_gb300.gates import CNOT
    n = 6
    cx = CNOT([2, 1], n)
    gates = [("RX", [0], 0), ("RY", [1], 1), ("RZ", [2], 2), ("RXX", [0, 1], 3), ("RYY", [2, 3], 4),
             ("RZZ", [3, 5], 5), ("fixed", list(cx.indices), np.asarray(cx.matrix)), ("RX", [4], 0),
             ("RYY", [5, 1], 3), ("RY", [3], 6)]
    terms = _tfi_terms(n) + [(0.4, "xyiiiz")]
    ba = BatchedAnsatz(n, gates, dtype=dtype)
    rng = np.random.default_rng(12)
    P = 3
    x = rng.uniform(-2, 2, size=(P, ba.nparams))
    _, grad = ba.energy_and_grad(x, terms)
    grad = grad.cpu().numpy()
    # per-gate angles: a structure with one private parameter per rotation gate
    rot = [i for i, g in enumerate(gates) if g[0] != "fixed"]
    private = [(g[0], g[1], rot.index(i)) if g[0] != "fixed" else g for i, g in enumerate(gates)]
    bp = BatchedAnsatz(n, private, dtype=torch.complex128)
    for s in range(P):
        th = np.array([x[s, gates[i][2]] for i in rot])
        R = len(rot)
        sh = np.concatenate([np.tile(th, (R, 1)) + np.pi / 4 * np.eye(R), np.tile(th, (R, 1)) - np.pi / 4 * np.eye(R)])
        e, _ = bp.energy_and_grad(sh, terms)
        e = e.cpu().numpy()
        per_gate = e[:R] - e[R:]
        want = np.zeros(ba.nparams)
        for j, i in enumerate(rot):
            want[gates[i][2]] += per_gate[j]
        assert np.max(np.abs(grad[s] - want)) / np.max(np.abs(want)) < tol


@pytest.mark.parametrize("dtype,tol", [(torch.complex64, 1e-5), (torch.complex128, 1e-11)])
def test_fused_forward_matches_per_gate_forward(dtype, tol):
    """The forward as fused 3- and 4-qubit blocks composed per parameter set on
    the device (the default) against one tile-pass op per gate, at 15 qubits
    (tiles smaller than the state), with mixed rotation kinds and a shared angle."""
    from qaravan_gb300.adjoint import BatchedAnsatz
    from qaravan_gb300.gates import CNOT
    n, P = 15, 4
    gates = []
    for l in range(3):
        for q in range(n):
            gates.append((("RY", "RX", "RZ")[(q + l) % 3], [q], 2 * (l * n + q)))
            gates.append(("RZ", [q], 2 * (l * n + q) + 1))
        for q in range(0, n - 1, 2):
            gates.append(("RZZ", [q, q + 1], 2 * l * n))
        for q in range(1, n - 1, 2):
            g = CNOT([q + 1, q], n)
            gates.append(("fixed", list(g.indices), np.asarray(g.matrix)))
    terms = _tfi_terms(n)
    rng = np.random.default_rng(4)
    x = rng.uniform(-2, 2, size=(P, 2 * 3 * n))
    ref_ba = BatchedAnsatz(n, gates, nparams=x.shape[1], dtype=dtype, fused_width=0)
    assert ref_ba._fused is None
    e0, g0 = (t.cpu().numpy() for t in ref_ba.energy_and_grad(x, terms))
    for width in (3, 4):
        ba = BatchedAnsatz(n, gates, nparams=x.shape[1], dtype=dtype, fused_width=width)
        assert ba._fused is not None and ba._fused["blocks"] < len(gates)
        e1, g1 = (t.cpu().numpy() for t in ba.energy_and_grad(x, terms))
        assert np.max(np.abs(e1 - e0)) < tol * np.max(np.abs(e0)) * 10
        assert np.max(np.abs(g1 - g0)) / np.max(np.abs(g0)) < tol


def test_large_tiles_single_cta_launch():
    """12-bit tiles of both vectors (128 KiB of shared memory: one CTA per SM,
    256 threads for complex64) against one pass per gate."""
    from qaravan_gb300 import workloads
    from qaravan_gb300.adjoint import BatchedAnsatz
    n, layers, P = 14, 2, 3
    terms = _tfi_terms(n)
    x = np.stack([workloads.hea_params(n, layers, 40 + s).reshape(-1) for s in range(P)])
    base = BatchedAnsatz.hea(n, layers)
    e0, g0 = (t.cpu().numpy() for t in BatchedAnsatz(n, base.gates, nparams=base.nparams, tile_bits=0)
              .energy_and_grad(x, terms))
    e1, g1 = (t.cpu().numpy() for t in BatchedAnsatz(n, base.gates, nparams=base.nparams, tile_bits=12)
              .energy_and_grad(x, terms))
    assert np.max(np.abs(e1 - e0)) < 1e-5
    assert np.max(np.abs(g1 - g0)) / np.max(np.abs(g0)) < 2e-5
