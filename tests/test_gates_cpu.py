"""Gate-object behaviour that decides numbers: rotation matrices against the
closed form expm(-i t P) = cos t I - i sin t P, and Circuit.copy() semantics of
parametrised gates (a copy is rebuilt from the angles, so a matrix replaced by
update_gate does not survive the copy; an untouched matrix is shared)."""
import numpy as np
import torch

from qaravan_gb300.circuits import Circuit
from qaravan_gb300.gates import RX, RXX, RY, RYY, RZ, RZZ

PX = np.array([[0, 1], [1, 0]], dtype=complex)
PY = np.array([[0, -1j], [1j, 0]])
PZ = np.diag([1.0, -1.0]).astype(complex)
GEN = {RX: PX, RY: PY, RZ: PZ, RXX: np.kron(PX, PX), RYY: np.kron(PY, PY), RZZ: np.kron(PZ, PZ)}


def test_rotation_matrices_closed_form():
    for cls, P in GEN.items():
        idx = [0] if P.shape[0] == 2 else [0, 1]
        for t in (0.3, -1.7, 2.9):
            want = np.cos(t) * np.eye(P.shape[0]) - 1j * np.sin(t) * P
            assert np.max(np.abs(np.asarray(cls(idx, t).matrix) - want)) < 1e-14
            tm = cls(idx, torch.tensor(t, dtype=torch.float64)).matrix
            assert np.max(np.abs(tm.detach().numpy() - want)) < 1e-9  # torch.linalg.matrix_exp accuracy


def test_copy_shares_angle_built_matrix_and_keeps_autograd():
    th = torch.tensor([0.4, -0.9], dtype=torch.float64, requires_grad=True)
    c = Circuit([RY([0], th[0]), RZZ([0, 1], th[1])], n=2)
    c2 = c.copy()
    for g, h in zip(c.gate_list, c2.gate_list):
        assert h.matrix is g.matrix and h.built_from_angles()
        assert h.indices == g.indices and h.indices is not g.indices
    c2.gate_list[0].matrix.real.sum().backward()
    assert th.grad is not None and th.grad[0] != 0


def test_copy_rebuilds_a_replaced_matrix_from_angles():
    c = Circuit([RX([0], 0.7), RY([1], 0.2)], n=2)
    new = np.eye(2, dtype=complex) * 1j
    c.update_gate(0, new)
    assert not c.gate_list[0].built_from_angles()
    c2 = c.copy()
    assert np.max(np.abs(np.asarray(c2.gate_list[0].matrix) - np.asarray(RX([0], 0.7).matrix))) < 1e-15
    assert c2.gate_list[0].built_from_angles()


def _decomp_circuit(z, requires_decomp):
    from qaravan_gb300.circuits import Circuit
    from qaravan_gb300.gates import CNOT, H, U
    n = int(z["n"])
    a, m = z["angles"], z["mats"]
    gates = [U([0], *a[0]), U([2], m[0]), CNOT([1, 0], n), U([1], *a[1]), U([3], m[1]), H(2), CNOT([3, 2], n)]
    return Circuit(gates, n=n, requires_decomp=requires_decomp)


def test_u_from_matrix_and_zsx_decomposition_match_the_reference():
    """Fixture from the reference (tests/golden/make_golden.py gen_sv_decomp): a U
    built from a matrix stores it without the phase of its top-left entry;
    Circuit.build() with requires_decomp replaces every U by the reference's
    RZ / SX sequence (gate for gate); the simulator's copy drops requires_decomp."""
    from conftest import golden
    from gateio import unpack_gates
    from oracle import ref
    z = golden("sv_decomp4.npz")
    plain = _decomp_circuit(z, False)
    for g, want in zip(plain.gate_list, unpack_gates(z, "u")):
        assert g.name == want.name and g.indices == list(want.indices)
        assert np.max(np.abs(np.asarray(g.matrix) - want.matrix)) < 1e-12
    built = _decomp_circuit(z, True).build()
    want = unpack_gates(z, "b")
    assert [(g.name, g.indices) for g in built.gate_list] == [(w.name, list(w.indices)) for w in want]
    for g, w in zip(built.gate_list, want):
        assert np.max(np.abs(np.asarray(g.matrix) - w.matrix)) < 1e-12
    n = int(z["n"])
    assert np.max(np.abs(ref.run_sv(want, n).reshape(-1) - z["sv_built"])) < 1e-12
    assert np.max(np.abs(ref.run_sv(unpack_gates(z, "u"), n).reshape(-1) - z["sv_plain"])) < 1e-12
    assert not _decomp_circuit(z, True).copy().requires_decomp


def test_cugate_and_embed_operator_match_the_reference():
    """Fixture from the reference (make_golden.py gen_gates_misc)."""
    from conftest import golden
    from qaravan_gb300.gates import CUGate, Gate, embed_operator
    z = golden("gates_misc.npz")
    for i in range(4):
        sub = z[f"cu{i}_sub"]
        g = CUGate(list(z[f"cu{i}_in"]), Gate("u", list(range(int(np.log2(sub.shape[0])))), sub))
        assert g.indices == list(z[f"cu{i}_idx"]) and g.bottom_heavy == bool(z[f"cu{i}_bottom"])
        assert np.max(np.abs(g.matrix - z[f"cu{i}_mat"])) < 1e-15
    assert np.max(np.abs(embed_operator(4, [1, 2], z["emb_block_op"]) - z["emb_block"])) < 1e-15
    ops = list(z["emb_ops"])
    assert np.max(np.abs(embed_operator(4, [0, 3], ops, dense=True) - z["emb_dense"])) < 1e-15
    assert np.max(np.abs(embed_operator(4, [0, 3], ops, dense=True, factor=True) - z["emb_dense_half"])) < 1e-15
    assert np.max(np.abs(embed_operator(4, [2, 1], ops).toarray() - z["emb_sparse"])) < 1e-15
    assert np.max(np.abs(embed_operator(3, [0, 1, 2], "xyz").toarray() - z["emb_pauli"])) < 1e-15


def test_superop_layers_skip_noise():
    from qaravan_gb300.circuits import Circuit
    from qaravan_gb300.gates import H, SuperOp
    from qaravan_gb300.noise import depolarizing
    m = np.kron(np.conj(H(0).matrix), H(0).matrix).reshape([2] * 4)
    c = Circuit([H(0), SuperOp("s", 1, m, start_idx=0), H(1)], n=3)
    c.construct_layers()  # [[H0, H1], [SuperOp on 0]]
    c.add_noise(depolarizing(0.01))
    assert [len(layer) for layer in c.layers] == [2 + 1, 1]  # the SuperOp's layer gets no noise carrier


def test_pretty_print_matches_the_reference():
    from conftest import golden
    from qaravan_gb300.core import pretty_print_dm, pretty_print_sv
    z = golden("pretty.npz")
    assert pretty_print_sv(z["sv"]) == str(z["sv_str"])
    assert pretty_print_dm(z["dm"]) == str(z["dm_str"])


def test_torch_angle_matrices_are_built_on_first_read():
    """A ParamGate with a torch angle builds its matrix when ``matrix`` is first
    read: bitwise the reference's eager ``matrix_exp`` value, with its autograd
    graph; building a circuit, layering it and copying it read no matrix."""
    th = torch.tensor([0.3, -1.1], dtype=torch.float64, requires_grad=True)
    Y = torch.tensor([[0, -1j], [1j, 0]], dtype=torch.complex128)
    g = RY(0, th[0])
    assert g.matrix_pending() and g.built_from_angles()
    c = Circuit([g, RZZ([0, 1], th[1])], n=2)
    c.construct_layers()
    cp = c.copy()
    assert all(h.matrix_pending() for h in c.gate_list + cp.gate_list)
    m = g.matrix
    assert torch.equal(m, torch.linalg.matrix_exp(-1.j * th[0] * Y)) and m.grad_fn is not None
    assert g.matrix is m and not g.matrix_pending() and g.built_from_angles()
    assert torch.equal(cp.gate_list[0].matrix, m)
    c.update_gate(1, np.eye(4))
    assert not c.gate_list[1].matrix_pending() and not c.gate_list[1].built_from_angles()
    assert not RZ(0, 0.3).matrix_pending()  # NumPy angles: built in the constructor, as before


def test_angle_changed_in_place_before_the_first_read():
    """The matrix has the angle's value at construction, as an eagerly built one
    would, and the gradient still reaches the angle."""
    th = torch.tensor([0.3, 0.5], dtype=torch.float64, requires_grad=True)
    g = RX(0, th[0])
    with torch.no_grad():
        th.add_(1.0)
    m = g.matrix
    X = torch.tensor([[0, 1], [1, 0]], dtype=torch.complex128)
    assert torch.equal(m.detach(), torch.linalg.matrix_exp(-1.j * torch.tensor(0.3, dtype=torch.float64) * X))
    m.real.sum().backward()  # 2 cos(theta)
    assert abs(th.grad[0].item() + 2 * np.sin(0.3)) < 1e-12 and th.grad[1].item() == 0


def test_closed_form_rotations_for_complex64_adjoint():
    """The complex64 adjoint takes cos(theta) I - i sin(theta) P for rotation
    gates not yet built, without building them; it agrees with matrix_exp to
    its series truncation."""
    from qaravan_gb300.adjoint import _matrices
    from qaravan_gb300.gates import CNOT
    rng = np.random.default_rng(3)
    th = torch.tensor(rng.uniform(0, 2 * np.pi, size=6), dtype=torch.float64, requires_grad=True)
    gates = [RX(0, th[0]), RY(1, th[1]), RZ(2, th[2]), RXX([0, 1], th[3]), RYY([1, 2], th[4]), RZZ([2, 0], th[5]),
             CNOT([0, 1], 3)]
    fast, _ = _matrices(gates, closed_form=True)
    assert all(g.matrix_pending() for g in gates[:6])
    slow, _ = _matrices(gates)
    for a, b in zip(fast, slow):
        assert a.shape == b.shape and torch.max(torch.abs(a - b.detach())).item() < 1e-9


def test_gradient_check_reads_no_pending_matrix():
    """The simulator decides whether a run needs the adjoint from the angles of
    gates whose matrix is not built yet, without building it."""
    from qaravan_gb300.gates import CNOT
    from qaravan_gb300.statevector import _gate_requires_grad
    th = torch.tensor([0.1, 0.2], dtype=torch.float64, requires_grad=True)
    gates = [RY(0, th[0]), RZ(1, th[1].detach()), CNOT([0, 1], 2)]
    assert [_gate_requires_grad(g) for g in gates] == [True, False, False]
    assert gates[0].matrix_pending() and gates[1].matrix_pending()


def test_stacked_angles_gather_from_one_parameter_tensor():
    """The adjoint's angle vector: one gather when every angle is an element view
    of the same tensor (also through a transposed view), a stack otherwise; the
    same values and the same gradient either way."""
    from qaravan_gb300.adjoint import _stack_angles
    th = torch.randn(5, 4, 2, dtype=torch.float64, requires_grad=True)
    views = [th[l, q, k] for l in range(5) for q in range(4) for k in range(2)][::-1]
    w = torch.randn(len(views), dtype=torch.float64)
    a = _stack_angles(views)
    assert a.grad_fn is not None and "IndexSelect" in type(a.grad_fn).__name__
    (a * w).sum().backward()
    g = th.grad.clone()
    th.grad = None
    b = torch.stack([v.reshape(()) for v in views])
    (b * w).sum().backward()
    assert torch.equal(a.detach(), b.detach()) and torch.equal(g, th.grad)
    tt = th.transpose(0, 2)
    assert torch.equal(_stack_angles([tt[1, 3, 4], tt[0, 2, 1]]).detach(), torch.stack([th[4, 3, 1], th[1, 2, 0]]).detach())
    other = torch.tensor([0.5, 0.25], dtype=torch.float64, requires_grad=True)
    mixed = _stack_angles([th[0, 0, 0], other[1], other * 2][:2])
    assert "Stack" in type(mixed.grad_fn).__name__ and mixed[1].item() == 0.25
