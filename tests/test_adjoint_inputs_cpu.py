"""Host side of the single-set adjoint on the CPU: the gate matrices handed to
the forward pass (``adjoint._matrices``) -- every gate's matrix and the same
matrices flattened into one complex128 buffer -- in closed form
(cos theta I - i sin theta P from the angles) against torch's matrix_exp of
the reference's ParamGate, with the angles gathered from one parameter tensor
or, after an in-place change of that tensor, taken at their construction-time
values (the values the reference's constructor used)."""
import numpy as np
import torch

from qaravan_gb300 import workloads


def _circuit(n, layers, th):
    from qaravan_gb300.gates import RXX, RZZ
    c = workloads.hea_circuit(n, layers, th)
    return list(c.gate_list) + [RXX([0, 3], th[0][1][0]), RZZ([2, 1], th[1][2][1])]


def test_flat_buffer_is_the_gate_matrices_in_order():
    from qaravan_gb300.adjoint import _matrices
    th = torch.tensor(workloads.hea_params(6, 2, 1), dtype=torch.float64, requires_grad=True)
    gates = _circuit(6, 2, th)
    for closed in (True, False):
        mats, flat = _matrices(gates, closed)
        assert len(mats) == len(gates)
        cat = np.concatenate([m.detach().reshape(-1).numpy() for m in mats])
        assert np.array_equal(cat, flat)


def test_closed_form_matches_matrix_exp():
    from qaravan_gb300.adjoint import _matrices
    th = torch.tensor(workloads.hea_params(6, 2, 3), dtype=torch.float64, requires_grad=True)
    _, closed = _matrices(_circuit(6, 2, th), True)
    _, expm = _matrices(_circuit(6, 2, th), False)  # reads every ParamGate's matrix (matrix_exp)
    assert np.max(np.abs(closed - expm)) < 1e-9


def test_angles_changed_in_place_use_construction_values():
    from qaravan_gb300.adjoint import _matrices
    vals = workloads.hea_params(6, 2, 5)
    th = torch.tensor(vals, dtype=torch.float64, requires_grad=True)
    gates = _circuit(6, 2, th)
    with torch.no_grad():
        th += 0.25
    _, changed = _matrices(gates, True)
    _, original = _matrices(_circuit(6, 2, torch.tensor(vals, dtype=torch.float64)), True)
    assert np.array_equal(changed, original)
