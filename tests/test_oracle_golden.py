"""Pin the CPU oracle (oracle/ref.py) to fixtures produced by the real reference."""
import numpy as np

from conftest import golden
from gateio import unpack_gates
from oracle import ref


def test_brickwork12_statevector():
    z = golden("sv_brickwork12.npz")
    gates = unpack_gates(z)
    assert len(gates) == 460
    sv = ref.run_sv(gates, int(z["n"]))
    assert np.max(np.abs(sv - z["sv"])) < 1e-12


def test_brickwork12_observables():
    z = golden("sv_brickwork12.npz")
    sv = z["sv"]
    ops = list(z["local_ops"])
    assert abs(ref.local_expectation(sv, ops) - float(z["local"])) < 1e-12
    for q in range(int(z["n"])):
        assert abs(ref.one_local_expectation(sv, ops[q], q) - z["one_local"][q]) < 1e-12
    for s, e in zip(z["tfi_strings"], z["tfi_exp"]):
        assert abs(ref.pauli_expectation_sv(sv, str(s)) - e) < 1e-12


def test_mixed7_statevector():
    z = golden("sv_mixed7.npz")
    gates = unpack_gates(z)
    sv = ref.run_sv(gates, int(z["n"]), init_state=str(z["init"]))
    assert np.max(np.abs(sv - z["sv"])) < 1e-12


def test_observables8():
    z = golden("sv_observables8.npz")
    sv, sv2 = z["sv"], z["sv2"]
    for s, e in zip(z["strings"], z["pexp"]):
        assert abs(ref.pauli_expectation_sv(sv, str(s)) - e) < 1e-12
    for i, row in enumerate(z["po_sites"]):
        sites = [int(x) for x in row if x >= 0]
        assert np.max(np.abs(ref.partial_overlap(sv, sv2, skip=sites) - z[f"po{i}"])) < 1e-12
        assert np.max(np.abs(ref.partial_overlap(sv, sv, skip=sites) - z[f"rdm{i}"])) < 1e-12


def test_dm_mixed5():
    z = golden("dm_mixed5.npz")
    n = int(z["n"])
    rho = ref.initial_dm(n)
    offs = z["superop_offs"]
    for i, k in enumerate(z["nlocs"]):
        s = z["superops"][offs[i]:offs[i + 1]]
        rho = ref.dm_apply_superop(rho, s, [int(x) for x in z["locs"][i][:k]], n)
    dm = rho.reshape(2 ** n, 2 ** n)
    assert np.max(np.abs(dm - z["dm"])) < 1e-12
    lops = list(z["local_ops"])
    assert abs(ref.dm_local_expectation(dm, lops) - float(z["local"])) < 1e-12
    for q in range(n):
        assert abs(ref.dm_one_local_expectation(dm, lops[q], q) - z["one_local"][q]) < 1e-12
    assert abs(ref.dm_global_expectation(dm, z["global_op"]) - float(z["global_exp"])) < 1e-12
    assert abs(ref.purity(dm) - float(z["purity"])) < 1e-12


def test_dm_mixed5_superops_match_channels():
    """Unitary superops equal kron(conj M, M); noise superops equal sum kron(conj K, K)."""
    z = golden("dm_mixed5.npz")
    gates = unpack_gates(z)
    offs = z["superop_offs"]
    for i, g in enumerate(gates):
        s = z["superops"][offs[i]:offs[i + 1]].reshape(4 ** g.span, 4 ** g.span)
        if not z["is_noise"][i]:
            assert np.max(np.abs(s - ref.to_superop(g.matrix))) < 1e-15


def test_dm_kats():
    z = golden("dm_kats.npz")
    assert abs(float(z["thermal_zzz"]) - 0.020609303627304454) < 1e-12  # .dev notebook cell 5
    assert abs(float(z["thermal_xxx"]) - 0.9369488105936169) < 1e-12   # cell 6
    assert abs(float(z["pauli_zzz"])) < 1e-12                           # cell 10
    assert abs(float(z["pauli_xxx"]) - 0.81) < 1e-12                    # cell 11
    assert abs(ref.dm_local_expectation(z["thermal_dm"], [ref.PAULI['z']] * 3) - float(z["thermal_zzz"])) < 1e-12
    assert abs(ref.dm_local_expectation(z["pauli_dm"], [ref.PAULI['x']] * 3) - float(z["pauli_xxx"])) < 1e-12
    ghz = np.zeros(8, complex)
    ghz[0] = ghz[7] = 1 / np.sqrt(2)
    assert np.max(np.abs(z["ghz_sv"] - ghz)) < 1e-7


def test_traj_dm10_oracle():
    """The oracle's per-gate-noise DM recipe reproduces the reference's DM run."""
    from qaravan_gb300.noise import depolarizing, amplitude_damping
    z = golden("traj_dm10_strong.npz")
    n = int(z["n"])
    gates = unpack_gates(z)
    chans = [depolarizing(float(z["p"])).get_kraus(), amplitude_damping(float(z["gamma"])).get_kraus()]
    rho = ref.initial_dm(n)
    for g in gates:
        rho = ref.dm_apply_gate_then_channels(rho, n, g, chans)
    dm = rho.reshape(2 ** n, 2 ** n)
    for q in range(n):
        assert abs(ref.dm_pauli_expectation(dm, 'i' * q + 'z' + 'i' * (n - q - 1)) - z["z"][q]) < 1e-12


def test_matrix_gradients_match_reference_autograd():
    """The oracle's reverse-sweep gradient, chained to the angles, matches the
    reference torch-backend autograd gradient (complex64 there)."""
    from qaravan_gb300 import workloads
    from qaravan_gb300.hamiltonians import TFI
    import torch
    z = golden("grad_hea6.npz")
    n, layers, params = int(z["n"]), int(z["layers"]), z["params"]
    th = torch.tensor(params, dtype=torch.float64, requires_grad=True)
    circ = workloads.hea_circuit(n, layers, th)
    terms = TFI(n, 1, 1).pauli_sum()
    grads = ref.matrix_gradients(circ.gate_list, n, terms)
    mats = [g.matrix for g in circ.gate_list]
    surrogate = 0
    for m, gm in zip(mats, grads):
        if torch.is_tensor(m) and m.requires_grad:
            # torch's grad for a real loss L is 2 dL/d conj(M) = gm, so
            # dL = Re sum conj(gm) * dM
            surrogate = surrogate + torch.real(torch.sum(torch.tensor(gm).conj() * m))
    surrogate.backward()
    g = th.grad.numpy()
    assert np.max(np.abs(g - z["grad"])) < 1e-4 * max(1.0, np.max(np.abs(z["grad"])))
    e = ref.energy(circ.gate_list, n, terms)
    assert abs(e - float(z["energy"])) < 1e-5


def test_matrix_gradients_central_differences():
    from qaravan_gb300 import workloads
    from qaravan_gb300.hamiltonians import TFI
    n, layers = 4, 2
    params = workloads.hea_params(n, layers, 3)
    terms = TFI(n, 1, 1).pauli_sum()

    def E(p):
        return ref.energy(workloads.hea_circuit(n, layers, p).gate_list, n, terms)

    import torch
    th = torch.tensor(params, dtype=torch.float64, requires_grad=True)
    circ = workloads.hea_circuit(n, layers, th)
    grads = ref.matrix_gradients(circ.gate_list, n, terms)
    s = 0
    for g, gm in zip(circ.gate_list, grads):
        if torch.is_tensor(g.matrix):
            s = s + torch.real(torch.sum(torch.tensor(gm).conj() * g.matrix))
    s.backward()
    eps = 1e-5
    for idx in [(0, 0, 0), (0, 1, 1), (1, 3, 0), (1, 2, 1)]:
        pp, pm = params.copy(), params.copy()
        pp[idx] += eps
        pm[idx] -= eps
        fd = (E(pp) - E(pm)) / (2 * eps)
        assert abs(fd - th.grad.numpy()[idx]) < 1e-8
