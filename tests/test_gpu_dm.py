"""GPU parity: density-matrix path (vec(rho) kernels) vs reference fixtures."""
import numpy as np
import pytest
import torch

from conftest import golden
from gateio import unpack_gates
from oracle import ref

pytestmark = pytest.mark.gpu
TOL = {torch.complex64: 1e-5, torch.complex128: 1e-12}
DTYPES = [torch.complex64, torch.complex128]


@pytest.fixture(scope="module", autouse=True)
def built(cuda_ok):
    from qaravan_gb300 import build
    build.build()


@pytest.mark.parametrize("dtype", DTYPES)
def test_superop_capi_replay(dtype):
    """qgb_dm_apply_superop with the reference's own superoperators (incl. unsorted sites)."""
    from qaravan_gb300 import _lib
    z = golden("dm_mixed5.npz")
    n = int(z["n"])
    rho = torch.zeros(4 ** n, dtype=dtype, device="cuda")
    rho[0] = 1
    offs = z["superop_offs"]
    keep = []
    for i, k in enumerate(z["nlocs"]):
        s = torch.as_tensor(z["superops"][offs[i]:offs[i + 1]]).to(dtype).cuda()
        keep.append(s)
        locs = [int(x) for x in z["locs"][i][:k]]
        _lib.check(_lib.lib().qgb_dm_apply_superop(rho.data_ptr(), _lib.dtype_code(dtype), n, _lib.int_array(locs),
                                                   int(k), s.data_ptr(), 1, 0, _lib.stream_ptr()))
    dm = rho.reshape(2 ** n, 2 ** n).cpu().numpy()
    assert np.max(np.abs(dm - z["dm"])) < TOL[dtype]


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("mode,width,tile", [("gate", 2, 13), ("fused", 4, 13), ("sweep", 4, 8), ("sweep", 2, 10)])
def test_dm_sim_mixed5(dtype, mode, width, tile):
    from qaravan_gb300 import DensityMatrixSim
    from qaravan_gb300.circuits import Circuit
    z = golden("dm_mixed5.npz")
    n = int(z["n"])
    gates = unpack_gates(z)
    offs = z["superop_offs"]

    class _NM:
        def __init__(self, s):
            self.s = s

        def get_superop(self, *a):
            return self.s
    for i, g in enumerate(gates):
        if z["is_noise"][i]:
            g.name, g.nm, g.time, g.dd = "ID", _NM(z["superops"][offs[i]:offs[i + 1]]), 0.0, False
    circ = Circuit(gates, n=n)
    circ.layers = [[g] for g in gates]  # the fixture's exact op order
    circ.built = True
    sim = DensityMatrixSim(circ, dtype=dtype, mode=mode, fusion_width=width, tile_bits=tile)
    sim.run()
    dm = sim.get_density_matrix().cpu().numpy()
    assert np.max(np.abs(dm - z["dm"])) < TOL[dtype]
    lops = list(z["local_ops"])
    t = 10 * TOL[dtype]
    assert abs(sim.local_expectation(lops) - float(z["local"])) < t
    for q in range(n):
        assert abs(sim.one_local_expectation(lops[q], q) - z["one_local"][q]) < t
    assert abs(sim.global_expectation(z["global_op"]) - float(z["global_exp"])) < t
    assert abs(sim.purity() - float(z["purity"])) < t


@pytest.mark.parametrize("dtype", DTYPES)
def test_dm_kats(dtype):
    from qaravan_gb300 import DensityMatrixSim, StatevectorSim
    from qaravan_gb300.circuits import Circuit
    from qaravan_gb300.gates import CNOT, H
    from qaravan_gb300.noise import PauliNoise, QubitNoise
    from qaravan_gb300.paulis import pauli_X, pauli_Z
    z = golden("dm_kats.npz")
    t = 10 * TOL[dtype]
    circ = Circuit([H(0), CNOT([1, 0], 3), CNOT([2, 1], 3)], 3)
    sim = DensityMatrixSim(circ, nm=QubitNoise(1000, 1000, 1, 5), dtype=dtype)
    assert abs(sim.local_expectation([pauli_Z] * 3) - 0.020609303627304454) < t
    assert abs(sim.local_expectation([pauli_X] * 3) - 0.9369488105936169) < t
    assert np.max(np.abs(sim.get_density_matrix().cpu().numpy() - z["thermal_dm"])) < t
    sim = DensityMatrixSim(circ, nm=PauliNoise(['iii', 'xxx', 'yyy', 'zyz'], [0.9, 0.05, 0.02, 0.03]), dtype=dtype)
    assert abs(sim.local_expectation([pauli_Z] * 3)) < t
    assert abs(sim.local_expectation([pauli_X] * 3) - 0.81) < t
    assert abs(sim.trace() - 1.0) < t
    sv = StatevectorSim(circ, dtype=dtype)
    assert np.max(np.abs(sv.get_statevector().cpu().numpy() - z["ghz_sv"])) < TOL[dtype]
    assert abs(sv.local_expectation([pauli_X] * 3) - 1.0) < t


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("mode,width,tile", [("sweep", 4, 12), ("auto", None, 13)])
def test_dm_noisy_tfi_10q(dtype, mode, width, tile):
    """Per-gate depolarising + amplitude damping on the 10-qubit TFI Trotter
    circuit, as vec(rho) on 20 bits, against the reference DM run; "auto" is the
    default path (6-qubit fused blocks on the tensor cores for complex64)."""
    from qaravan_gb300 import DensityMatrixSim
    from qaravan_gb300.circuits import Circuit
    from qaravan_gb300.gates import ID
    from qaravan_gb300.noise import amplitude_damping, depolarizing
    z = golden("traj_dm10_strong.npz")
    n = int(z["n"])
    dep, ad = depolarizing(float(z["p"])), amplitude_damping(float(z["gamma"]))
    seq = []
    for g in unpack_gates(z):
        seq.append(g)
        for q in g.indices:
            seq.append(ID(2, 0.0, [q], nm=dep))
            seq.append(ID(2, 0.0, [q], nm=ad))
    circ = Circuit([g for g in seq if g.name != "ID"], n=n)
    circ.layers = [[g] for g in seq]
    circ.built = True
    sim = DensityMatrixSim(circ, dtype=dtype, mode=mode, fusion_width=width, tile_bits=tile)
    sim.run()
    zs = sim.pauli_expectations([(1.0, 'i' * q + 'z' + 'i' * (n - q - 1)) for q in range(n)]).cpu().numpy()
    assert np.max(np.abs(zs - z["z"])) < 10 * TOL[dtype]
    zz = sim.pauli_expectations([(1.0, 'i' * q + 'zz' + 'i' * (n - q - 2)) for q in range(n - 1)]).cpu().numpy()
    assert np.max(np.abs(zz - z["zz"])) < 10 * TOL[dtype]
    assert abs(sim.purity() - float(z["purity"])) < 10 * TOL[dtype]


@pytest.mark.parametrize("dtype", DTYPES)
def test_superop_applies_its_matrix(dtype):
    """A SuperOp holding a gate's to_superop() acts like the gate
    (tensorQ/density_matrix_sim.py:38-42 applies SuperOp.matrix as is); its
    layer gets no noise carrier (core/circuits.py:64-84)."""
    from qaravan_gb300 import DensityMatrixSim, workloads
    from qaravan_gb300.circuits import Circuit
    from qaravan_gb300.gates import CNOT, Gate, H, SuperOp
    rng = np.random.default_rng(21)
    n = 4
    u = workloads.haar_unitary(4, rng)
    g = Gate("u", [1, 2], u)
    with_gate = Circuit([H(0), CNOT([1, 0], n), g, H(3), CNOT([3, 2], n)], n=n)
    with_sop = Circuit([H(0), CNOT([1, 0], n), SuperOp("u", 2, g.to_superop(), start_idx=1), H(3),
                        CNOT([3, 2], n)], n=n)
    a = DensityMatrixSim(with_gate, dtype=dtype).get_density_matrix()
    b = DensityMatrixSim(with_sop, dtype=dtype).get_density_matrix()
    a = a.cpu().numpy() if torch.is_tensor(a) else np.asarray(a)
    b = b.cpu().numpy() if torch.is_tensor(b) else np.asarray(b)
    tol = 1e-5 if dtype == torch.complex64 else 1e-12
    assert np.max(np.abs(a - b)) < tol


@pytest.mark.parametrize("dtype", DTYPES)
def test_wide_pauli_channel_matches_oracle_superoperator(dtype):
    """Circuit-level Pauli noise on all 5 sites (a 10-bit superoperator, wider
    than a dense block) runs as a Pauli mixture on vec(rho); against the
    oracle's superoperator of the reference's Kraus operators, a negative
    (quasi-probability) weight included."""
    from qaravan_gb300 import DensityMatrixSim, workloads
    from qaravan_gb300.circuits import Circuit
    from qaravan_gb300.noise import PauliNoise
    n = 5
    gates = workloads.brickwork_gates(n, 2, 41)
    nm = PauliNoise(["iiiii", "xiiyi", "izizi", "yyiix", "iiiiz"], [0.93, 0.03, 0.05, 0.01, -0.02])
    sim = DensityMatrixSim(Circuit(gates, n=n), nm=nm, dtype=dtype)
    rho = sim.get_density_matrix().cpu().numpy()
    c = Circuit(gates, n=n)
    c.build(nm)
    want = ref.run_dm([g for layer in c.layers for g in layer], n, layered=False)
    tol = 1e-5 if dtype == torch.complex64 else 1e-12
    assert np.max(np.abs(rho - want)) < tol
