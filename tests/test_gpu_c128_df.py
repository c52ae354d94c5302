"""complex128 tile sweeps in double-float arithmetic (the default) against the
float64 sweep kernel, the oracle and the reference's own fixture, through the
C ABI: the same 1e-12 amplitude bar as every complex128 path, on every op
width (1-4), several tile splits, batches of states, states with
zero and tiny components, and a 22-qubit depth-20 brickwork."""
import numpy as np
import pytest
import torch

from conftest import golden
from oracle import ref

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built(cuda_ok):
    from qaravan_gb300 import _lib, build
    build.build()
    L = _lib.lib()
    before = L.qgb_get_c128_arith()
    yield
    _lib.check(L.qgb_set_c128_arith(before), "set_c128_arith")


def _sweep(n, gates, width, tile, low, arith, init, batch=1):
    from qaravan_gb300 import _lib, compiler
    from qaravan_gb300.engine import Executor
    from qaravan_gb300.statevector import gates_to_ops
    L = _lib.lib()
    _lib.check(L.qgb_set_c128_arith(arith), "set_c128_arith")
    plan = compiler.compile_ops(gates_to_ops(gates, n), n, mode="sweep", width=width, tile_bits=tile, low_bits=low,
                                max_sweep_k=4, itemsize=16)
    ex = Executor(plan, torch.complex128, "cuda")
    st = torch.as_tensor(init).to(torch.complex128).cuda().contiguous()
    ex.run(st, batch=batch, stride=2 ** n if batch > 1 else 0)
    _lib.check(L.qgb_check_status(None), "status")
    return st.cpu().numpy(), plan


def test_default_is_double_float():
    from qaravan_gb300 import _lib
    assert _lib.lib().qgb_get_c128_arith() == 1
    assert _lib.lib().qgb_set_c128_arith(2) != 0  # unknown mode rejected


def test_reference_fixture_12_qubits():
    from qaravan_gb300 import StatevectorSim
    from qaravan_gb300.circuits import Circuit
    from qaravan_gb300 import _lib
    from gateio import unpack_gates
    g = golden("sv_brickwork12.npz")
    gates = unpack_gates(g)
    _lib.check(_lib.lib().qgb_set_c128_arith(1), "set_c128_arith")
    sim = StatevectorSim(Circuit(gates, n=12), dtype=torch.complex128, mode="sweep", fusion_width=3, tile_bits=10)
    got = sim.get_statevector().cpu().numpy().reshape(-1)
    assert np.max(np.abs(got - g["sv"].reshape(-1))) < 1e-12


GEOMS = [(14, 1, 10, 4), (14, 2, 12, 5), (14, 3, 9, 3), (16, 4, 13, 6), (16, 3, 12, None), (18, 2, 13, 4),
         (18, 4, 12, 7), (12, 3, 12, None)]


@pytest.mark.parametrize("n,width,tile,low", GEOMS)
def test_double_float_matches_float64_and_oracle(n, width, tile, low):
    from qaravan_gb300 import workloads
    gates = workloads.brickwork_gates(n, 4, 300 + n + width)
    exp = ref.run_sv(gates, n).reshape(-1)
    v0 = np.zeros(2 ** n, complex)
    v0[0] = 1
    a, plan = _sweep(n, gates, width, tile, low, 1, v0)
    b, _ = _sweep(n, gates, width, tile, low, 0, v0)
    assert plan.n_sweeps >= 1
    assert np.max(np.abs(a - exp)) < 1e-12
    assert np.max(np.abs(a - b)) < 1e-12


def test_random_state_every_width_relative():
    """A random normalised state through dense ops of widths 1-4 on scattered
    bits: double-float against float64 relative to the largest amplitude."""
    from qaravan_gb300 import workloads
    from qaravan_gb300.gates import Gate
    rng = np.random.default_rng(5)
    n = 17
    gates = []
    for i in range(24):
        k = 1 + i % 4
        sites = [int(s) for s in rng.choice(n, size=k, replace=False)]
        gates.append(Gate("U", sites, workloads.haar_unitary(2 ** k, rng)))
    v0 = rng.standard_normal(2 ** n) + 1j * rng.standard_normal(2 ** n)
    v0 /= np.linalg.norm(v0)
    exp = ref.run_sv(gates, n, init_state=v0).reshape(-1)
    a, _ = _sweep(n, gates, 4, 13, 5, 1, v0)
    b, _ = _sweep(n, gates, 4, 13, 5, 0, v0)
    scale = np.max(np.abs(exp))
    assert np.max(np.abs(a - exp)) / scale < 1e-12
    assert np.max(np.abs(a - b)) / scale < 1e-12
    assert abs(np.linalg.norm(a) - 1) < 1e-13


def test_zero_and_tiny_components():
    """Exact zeros stay zero; a component of 2e-20 keeps 48 significant bits; one
    of 1e-30 keeps its value to the double-float's absolute floor, 2^-126 (the
    low float of a pair cannot go below float's smallest normal number)."""
    from qaravan_gb300.gates import Gate
    n = 14
    v0 = np.zeros(2 ** n, complex)
    v0[0] = 1.0
    v0[1] = 1e-30j
    v0[3] = -2e-20
    x = np.array([[0, 1], [1, 0]], complex)
    gates = [Gate("X", [n - 3], x), Gate("X", [n - 3], x)]  # X twice on site n-3: the identity
    a, _ = _sweep(n, gates, 1, 12, 4, 1, v0)
    assert a[0] == 1.0
    assert np.count_nonzero(a) == 3
    assert abs(a[1] - 1e-30j) < 2.0 ** -125 and abs(a[3] + 2e-20) < 2e-20 * 2.0 ** -47


def test_batch_of_states():
    """Three random (unnormalised) states in one batched sweep launch."""
    from qaravan_gb300 import _lib, compiler, workloads
    from qaravan_gb300.engine import Executor
    from qaravan_gb300.statevector import gates_to_ops
    n, batch = 13, 3
    gates = workloads.brickwork_gates(n, 2, 77)
    ops = gates_to_ops(gates, n)
    plan = compiler.compile_ops(ops, n, mode="sweep", width=3, tile_bits=11, low_bits=4, max_sweep_k=4, itemsize=16,
                                device_fusion=False)
    rng = np.random.default_rng(9)
    states = rng.standard_normal((batch, 2 ** n)) + 1j * rng.standard_normal((batch, 2 ** n))
    outs = {}
    for arith in (1, 0):
        _lib.check(_lib.lib().qgb_set_c128_arith(arith), "set_c128_arith")
        ex = Executor(plan, torch.complex128, "cuda")
        st = torch.as_tensor(states).cuda().contiguous()
        ex.run(st, batch=batch, stride=2 ** n)
        _lib.check(_lib.lib().qgb_check_status(None), "status")
        outs[arith] = st.cpu().numpy()
    for b in range(batch):
        exp = ref.run_sv(gates, n, init_state=states[b]).reshape(-1)
        assert np.max(np.abs(outs[1][b] - exp)) / np.max(np.abs(exp)) < 1e-12
    assert np.max(np.abs(outs[1] - outs[0])) / np.max(np.abs(outs[0])) < 1e-12


def test_22_qubit_brickwork_depth_20():
    from qaravan_gb300 import StatevectorSim, _lib, workloads
    from qaravan_gb300.circuits import Circuit
    n = 22
    gates = workloads.brickwork_gates(n, 20, 2022)
    L = _lib.lib()
    res = {}
    for arith in (1, 0):
        _lib.check(L.qgb_set_c128_arith(arith), "set_c128_arith")
        sim = StatevectorSim(Circuit(gates, n=n), dtype=torch.complex128, mode="sweep", fusion_width=3, tile_bits=13)
        res[arith] = sim.get_statevector().reshape(-1).cpu().numpy()
    assert np.max(np.abs(res[1] - res[0])) < 1e-12
    assert abs(np.linalg.norm(res[1]) - 1) < 1e-12
