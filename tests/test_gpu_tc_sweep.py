"""The tensor-core tile sweep (several fused 5-qubit blocks per HBM pass,
qgb_apply_tc_sweep) through the C ABI: every tile geometry (runs of 16 to 8192
amplitudes, high bits anywhere), 1 to 4 blocks per pass, blocks on tile bit 0
(paired components) and the last block on flat bits 0 and 1 (staged stores),
unitary blocks with the norm chain and general (non-unitary) blocks, against a
complex128 application of the same blocks; and the compiled "tcsweep" mode of
StatevectorSim against the oracle and the reference's 12-qubit fixture
circuit (run on 14 qubits), and against complex128 on a 22-qubit depth-20
brickwork."""
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


def _rand_state(n, seed):
    g = torch.Generator().manual_seed(seed)
    v = torch.complex(torch.randn(2 ** n, generator=g, dtype=torch.float64),
                      torch.randn(2 ** n, generator=g, dtype=torch.float64))
    return v / torch.linalg.vector_norm(v)


def _rand_op(seed, unitary=True):
    rng = np.random.default_rng(seed)
    z = (rng.normal(size=(32, 32)) + 1j * rng.normal(size=(32, 32))) / np.sqrt(2)
    if not unitary:
        return z / 8.0
    q, r = np.linalg.qr(z)
    return q * (np.diag(r) / np.abs(np.diag(r)))


def _sweep_struct(low, high, blocks, offs):
    from qaravan_gb300 import _lib
    ts = _lib.TcSweep()
    ts.low_bits = low
    for i, b in enumerate(high):
        ts.high_bits[i] = b
    ts.n_blocks = len(blocks)
    for i, pos in enumerate(blocks):
        for j, p in enumerate(pos):
            ts.block_pos[i][j] = p
        ts.block_mat[i] = offs[i]
    return ts


def _run(n, low, high, blocks, mats, v0, chain=None, link=0):
    """Applies the sweep to v0 (complex64 on the GPU); returns the result and the
    complex128 expectation (each block through the oracle's op_action)."""
    import ctypes as C
    from qaravan_gb300 import _lib
    L = _lib.lib()
    tile = list(range(low)) + list(high)
    flat = np.concatenate([m.reshape(-1) for m in mats])
    dev_m = torch.as_tensor(flat).to(torch.complex64).cuda()
    offs = [32 * 32 * i for i in range(len(mats))]
    ts = _sweep_struct(low, high, blocks, offs)
    sv = v0.to(torch.complex64).cuda().contiguous()
    _lib.check(L.qgb_apply_tc_sweep(sv.data_ptr(), _lib.QGB_C64, n, C.byref(ts), dev_m.data_ptr(),
                                    chain.data_ptr() if chain is not None else None, link, _lib.stream_ptr()),
               "apply_tc_sweep")
    _lib.check(L.qgb_check_status(_lib.stream_ptr()), "status")
    exp = v0.numpy().reshape([2] * n)
    for pos, m in zip(blocks, mats):
        exp = ref.op_action(m, [n - 1 - tile[p] for p in pos], exp)
    return sv.cpu().numpy(), exp.reshape(-1)


# (n, low bits, high bits, blocks as tile positions in matrix order)
GEOMS = [
    (14, 13, [], [[0, 1, 2, 3, 4]]),
    (14, 4, [5, 6, 7, 8, 9, 10, 11, 12, 13], [[4, 5, 6, 7, 8], [0, 9, 10, 11, 12]]),
    (16, 5, [6, 7, 9, 10, 11, 12, 13, 15], [[12, 11, 10, 9, 8], [3, 8, 0, 5, 12], [1, 0, 7, 2, 6]]),
    (18, 8, [9, 12, 14, 16, 17], [[8, 9, 10, 11, 12], [2, 4, 6, 9, 11], [12, 0, 1, 5, 3], [7, 6, 10, 4, 8]]),
    (20, 4, [5, 7, 9, 11, 13, 15, 17, 18, 19], [[0, 1, 4, 9, 12], [6, 7, 8, 10, 11], [2, 3, 5, 12, 0]]),
    (20, 6, [8, 10, 12, 14, 16, 18, 19], [[12, 6, 7, 11, 2], [0, 1, 2, 3, 4]]),  # last block on flat bits 0, 1
    (22, 4, [6, 8, 10, 12, 14, 16, 18, 20, 21], [[9, 10, 11, 12, 4]]),
]


@pytest.mark.parametrize("n,low,high,blocks", GEOMS)
def test_tc_sweep_matches_complex128(n, low, high, blocks):
    mats = [_rand_op(97 * n + 13 * i + low) for i in range(len(blocks))]
    v0 = _rand_state(n, 5 * n + low)
    got, exp = _run(n, low, high, blocks, mats, v0)
    scale = np.max(np.abs(exp))
    # each block an fp32 dot product of length 32 (a few units of 2^-24), four blocks in a row
    assert np.max(np.abs(got - exp)) / scale < 4e-6


def test_tc_sweep_non_unitary_blocks():
    n = 17
    low, high = 5, [6, 7, 8, 10, 12, 13, 14, 16]
    blocks = [[0, 2, 4, 6, 8], [12, 11, 1, 3, 5], [7, 9, 10, 0, 1]]
    mats = [_rand_op(300 + i, unitary=False) for i in range(3)]
    v0 = _rand_state(n, 77)
    got, exp = _run(n, low, high, blocks, mats, v0)
    assert np.max(np.abs(got - exp)) / np.max(np.abs(exp)) < 4e-6


def test_tc_sweep_norm_chain_holds_the_norm():
    """50 unitary passes as one norm chain: the norm stays within one epoch's
    drift of its start (0.7 here), where the passes without the chain drift."""
    from qaravan_gb300 import _lib
    import ctypes as C
    n = 18
    L = _lib.lib()
    low, high = 4, [5, 6, 8, 9, 11, 12, 14, 15, 17]
    blocks = [[0, 1, 2, 3, 4], [5, 6, 7, 8, 9], [12, 11, 10, 2, 0]]
    mats = [_rand_op(900 + i) for i in range(3)]
    flat = np.concatenate([m.reshape(-1) for m in mats])
    dev_m = torch.as_tensor(flat).to(torch.complex64).cuda()
    ts = _sweep_struct(low, high, blocks, [0, 1024, 2048])
    norms = {}
    for use_chain in (True, False):
        sv = (_rand_state(n, 3) * 0.7).to(torch.complex64).cuda()
        chain = torch.zeros(6, dtype=torch.float64, device="cuda")
        for link in range(50):
            _lib.check(L.qgb_apply_tc_sweep(sv.data_ptr(), _lib.QGB_C64, n, C.byref(ts), dev_m.data_ptr(),
                                            chain.data_ptr() if use_chain else None, link if use_chain else 0,
                                            _lib.stream_ptr()), "apply_tc_sweep")
        _lib.check(L.qgb_check_status(_lib.stream_ptr()), "status")
        norms[use_chain] = float(torch.linalg.vector_norm(sv.to(torch.complex128)).item())
    assert abs(norms[True] - 0.7) < 1e-6
    assert abs(norms[True] - 0.7) < abs(norms[False] - 0.7)


def test_tc_sweep_rejects_bad_arguments():
    import ctypes as C
    from qaravan_gb300 import _lib
    L = _lib.lib()
    sv = torch.zeros(2 ** 14, dtype=torch.complex64, device="cuda")
    m = torch.zeros(1024, dtype=torch.complex64, device="cuda")
    good = (4, [5, 6, 7, 8, 9, 10, 11, 12, 13], [[0, 1, 2, 3, 4]])
    bad = [
        (3, [4, 5, 6, 7, 8, 9, 10, 11, 12], [[0, 1, 2, 3, 4]]),           # low bits < 4
        (4, [5, 6, 7, 8, 9, 10, 11, 13, 12], [[0, 1, 2, 3, 4]]),          # high bits not ascending
        (4, [5, 6, 7, 8, 9, 10, 11, 12, 14], [[0, 1, 2, 3, 4]]),          # high bit >= n
        (4, [5, 6, 7, 8, 9, 10, 11, 12, 13], [[0, 1, 2, 3, 3]]),          # repeated tile bit
        (4, [5, 6, 7, 8, 9, 10, 11, 12, 13], [[0, 1, 2, 3, 13]]),         # tile bit out of range
    ]
    for low, high, blocks in bad:
        ts = _sweep_struct(low, high, blocks, [0])
        assert L.qgb_apply_tc_sweep(sv.data_ptr(), _lib.QGB_C64, 14, C.byref(ts), m.data_ptr(), None, 0,
                                    _lib.stream_ptr()) == _lib.QGB_EINVAL
    ts = _sweep_struct(*good, [0])
    ts.n_blocks = 5
    assert L.qgb_apply_tc_sweep(sv.data_ptr(), _lib.QGB_C64, 14, C.byref(ts), m.data_ptr(), None, 0,
                                _lib.stream_ptr()) == _lib.QGB_EINVAL
    ts = _sweep_struct(*good, [0])
    assert L.qgb_apply_tc_sweep(sv.data_ptr(), _lib.QGB_C64, 13, C.byref(ts), m.data_ptr(), None, 0,
                                _lib.stream_ptr()) == _lib.QGB_EINVAL  # fewer than 14 qubits
    assert L.qgb_apply_tc_sweep(sv.data_ptr(), _lib.QGB_C128, 14, C.byref(ts), m.data_ptr(), None, 0,
                                _lib.stream_ptr()) == _lib.QGB_EINVAL  # complex64 only
    _lib.check(L.qgb_check_status(_lib.stream_ptr()), "status")


@pytest.mark.parametrize("n,depth,seed", [(14, 6, 1), (16, 8, 2), (19, 5, 3)])
def test_tcsweep_mode_matches_oracle(n, depth, seed):
    from qaravan_gb300 import StatevectorSim, workloads
    from qaravan_gb300.circuits import Circuit
    gates = workloads.brickwork_gates(n, depth, seed)
    exp = ref.run_sv(gates, n).reshape(-1)
    sim = StatevectorSim(Circuit(gates, n=n), dtype=torch.complex64, mode="tcsweep")
    got = sim.get_statevector().reshape(-1).cpu().numpy()
    assert sim.compile().plan.n_sweeps >= 1
    assert np.max(np.abs(got - exp)) < 1e-5


def test_tcsweep_mode_reference_fixture_circuit():
    """The reference's 12-qubit depth-20 brickwork gates on sites 0..11 of a
    14-qubit state: the first 12 sites' amplitudes (sites 12, 13 in |0>) equal
    the fixture's statevector."""
    from qaravan_gb300 import StatevectorSim
    from qaravan_gb300.circuits import Circuit
    from gateio import unpack_gates
    z = golden("sv_brickwork12.npz")
    gates = unpack_gates(z)
    sim = StatevectorSim(Circuit(gates, n=14), dtype=torch.complex64, mode="tcsweep")
    got = sim.get_statevector().reshape(2 ** 12, 4)[:, 0].cpu().numpy()
    assert np.max(np.abs(got - z["sv"].reshape(-1))) < 1e-5


def test_tcsweep_mode_22_qubits_depth_20_against_complex128():
    from qaravan_gb300 import StatevectorSim, workloads
    from qaravan_gb300.circuits import Circuit
    n = 22
    gates = workloads.brickwork_gates(n, 20, 22)
    c = Circuit(gates, n=n)
    a = StatevectorSim(c, dtype=torch.complex64, mode="tcsweep").get_statevector().reshape(-1)
    b = StatevectorSim(c, dtype=torch.complex128).get_statevector().reshape(-1)
    d = (a.to(torch.complex128) - b).abs()
    assert float(d.max()) < 1e-6
    assert abs(float(torch.linalg.vector_norm(a.to(torch.complex128))) - 1.0) < 1e-6
