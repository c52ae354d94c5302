"""The tensor-core dense kernel (tcgen05, split-tf32 operands, fp32
accumulation) against the CUDA-core kernel and a complex128 application of the
same op, for 4-, 5- and 6-qubit blocks on every kind of target set: the lowest
bit (16-byte loads), only high bits, contiguous and scattered bits, output bits
permuted against input bits (density-matrix superoperators on unsorted sites),
and batched states. Also fused 4- to 6-qubit blocks against the 12-qubit
depth-20 brickwork fixture (run on 14 qubits, the kernel's smallest size) and
against the oracle at 16 qubits."""
import numpy as np
import pytest
import torch

from conftest import golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built(cuda_ok):
    from qaravan_gb300 import _lib, build
    build.build()
    before = _lib.lib().qgb_get_dense_impl()
    yield
    _lib.lib().qgb_set_dense_impl(before)


def _apply(sv, n, bits_in, bits_out, mat, impl, batch=1, stride=0):
    """Dense op through the C ABI's bit-level entry (qgb_op_action for equal
    bit lists, qgb_dm_apply_superop otherwise)."""
    from qaravan_gb300 import _lib
    L = _lib.lib()
    _lib.check(L.qgb_set_dense_impl(impl))
    k = len(bits_in)
    m = torch.as_tensor(mat).to(sv.dtype).cuda().contiguous()
    sites = [n - 1 - b for b in bits_in]
    _lib.check(L.qgb_op_action(sv.data_ptr(), _lib.dtype_code(sv.dtype), n, _lib.int_array(sites), k, m.data_ptr(),
                               0, batch, stride, _lib.stream_ptr()), "op_action")
    _lib.check(L.qgb_check_status(_lib.stream_ptr()), "status")
    return sv


def _rand_state(n, batch, seed):
    g = torch.Generator().manual_seed(seed)
    v = torch.complex(torch.randn(batch * 2 ** n, generator=g, dtype=torch.float64),
                      torch.randn(batch * 2 ** n, generator=g, dtype=torch.float64))
    return v / torch.linalg.vector_norm(v) * np.sqrt(batch)


def _rand_op(k, seed):
    rng = np.random.default_rng(seed)
    d = 2 ** k
    z = (rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))) / np.sqrt(2)
    q, r = np.linalg.qr(z)
    return q * (np.diag(r) / np.abs(np.diag(r)))


CASES = [
    (4, 13, [0, 1, 2, 3]), (4, 14, [0, 5, 9, 11]), (4, 16, [3, 7, 12, 15]), (4, 20, [19, 18, 0, 10]),
    (5, 13, [0, 1, 2, 3, 4]), (5, 16, [15, 0, 7, 3, 9]), (5, 18, [4, 5, 6, 7, 8]), (5, 20, [1, 6, 11, 16, 19]),
    (6, 13, [0, 1, 2, 3, 4, 5]), (6, 13, [7, 8, 9, 10, 11, 12]), (6, 16, [2, 0, 15, 9, 4, 11]),
    (6, 20, [19, 17, 13, 8, 5, 1]), (6, 22, [0, 3, 6, 9, 12, 21]),
]


@pytest.mark.parametrize("k,n,bits", CASES)
def test_tensor_core_dense_matches_cuda_cores_and_complex128(k, n, bits):
    u = _rand_op(k, 7 * n + k)
    v0 = _rand_state(n, 1, n + 31 * k)
    ref128 = _apply(v0.to(torch.complex128).cuda(), n, bits, bits, u, 0).cpu().numpy()
    cc = _apply(v0.to(torch.complex64).cuda(), n, bits, bits, u, 0).cpu().numpy()
    tc = _apply(v0.to(torch.complex64).cuda(), n, bits, bits, u, 2).cpu().numpy()
    scale = np.max(np.abs(ref128))
    # fp32 dot products of length 2^k: a few units of 2^-24 relative
    assert np.max(np.abs(tc - ref128)) / scale < 2e-6
    assert np.max(np.abs(tc - cc)) / scale < 2e-6


@pytest.mark.parametrize("k", [4, 5, 6])
def test_tensor_core_dense_batched_states(k):
    n, batch = 14, 3
    bits = list(range(0, 2 * k, 2))
    u = _rand_op(k, 99 + k)
    v0 = _rand_state(n, batch, 5 + k)
    ref128 = _apply(v0.to(torch.complex128).cuda(), n, bits, bits, u, 0, batch, 2 ** n).cpu().numpy()
    tc = _apply(v0.to(torch.complex64).cuda(), n, bits, bits, u, 2, batch, 2 ** n).cpu().numpy()
    assert np.max(np.abs(tc - ref128)) / np.max(np.abs(ref128)) < 2e-6


@pytest.mark.parametrize("sites", [[4, 1], [0, 5], [3, 2]])
def test_tensor_core_superoperator_with_permuted_output_bits(sites):
    """A 2-site superoperator acts on 4 bits of vec(rho); with unsorted sites
    its output legs follow ascending site order, so the output bit list is a
    permutation of the input list."""
    from qaravan_gb300 import _lib
    L = _lib.lib()
    n = 7  # 14 bits of vec(rho): two 8192-amplitude tiles
    rng = np.random.default_rng(sum(sites))
    sup = (rng.normal(size=(16, 16)) + 1j * rng.normal(size=(16, 16))) / 4
    rho = _rand_state(2 * n, 1, 3 + sites[0])
    outs = []
    for dtype, impl in ((torch.complex128, 0), (torch.complex64, 0), (torch.complex64, 2)):
        _lib.check(L.qgb_set_dense_impl(impl))
        r = rho.to(dtype).cuda().contiguous()
        m = torch.as_tensor(sup).to(dtype).cuda().contiguous()
        _lib.check(L.qgb_dm_apply_superop(r.data_ptr(), _lib.dtype_code(dtype), n, _lib.int_array(sites), 2,
                                          m.data_ptr(), 1, 0, _lib.stream_ptr()), "superop")
        _lib.check(L.qgb_check_status(_lib.stream_ptr()))
        outs.append(r.cpu().numpy())
    scale = np.max(np.abs(outs[0]))
    assert np.max(np.abs(outs[2] - outs[0])) / scale < 2e-6
    assert np.max(np.abs(outs[2] - outs[1])) / scale < 2e-6


@pytest.mark.parametrize("width", [4, 5, 6])
def test_fused_blocks_on_tensor_cores_match_brickwork_fixture(width):
    """The 12-qubit fixture circuit on 14 qubits (sites 12, 13 idle in |0>, the
    two lowest bits), so that the tensor-core kernel takes every block."""
    from gateio import unpack_gates
    from qaravan_gb300 import StatevectorSim, _lib
    from qaravan_gb300.circuits import Circuit
    _lib.check(_lib.lib().qgb_set_dense_impl(2))
    z = golden("sv_brickwork12.npz")
    n = int(z["n"])
    sim = StatevectorSim(Circuit(unpack_gates(z), n=n + 2), dtype=torch.complex64, mode="fused", fusion_width=width)
    sv = sim.get_statevector().cpu().numpy().reshape(2 ** n, 4)
    assert np.max(np.abs(sv[:, 0] - z["sv"])) < 1e-5
    assert np.max(np.abs(sv[:, 1:])) < 1e-6


@pytest.mark.parametrize("width", [4, 5, 6])
def test_fused_blocks_on_tensor_cores_match_oracle_16q(width):
    from oracle import ref
    from qaravan_gb300 import StatevectorSim, _lib, workloads
    from qaravan_gb300.circuits import Circuit
    _lib.check(_lib.lib().qgb_set_dense_impl(2))
    n = 16
    gates = workloads.brickwork_gates(n, 8, 4242)
    exp = ref.run_sv(gates, n)
    sim = StatevectorSim(Circuit(gates, n=n), dtype=torch.complex64, mode="fused", fusion_width=width)
    sv = sim.get_statevector().cpu().numpy()
    assert np.max(np.abs(sv - exp)) < 1e-5


def test_unitary_blocks_keep_the_norm_on_tensor_cores():
    """Fused unitary blocks go through qgb_op_action_unitary: the tensor-core
    kernel restores each group's norm, so 20 layers at 20 qubits keep the state
    norm to fp32 level (without it the tensor cores' round-toward-zero
    accumulation shrinks it by about 1e-7 per pass), and amplitudes stay within
    the complex64 bar of the complex128 result."""
    from qaravan_gb300 import StatevectorSim, _lib, workloads
    from qaravan_gb300.circuits import Circuit
    _lib.check(_lib.lib().qgb_set_dense_impl(2))
    n = 20
    circ = Circuit(workloads.brickwork_gates(n, 20, 31), n=n)
    v64 = StatevectorSim(circ, dtype=torch.complex64).get_statevector().to(torch.complex128).cpu().numpy()
    v128 = StatevectorSim(circ, dtype=torch.complex128).get_statevector().cpu().numpy()
    assert abs(np.linalg.norm(v64) - 1.0) < 1.5e-6
    assert np.max(np.abs(v64 - v128)) < 1e-6


@pytest.mark.parametrize("k,bits", [(6, [0, 1, 2, 3, 4, 5]), (6, [3, 8, 11, 14, 17, 19]), (5, [2, 7, 12, 16, 19]),
                                    (4, [0, 1, 9, 18])])
def test_unitary_entry_point_matches_and_preserves_group_norms(k, bits):
    from qaravan_gb300 import _lib
    L = _lib.lib()
    _lib.check(L.qgb_set_dense_impl(2))
    n = 20
    u = _rand_op(k, 11 + k)
    v0 = _rand_state(n, 1, 5 * k)
    ref128 = _apply(v0.to(torch.complex128).cuda(), n, bits, bits, u, 0).cpu().numpy()
    sv = v0.to(torch.complex64).cuda().contiguous()
    m = torch.as_tensor(u).to(torch.complex64).cuda().contiguous()
    sites = _lib.int_array([n - 1 - b for b in bits])
    for _ in range(50):  # 50 applications of U, then compare against 50 in complex128
        _lib.check(L.qgb_op_action_unitary(sv.data_ptr(), _lib.QGB_C64, n, sites, k, m.data_ptr(), 0, 1, 0,
                                           _lib.stream_ptr()))
    _lib.check(L.qgb_check_status(_lib.stream_ptr()))
    ref = v0.to(torch.complex128).cuda()
    mref = torch.as_tensor(u).to(torch.complex128).cuda().contiguous()
    for _ in range(50):
        _lib.check(L.qgb_op_action(ref.data_ptr(), _lib.QGB_C128, n, sites, k, mref.data_ptr(), 0, 1, 0,
                                   _lib.stream_ptr()))
    got, want = sv.to(torch.complex128).cpu().numpy(), ref.cpu().numpy()
    assert abs(np.linalg.norm(got) - 1.0) < 2e-6
    assert np.max(np.abs(got - want)) / np.max(np.abs(want)) < 2e-5
    assert ref128.shape == got.shape


@pytest.mark.parametrize("k,bits", [(6, [0, 1, 2, 3, 4, 5]), (6, [3, 8, 11, 14, 17, 19]), (5, [2, 7, 12, 16, 19]),
                                    (4, [0, 1, 9, 18])])
def test_norm_chain_holds_the_reference_norm(k, bits):
    """50 applications of a unitary as links 0..49 of one norm chain
    (qgb_op_action_unitary_chain), from a state of norm 0.7: the norm stays at
    0.7 to within a pass's shrinkage, amplitudes match complex128; halfway a
    3-qubit link (not a tensor-core block) clears the chain and the next link
    starts a new one from the state as it is."""
    from qaravan_gb300 import _lib
    L = _lib.lib()
    _lib.check(L.qgb_set_dense_impl(2))
    n = 20
    u = _rand_op(k, 11 + k)
    u3 = _rand_op(3, 77)
    v0 = _rand_state(n, 1, 5 * k) * 0.7
    sv = v0.to(torch.complex64).cuda().contiguous()
    ref = v0.to(torch.complex128).cuda().contiguous()
    m = torch.as_tensor(u).to(torch.complex64).cuda().contiguous()
    m3 = torch.as_tensor(u3).to(torch.complex64).cuda().contiguous()
    mref = torch.as_tensor(u).to(torch.complex128).cuda().contiguous()
    m3ref = torch.as_tensor(u3).to(torch.complex128).cuda().contiguous()
    sites = _lib.int_array([n - 1 - b for b in bits])
    sites3 = _lib.int_array([2, 9, 15])
    chain = torch.zeros(6, dtype=torch.float64, device="cuda")
    st = _lib.stream_ptr()
    for i in range(50):
        if i == 25:
            _lib.check(L.qgb_op_action_unitary_chain(sv.data_ptr(), _lib.QGB_C64, n, sites3, 3, m3.data_ptr(), 0, 1, 0,
                                                     chain.data_ptr(), i, st))
            _lib.check(L.qgb_op_action(ref.data_ptr(), _lib.QGB_C128, n, sites3, 3, m3ref.data_ptr(), 0, 1, 0, st))
        _lib.check(L.qgb_op_action_unitary_chain(sv.data_ptr(), _lib.QGB_C64, n, sites, k, m.data_ptr(), 0, 1, 0,
                                                 chain.data_ptr(), i + (i >= 25), st))
        _lib.check(L.qgb_op_action(ref.data_ptr(), _lib.QGB_C128, n, sites, k, mref.data_ptr(), 0, 1, 0, st))
    _lib.check(L.qgb_check_status(st))
    got, want = sv.to(torch.complex128).cpu().numpy(), ref.cpu().numpy()
    assert abs(np.linalg.norm(got) - 0.7) < 0.7 * 1e-6
    assert np.max(np.abs(got - want)) / np.max(np.abs(want)) < 2e-5


def test_norm_modes_of_the_executor_agree():
    """The same 20-qubit brickwork with the norm chain (default), group norms
    restored in every pass, and no norm control: chain and row modes keep the
    norm, all agree with complex128 within the complex64 bar, and without
    control the norm drifts by the tensor cores' shrinkage."""
    from qaravan_gb300 import StatevectorSim, _lib, engine, workloads
    from qaravan_gb300.circuits import Circuit
    _lib.check(_lib.lib().qgb_set_dense_impl(2))
    n = 20
    circ = Circuit(workloads.brickwork_gates(n, 20, 31), n=n)
    v128 = StatevectorSim(circ, dtype=torch.complex128).get_statevector().cpu().numpy()
    out = {}
    try:
        for mode in ("chain", "row", "off"):
            engine.set_norm_restore(mode)
            out[mode] = StatevectorSim(circ, dtype=torch.complex64).get_statevector().to(torch.complex128).cpu().numpy()
    finally:
        engine.set_norm_restore("chain")
    for mode in ("chain", "row"):
        assert abs(np.linalg.norm(out[mode]) - 1.0) < 1.5e-6
    for v in out.values():
        assert np.max(np.abs(v - v128)) < 1e-6
    assert np.linalg.norm(out["off"]) < np.linalg.norm(out["chain"])
