"""The TMA-staged sweep kernel and the load/store sweep kernel agree with the
oracle on every tile geometry (low/high bit splits, op widths 1..5, batched
states with per-state matrices)."""
import numpy as np
import pytest
import torch

from oracle import ref

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built(cuda_ok):
    from qaravan_gb300 import build
    build.build()
    yield
    from qaravan_gb300 import _lib
    _lib.lib().qgb_set_sweep_impl(0)


def _run_plan(dtype, n, gates, width, tile, low, impl, batch=1, init=None):
    from qaravan_gb300 import _lib, compiler
    from qaravan_gb300.engine import Executor
    from qaravan_gb300.statevector import gates_to_ops
    _lib.check(_lib.lib().qgb_set_sweep_impl(impl))
    ops = gates_to_ops(gates, n)
    isz = 8 if dtype == torch.complex64 else 16
    plan = compiler.compile_ops(ops, n, mode="sweep", width=width, tile_bits=tile, low_bits=low,
                                max_sweep_k=5 if isz == 8 else 4, itemsize=isz)
    ex = Executor(plan, dtype, "cuda")
    st = torch.as_tensor(init).to(dtype).cuda().contiguous()
    ex.run(st, batch=batch, stride=2 ** n if batch > 1 else 0)
    _lib.check(_lib.lib().qgb_check_status(None))
    return st.cpu().numpy()


GEOMS = [(14, 2, 10, 4), (14, 3, 12, 5), (14, 4, 9, 3), (16, 2, 13, 6), (16, 5, 13, 5), (12, 2, 12, None),
         (18, 2, 14, 4), (18, 3, 8, 7)]


@pytest.mark.parametrize("dtype", [torch.complex64, torch.complex128])
@pytest.mark.parametrize("n,width,tile,low", GEOMS)
def test_sweep_kernels_agree_with_oracle(dtype, n, width, tile, low):
    from qaravan_gb300 import workloads
    if dtype == torch.complex128 and width > 4:
        width = 4
    gates = workloads.brickwork_gates(n, 3, 100 + n + width)
    exp = ref.run_sv(gates, n)
    v0 = np.zeros(2 ** n, complex)
    v0[0] = 1
    tol = 1e-5 if dtype == torch.complex64 else 1e-12
    a = _run_plan(dtype, n, gates, width, tile, low, 0, init=v0)
    b = _run_plan(dtype, n, gates, width, tile, low, 1, init=v0)
    assert np.max(np.abs(a - exp)) < tol
    assert np.max(np.abs(b - exp)) < tol


@pytest.mark.parametrize("dtype", [torch.complex64, torch.complex128])
@pytest.mark.parametrize("impl", [0, 1])
def test_batched_sweep_per_state_matrices(dtype, impl):
    from qaravan_gb300 import _lib, compiler, workloads
    from qaravan_gb300.engine import Executor
    from qaravan_gb300.statevector import gates_to_ops
    n, B = 12, 6
    base = workloads.brickwork_gates(n, 2, 5)
    ops = gates_to_ops(base, n)
    isz = 8 if dtype == torch.complex64 else 16
    plan = compiler.compile_ops(ops, n, mode="sweep", width=2, tile_bits=9, low_bits=4, itemsize=isz,
                                max_sweep_k=4)
    # per-state matrices: each state gets its own random unitaries in the plan's slots
    rng = np.random.default_rng(1)
    per = []
    for b in range(B):
        per.append([workloads.haar_unitary(m.shape[0], rng) for m in plan.matrices])
    flat = np.stack([np.concatenate([m.reshape(-1) for m in mats]) for mats in per])
    mats = torch.as_tensor(flat).to(dtype).cuda().contiguous()
    ex = Executor(plan, dtype, "cuda")
    _lib.check(_lib.lib().qgb_set_sweep_impl(impl))
    st = torch.zeros(B, 2 ** n, dtype=dtype, device="cuda")
    st[:, 0] = 1
    ex.run(st, batch=B, stride=2 ** n, mats=mats, mat_stride=flat.shape[1])
    got = st.cpu().numpy()
    tol = 1e-5 if dtype == torch.complex64 else 1e-12
    for b in range(B):
        v = np.zeros(2 ** n, complex)
        v[0] = 1
        for s in plan.steps:
            tile_to_bit = list(range(s.low_bits)) + list(s.high_bits)
            for pos, mi in s.ops:
                v = ref.op_action(per[b][mi], [n - 1 - tile_to_bit[p] for p in pos], v)
        assert np.max(np.abs(got[b] - v)) < tol
