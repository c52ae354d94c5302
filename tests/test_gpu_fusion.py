"""Block matrices composed on the device (qgb_fuse_blocks) against the same
recipes composed on the host in complex128, for statevector and
density-matrix plans in every fused mode; and an out-of-bounds table entry is
skipped and reported."""
import numpy as np
import pytest
import torch

from qaravan_gb300 import compiler, workloads

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built(cuda_ok):
    from qaravan_gb300 import build
    build.build()


def _sv_ops(n, depth, seed):
    from qaravan_gb300.statevector import gates_to_ops
    return gates_to_ops(workloads.brickwork_gates(n, depth, seed), n)


def _dm_ops(n, depth, seed):
    from qaravan_gb300.density_matrix import dm_ops_for_gate
    circ = workloads.noisy_brickwork_circuit(n, depth, seed, p=2e-3)
    return [o for layer in circ.layers for g in layer for o in dm_ops_for_gate(g, n)]


@pytest.mark.parametrize("dtype", [torch.complex64, torch.complex128])
@pytest.mark.parametrize("which,mode,width", [("sv", "fused", 4), ("sv", "fused", 6), ("sv", "sweep", 3),
                                              ("dm", "fused", 6), ("dm", "sweep", 4)])
def test_device_fused_blocks_match_host_composition(dtype, which, mode, width):
    from qaravan_gb300 import _lib
    from qaravan_gb300.engine import Executor
    if which == "sv":
        nb, ops = 14, _sv_ops(14, 6, 21)
    else:
        nb, ops = 12, _dm_ops(6, 4, 22)
    isz = 8 if dtype == torch.complex64 else 16
    plan = compiler.compile_ops(ops, nb, mode=mode, width=width, tile_bits=10, itemsize=isz, device_fusion=True)
    ex = Executor(plan, dtype, "cuda")
    _lib.check(_lib.lib().qgb_check_status(_lib.stream_ptr()))
    got = ex.mats.cpu().numpy()
    tol = 2e-6 if dtype == torch.complex64 else 1e-13
    for i, m in enumerate(plan.matrices):
        want = compiler.recipe_matrix(m, plan.op_matrices)
        g = got[ex.mat_offsets[i]:ex.mat_offsets[i] + want.size].reshape(want.shape)
        assert np.max(np.abs(g - want)) < tol


def test_out_of_bounds_entry_is_skipped_and_reported():
    from qaravan_gb300 import _lib
    from qaravan_gb300.engine import _FUSE_BLOCK, _FUSE_ENTRY
    L = _lib.lib()
    blocks = np.zeros(1, dtype=_FUSE_BLOCK)
    blocks[0] = (0, 2, 0, 2, 0)
    ents = np.zeros(2, dtype=_FUSE_ENTRY)
    ents["k"][0], ents["pos"][0, 0], ents["mat"][0] = 1, 1, 0
    ents["k"][1], ents["pos"][1, 0], ents["mat"][1] = 1, 0, 1000  # matrix offset beyond op_elems
    opm = torch.tensor([0, 1, 1, 0], dtype=torch.complex128, device="cuda")  # X
    tb = torch.from_numpy(blocks.view(np.uint8).copy()).cuda()
    te = torch.from_numpy(ents.view(np.uint8).copy()).cuda()
    out = torch.empty(16, dtype=torch.complex128, device="cuda")
    _lib.check(L.qgb_fuse_blocks(out.data_ptr(), _lib.QGB_C128, 16, tb.data_ptr(), 1, te.data_ptr(), 2,
                                 opm.data_ptr(), 4, _lib.stream_ptr()))
    rc = L.qgb_check_status(_lib.stream_ptr())
    assert rc == -1 and b"fusion" in L.qgb_last_error()
    want = np.kron(np.eye(2), np.array([[0, 1], [1, 0]]))  # the valid entry: X on the low bit
    assert np.max(np.abs(out.cpu().numpy().reshape(4, 4) - want)) < 1e-15
    assert L.qgb_check_status(_lib.stream_ptr()) == 0  # the status was cleared
