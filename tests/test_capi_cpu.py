"""C ABI checks that need no GPU: the library builds, loads, exports every
symbol ``include/qgb.h`` declares, the ctypes struct matches the C layout, and
argument errors are rejected on the host before any CUDA call."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "qgb.h")


def _declared():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|size_t|void|const char\*)\s+(qgb_\w+)\s*\(", text, re.M)))


@pytest.fixture(scope="module")
def lib():
    from qaravan_gb300 import build, _lib
    build.build()
    return _lib.lib()


def test_header_symbols_exported(lib):
    names = _declared()
    assert len(names) >= 15
    out = subprocess.run(["nm", "-D", "--defined-only", os.path.join(ROOT, "qaravan_gb300", "_lib", "libqgb.so")],
                         capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (qgb_\w+)", out))
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    from qaravan_gb300 import _lib
    bound = set(_lib.SIGNATURES)
    assert set(names) <= bound | {"qgb_sweep_noalloc"}, set(names) - bound


def test_sweep_struct_layout(lib):
    from qaravan_gb300 import _lib
    src = r'''
#include <stdio.h>
#include <stddef.h>
#include "qgb.h"
int main(void) {
  printf("%zu %zu %zu %zu\n", sizeof(qgb_sweep), offsetof(qgb_sweep, op_k), offsetof(qgb_sweep, op_pos),
         offsetof(qgb_sweep, op_mat));
  return 0;
}
'''
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        open(c, "w").write(src)
        exe = os.path.join(d, "t")
        subprocess.check_call(["gcc", "-I" + os.path.join(ROOT, "include"), c, "-o", exe])
        vals = [int(x) for x in subprocess.check_output([exe]).split()]
    S = _lib.Sweep
    assert vals == [C.sizeof(S), S.op_k.offset, S.op_pos.offset, S.op_mat.offset]


def test_abi_version_and_host_validation(lib):
    from qaravan_gb300 import _lib
    assert lib.qgb_abi_version() == 1
    idx = _lib.int_array([0])
    # n out of range, k out of range, bad site, bad dtype: all rejected before touching CUDA
    assert lib.qgb_op_action(4096, 0, 0, idx, 1, 4096, 0, 1, 0, None) == -1
    assert lib.qgb_op_action(4096, 0, 4, idx, 7, 4096, 0, 1, 0, None) == -1
    assert lib.qgb_op_action(4096, 0, 4, _lib.int_array([5]), 1, 4096, 0, 1, 0, None) == -1
    assert b"out of range" in lib.qgb_last_error()
    assert lib.qgb_op_action(4096, 7, 4, idx, 1, 4096, 0, 1, 0, None) == -1
    assert lib.qgb_op_action(4096, 0, 4, _lib.int_array([1, 1]), 2, 4096, 0, 1, 0, None) == -1
    assert b"repeated" in lib.qgb_last_error()
    sw = _lib.Sweep()
    sw.low_bits, sw.n_high, sw.n_ops = 20, 0, 0
    assert lib.qgb_apply_sweep(4096, 0, 10, C.byref(sw), 4096, 0, 1, 0, None) == -1  # tile wider than state
    assert lib.qgb_pauli_expectation(4096, 0, 3, b"ixq", None, 1, 1, 0, 1, 1, 1 << 20, None) == -1
    assert lib.qgb_reduce_scratch_bytes(20, 3, 1) > 0
    assert lib.qgb_dm_apply_superop(4096, 0, 3, _lib.int_array([0, 1, 2, 0]), 4, 1, 1, 0, None) == -1
    # norm chain: a missing or misaligned chain buffer and a negative link, then the op checks
    assert lib.qgb_op_action_unitary_chain(4096, 0, 4, idx, 1, 4096, 0, 1, 0, None, 0, None) == -1
    assert b"chain" in lib.qgb_last_error()
    assert lib.qgb_op_action_unitary_chain(4096, 0, 4, idx, 1, 4096, 0, 1, 0, 4100, 0, None) == -1
    assert lib.qgb_op_action_unitary_chain(4096, 0, 4, idx, 1, 4096, 0, 1, 0, 4096, -1, None) == -1
    assert b"link" in lib.qgb_last_error()
    assert lib.qgb_op_action_unitary_chain(4096, 0, 4, _lib.int_array([5]), 1, 4096, 0, 1, 0, 4096, 0, None) == -1
    assert b"out of range" in lib.qgb_last_error()


ADJ_FIELDS = ["op_k", "op_pos", "op_mat", "op_out", "op_gen_col", "op_gen_val"]
ADJ_SRC = r'''
#include <stdio.h>
#include <stddef.h>
#include "qgb.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu %zu\n", sizeof(qgb_adjoint_sweep), offsetof(qgb_adjoint_sweep, op_k),
         offsetof(qgb_adjoint_sweep, op_pos), offsetof(qgb_adjoint_sweep, op_mat),
         offsetof(qgb_adjoint_sweep, op_out), offsetof(qgb_adjoint_sweep, op_gen_col),
         offsetof(qgb_adjoint_sweep, op_gen_val));
  return 0;
}
'''


def test_adjoint_sweep_struct_layout(lib):
    from qaravan_gb300 import _lib
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        open(c, "w").write(ADJ_SRC)
        exe = os.path.join(d, "t")
        subprocess.check_call(["gcc", "-I" + os.path.join(ROOT, "include"), c, "-o", exe])
        vals = [int(x) for x in subprocess.check_output([exe]).split()]
    S = _lib.AdjointSweep
    assert vals == [C.sizeof(S)] + [getattr(S, f).offset for f in ADJ_FIELDS]


def test_adjoint_sweep_host_validation(lib):
    """Malformed adjoint-sweep descriptions are rejected before any CUDA call."""
    from qaravan_gb300 import _lib

    def sweep(k=1, pos=(0, 1), out=-1, col=(1, 0), val=((1, 0), (1, 0))):
        sw = _lib.AdjointSweep()
        sw.low_bits, sw.n_high, sw.n_ops = 3, 2, 1
        sw.high_bits[0], sw.high_bits[1] = 5, 7
        sw.op_k[0] = k
        sw.op_pos[0][0], sw.op_pos[0][1] = pos
        sw.op_out[0] = out
        for r in range(2):
            sw.op_gen_col[0][r] = col[r]
            sw.op_gen_val[0][r][0], sw.op_gen_val[0][r][1] = val[r]
        return sw

    A, B, M = 1 << 20, 1 << 24, 4096  # distinct fake aligned pointers: nothing is launched

    def call(sw, n=10, out=B + (1 << 22), scr=None, nb=0):
        return lib.qgb_adjoint_sweep_step(A, B, 0, n, C.byref(sw), M, 0, 1, 0, out, scr, nb, None)

    assert call(sweep(k=3)) == -1 and b"width" in lib.qgb_last_error()
    assert call(sweep(k=2, pos=(1, 1))) == -1 and b"tile bit" in lib.qgb_last_error()
    assert call(sweep(pos=(5, 0))) == -1  # the tile has 5 bits
    assert call(sweep(), n=4) == -1  # tile wider than the state
    assert call(sweep(out=0, val=((0.5, 0), (1, 0)))) == -1 and b"Pauli" in lib.qgb_last_error()
    assert call(sweep(out=0, col=(1, 1))) == -1 and b"permutation" in lib.qgb_last_error()  # rows share a column
    assert call(sweep(out=0)) == -4  # derivative wanted, no scratch
    assert call(sweep(out=0), out=None) == -1
    assert lib.qgb_adjoint_sweep_step(A, A + 64, 0, 10, C.byref(sweep()), M, 0, 1, 0, None, None, 0, None) == -1
    assert b"overlap" in lib.qgb_last_error()
    assert lib.qgb_adjoint_sweep_scratch_bytes(20, 12, 64, 64) == 8 * 64 * 32 * 64
    assert lib.qgb_adjoint_sweep_scratch_bytes(24, 12, 10, 1) == 8 * 2048 * 10


def test_dm_batch_tables_are_checked_on_the_host(lib):
    """qgb_dm_batch_build validates circuits and passes before anything runs
    (host code only: no GPU needed)."""
    import ctypes as C
    import numpy as np
    from qaravan_gb300 import _lib
    from qaravan_gb300.batch import _DMB_CIRC, _DMB_PASS
    assert lib.qgb_dm_batch_circuit_bytes() == _DMB_CIRC.itemsize
    assert lib.qgb_dm_batch_pass_bytes() == _DMB_PASS.itemsize

    def tables(n=8, npass=3, **over):
        c = np.zeros(1, dtype=_DMB_CIRC)
        c[0] = (4096, n, 0, npass, 0)
        p = np.zeros(npass, dtype=_DMB_PASS)
        for j in range(npass):
            p[j]["mat"] = 8192
            p[j]["circ"] = 0
            p[j]["bits"] = [0, 1, 2, 3, 4, 5]
            p[j]["flags"] = (8 if j == 0 else 0) | (4 if j == npass - 1 else 0)
            p[j]["tslot"] = -1
        for k, v in over.items():
            idx, field = k.split("_", 1)
            p[int(idx[1:])][field] = v
        return c, p

    def build(c, p):
        n_items = lib.qgb_dm_batch_items(c.ctypes.data, len(c), 4)
        nbytes = lib.qgb_dm_batch_table_bytes(len(c), len(p), n_items)
        buf = np.zeros(nbytes, dtype=np.uint8)
        return lib.qgb_dm_batch_build(buf.ctypes.data, nbytes, c.ctypes.data, len(c), p.ctypes.data, len(p), 4)

    c, p = tables()
    assert build(c, p) == 0
    # 8 qubits: 2^16 entries = 8 tiles -> one item per pass (items hold 16 tiles unless the pass
    # has fewer), 3 passes, 1 finishing item; 12 qubits: 2048 tiles -> min(4, 2048 / 16) = 4 items
    assert lib.qgb_dm_batch_items(c.ctypes.data, 1, 4) == 4
    c12, _ = tables(n=12)
    assert lib.qgb_dm_batch_items(c12.ctypes.data, 1, 4) == 3 * 4 + 1
    assert build(*tables(p1_bits=[0, 1, 2, 3, 4, 4])) == _lib.QGB_EINVAL      # repeated bit
    assert build(*tables(p1_bits=[0, 1, 2, 3, 4, 16])) == _lib.QGB_EINVAL     # bit beyond 2n
    assert build(*tables(p1_flags=8)) == _lib.QGB_EINVAL                      # first-pass flag on pass 1
    assert build(*tables(p2_flags=0)) == _lib.QGB_EINVAL                      # last pass not flagged
    assert build(*tables(p2_flags=5, p2_tslot=1)) == _lib.QGB_EINVAL          # head reads a pass that is no tail
    assert build(*tables(p1_flags=2, p2_flags=5, p2_tslot=1)) == 0             # tail then head
    assert build(*tables(n=15)) == _lib.QGB_EINVAL                             # beyond 14 qubits
    assert build(*tables(p0_mat=0)) == _lib.QGB_EINVAL                         # no matrix
