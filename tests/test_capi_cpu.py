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
    assert call(sweep(out=0)) == -4  # derivative wanted, no scratch
    assert call(sweep(out=0), out=None) == -1
    assert lib.qgb_adjoint_sweep_step(A, A + 64, 0, 10, C.byref(sweep()), M, 0, 1, 0, None, None, 0, None) == -1
    assert b"overlap" in lib.qgb_last_error()
    assert lib.qgb_adjoint_sweep_scratch_bytes(20, 12, 64, 64) == 8 * 64 * 32 * 64
    assert lib.qgb_adjoint_sweep_scratch_bytes(24, 12, 10, 1) == 8 * 2048 * 10
