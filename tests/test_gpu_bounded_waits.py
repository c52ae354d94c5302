"""The failure path of the library's bounded device waits, without a GPU fault.

Every wait in the kernels (tile staged, MMAs complete, flags) gives up after a
time limit, records a status word and returns; ``qgb_check_status`` then
reports QGB_ETIMEOUT and the context stays usable. Here the shared wait helper
runs, through ``qgb_wait_probe``, on waits that cannot finish (an mbarrier
nobody arrives on, a flag nothing sets) with a 2 ms limit."""
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def L(cuda_ok):
    from qaravan_gb300 import _lib, build
    build.build()
    lib = _lib.lib()
    assert lib.qgb_check_status(_lib.stream_ptr()) == 0  # nothing pending from earlier tests
    return lib


def _next_launch_ok(L):
    """A normal launch after the timeout runs and is correct: the context is usable."""
    from qaravan_gb300 import _lib
    n = 14
    sv = torch.zeros(2 ** n, dtype=torch.complex64, device="cuda")
    _lib.check(L.qgb_init_basis(sv.data_ptr(), _lib.QGB_C64, n, 5, 1, 0, _lib.stream_ptr()), "init_basis")
    x = torch.tensor([[0, 1], [1, 0]], dtype=torch.complex64, device="cuda")
    _lib.check(L.qgb_op_action(sv.data_ptr(), _lib.QGB_C64, n, _lib.int_array([n - 1]), 1, x.data_ptr(), 0, 1, 0,
                               _lib.stream_ptr()), "op_action")
    assert L.qgb_check_status(_lib.stream_ptr()) == 0
    assert sv[4].item() == 1 and torch.count_nonzero(sv).item() == 1


@pytest.mark.parametrize("mode,code", [(0, b"code 3"), (1, b"code 4")])
def test_wait_that_cannot_finish_reports_timeout(L, mode, code):
    from qaravan_gb300 import _lib
    flag = torch.zeros(1, dtype=torch.int32, device="cuda")
    st = _lib.stream_ptr()
    assert L.qgb_wait_probe(mode, 2_000_000, flag.data_ptr(), st) == 0
    assert L.qgb_check_status(st) == -3  # QGB_ETIMEOUT
    assert code in L.qgb_last_error()
    assert L.qgb_check_status(st) == 0  # read and cleared
    _next_launch_ok(L)


def test_wait_that_completes_reports_nothing(L):
    from qaravan_gb300 import _lib
    st = _lib.stream_ptr()
    assert L.qgb_wait_probe(2, 2_000_000, None, st) == 0
    assert L.qgb_check_status(st) == 0


def test_wait_probe_rejects_bad_arguments(L):
    from qaravan_gb300 import _lib
    st = _lib.stream_ptr()
    assert L.qgb_wait_probe(7, 1000, None, st) == -1
    assert L.qgb_wait_probe(1, 1000, None, st) == -1
    assert L.qgb_wait_probe(0, 20_000_000_000, None, st) == -1
