"""The allocation-free Pauli expectation gives the same numbers as the
buffer-taking one.

qgb_pauli_expectation_noalloc exists for callers that may not allocate device
memory (real-time loops that may not stall on the allocator, plugins inside an
application that owns all device memory, fully reserved GPUs): it keeps its
partial sums in a fixed device array inside the library instead of a caller
buffer. This file is collected last so that, if it fails, a run that stops at
the first failure has already run every other test; it also passes alone in a
fresh process (it builds the library and makes its own states).
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _state(n, dtype, seed):
    g = torch.Generator().manual_seed(seed)
    re = torch.randn(2 ** n, generator=g, dtype=torch.float64)
    im = torch.randn(2 ** n, generator=g, dtype=torch.float64)
    v = torch.complex(re, im)
    v = v / torch.linalg.vector_norm(v)
    return v.to(dtype).cuda().contiguous()


def _terms(n, seed):
    rng = np.random.default_rng(seed)
    terms = [(1.0, 'i' * q + 'zz' + 'i' * (n - q - 2)) for q in range(n - 1)]
    terms += [(0.7, 'i' * q + 'x' + 'i' * (n - q - 1)) for q in range(n)]
    terms += [(float(rng.normal()), ''.join(rng.choice(list('ixyz'), size=n))) for _ in range(12)]
    return terms


@pytest.mark.parametrize("dtype,n", [(torch.complex64, 20), (torch.complex128, 18), (torch.complex64, 5)])
def test_noalloc_matches_buffered_entry_point_twice(cuda_ok, dtype, n):
    from qaravan_gb300 import _lib, build
    build.build()
    L = _lib.lib()
    code = _lib.dtype_code(dtype)
    st = _lib.stream_ptr()
    sv = _state(n, dtype, 123 + n)
    terms = _terms(n, n)
    strings = "".join(s for _, s in terms).encode()
    coeff = _lib.double_array([c for c, _ in terms])
    nt = len(terms)
    ref = torch.empty(nt, dtype=torch.float64, device="cuda")
    nbytes = L.qgb_reduce_scratch_bytes(n, nt, 1)
    scratch = torch.empty(nbytes // 8 + 1, dtype=torch.float64, device="cuda")
    _lib.check(L.qgb_pauli_expectation(sv.data_ptr(), code, n, strings, coeff, nt, 1, 0, ref.data_ptr(),
                                       scratch.data_ptr(), nbytes, st), "pauli_expectation")
    tol = 1e-5 if dtype == torch.complex64 else 1e-12
    for _ in range(2):  # two calls in a row share the fixed array
        out = torch.full((nt,), float("nan"), dtype=torch.float64, device="cuda")
        _lib.check(L.qgb_pauli_expectation_noalloc(sv.data_ptr(), code, n, strings, coeff, nt, out.data_ptr(), st),
                   "pauli_expectation_noalloc")
        torch.cuda.synchronize()
        assert torch.max(torch.abs(out - ref)).item() < tol


def test_noalloc_rejects_sizes_beyond_its_fixed_scratch(cuda_ok):
    from qaravan_gb300 import _lib, build
    build.build()
    L = _lib.lib()
    n = 24  # 1216 partial sums per term: at most 107 terms fit, and the entry point caps at 64
    sv = _state(n, torch.complex64, 1)
    out = torch.empty(80, dtype=torch.float64, device="cuda")
    strings = ("z" + "i" * (n - 1)).encode() * 80
    rc = L.qgb_pauli_expectation_noalloc(sv.data_ptr(), _lib.QGB_C64, n, strings, None, 80, out.data_ptr(),
                                         _lib.stream_ptr())
    assert rc == -1
    assert b"1..64" in L.qgb_last_error()
