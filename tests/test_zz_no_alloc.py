"""The allocation-free Pauli expectation gives the same numbers as the
buffer-taking one.

qgb_pauli_expectation_noalloc exists for callers that may not allocate device
memory (real-time loops that may not stall on the allocator, plugins inside an
application that owns all device memory, fully reserved GPUs): it keeps its
partial sums in a fixed device array inside the library, which holds the
partial sums of up to 64 terms, instead of a caller buffer. This file is
collected last so that, if it fails, a run that stops at the first failure has
already run every other test; it also passes alone in a fresh process (it
builds the library and makes its own states).
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


def _compare(L, sv, n, code, terms, tol, calls=2):
    from qaravan_gb300 import _lib
    st = _lib.stream_ptr()
    strings = "".join(s for _, s in terms).encode()
    coeff = _lib.double_array([c for c, _ in terms])
    nt = len(terms)
    ref = torch.empty(nt, dtype=torch.float64, device="cuda")
    nbytes = L.qgb_reduce_scratch_bytes(n, nt, 1)
    scratch = torch.empty(nbytes // 8 + 1, dtype=torch.float64, device="cuda")
    _lib.check(L.qgb_pauli_expectation(sv.data_ptr(), code, n, strings, coeff, nt, 1, 0, ref.data_ptr(),
                                       scratch.data_ptr(), nbytes, st), "pauli_expectation")
    for _ in range(calls):
        out = torch.full((nt,), float("nan"), dtype=torch.float64, device="cuda")
        _lib.check(L.qgb_pauli_expectation_noalloc(sv.data_ptr(), code, n, strings, coeff, nt, out.data_ptr(), st),
                   "pauli_expectation_noalloc")
        torch.cuda.synchronize()
        scale = max(1.0, torch.max(torch.abs(ref)).item())
        assert torch.max(torch.abs(out - ref)).item() < tol * scale


def test_noalloc_64_terms_with_one_x_mask_split_over_two_launches(cuda_ok):
    # 40 consecutive terms share the X mask of 'x' on site 0: more than the 32 terms one
    # launch takes, so that run is split in two; 64 terms is the entry point's maximum
    from qaravan_gb300 import _lib, build
    build.build()
    L = _lib.lib()
    n = 16
    rng = np.random.default_rng(5)
    sv = _state(n, torch.complex64, 77)
    terms = [(float(rng.normal()), 'x' + ''.join(rng.choice(list('iz'), size=n - 1))) for _ in range(40)]
    terms += [(float(rng.normal()), ''.join(rng.choice(list('ixyz'), size=n))) for _ in range(24)]
    assert len(terms) == 64
    _compare(L, sv, n, _lib.QGB_C64, terms, 1e-5)


def test_noalloc_64_bit_indices_on_32_qubits(cuda_ok):
    # 2^32 amplitudes (34 GB of complex64): the reduction kernels switch to 64-bit indices above 31 qubits
    from qaravan_gb300 import _lib, build
    build.build()
    L = _lib.lib()
    n = 32
    sv = torch.empty(2 ** n, dtype=torch.complex64, device="cuda")
    torch.view_as_real(sv).normal_(generator=torch.Generator(device="cuda").manual_seed(3))
    terms = [(1.0, 'z' + 'i' * (n - 1)), (0.5, 'i' * (n - 1) + 'x'), (-0.25, 'y' + 'i' * (n - 2) + 'y'),
             (2.0, 'x' * n)]
    _compare(L, sv, n, _lib.QGB_C64, terms, 1e-5)
    del sv
    torch.cuda.empty_cache()


def test_noalloc_second_call_leaves_free_device_memory_unchanged(cuda_ok):
    # the first call loads the library's reduction code and reserves the fixed array;
    # after it, calls reserve nothing
    from qaravan_gb300 import _lib, build
    build.build()
    L = _lib.lib()
    n = 20
    sv = _state(n, torch.complex64, 9)
    terms = _terms(n, 4)
    strings = "".join(s for _, s in terms).encode()
    coeff = _lib.double_array([c for c, _ in terms])
    out = torch.empty(len(terms), dtype=torch.float64, device="cuda")
    st = _lib.stream_ptr()
    _lib.check(L.qgb_pauli_expectation_noalloc(sv.data_ptr(), _lib.QGB_C64, n, strings, coeff, len(terms),
                                               out.data_ptr(), st), "pauli_expectation_noalloc")
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        _lib.check(L.qgb_pauli_expectation_noalloc(sv.data_ptr(), _lib.QGB_C64, n, strings, coeff, len(terms),
                                                   out.data_ptr(), st), "pauli_expectation_noalloc")
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


def test_noalloc_rejects_sizes_beyond_its_fixed_scratch(cuda_ok):
    from qaravan_gb300 import _lib, build
    build.build()
    L = _lib.lib()
    n = 24  # the entry point takes at most 64 terms
    sv = _state(n, torch.complex64, 1)
    out = torch.empty(80, dtype=torch.float64, device="cuda")
    strings = ("z" + "i" * (n - 1)).encode() * 80
    rc = L.qgb_pauli_expectation_noalloc(sv.data_ptr(), _lib.QGB_C64, n, strings, None, 80, out.data_ptr(),
                                         _lib.stream_ptr())
    assert rc == -1
    assert b"1..64" in L.qgb_last_error()
