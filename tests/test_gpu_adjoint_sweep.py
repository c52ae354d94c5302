"""The adjoint tile sweep (many gates per pass over state and co-state) against
the per-gate reverse steps through the C ABI: final states, co-states and every
rotation derivative, for batches with per-state matrices, 1- and 2-site gates
(dense, diagonal, and permutations such as CNOT, SWAP, X) on low and high bits,
tiles that force several passes, with the gates applied in register runs
(the default: consecutive gates on at most 3 tile bits per shared-memory pass)
and one shared-memory pass per gate; and the batched ansatz with and without
tile passes."""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built(cuda_ok):
    from qaravan_gb300 import build
    build.build()


def _haar(d, rng):
    q, r = np.linalg.qr(rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d)))
    return q * (np.diag(r) / np.abs(np.diag(r)))


_PERMS = [np.array([[0, 1], [1, 0]], complex),                                       # X
          np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0]], complex),  # CNOT
          np.array([[1, 0, 0, 0], [0, 0, 1, 0], [0, 1, 0, 0], [0, 0, 0, 1]], complex),  # SWAP
          np.array([[1, 0, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0], [0, 1, 0, 0]], complex),  # CNOT, control second
          np.array([[0, 0, 1, 0], [0, 0, 0, 1], [1, 0, 0, 0], [0, 1, 0, 0]], complex)]  # X on the first site


@pytest.fixture(scope="module", autouse=True)
def extra_generators():
    """Two-site generators whose rows are neither diagonal nor flipped (X (x) Z,
    Y (x) X), as rotation kinds 7 and 8 of the tables the sweep structs read."""
    from qaravan_gb300 import _lib, adjoint
    px, py, pz = adjoint._PX, adjoint._PY, adjoint._PZ
    extra = {7: np.kron(px, pz), 8: np.kron(py, px)}
    for k, m in extra.items():
        adjoint._GEN[k] = m
        adjoint._GEN_C[k] = _lib.double_array(np.stack([m.real, m.imag], axis=-1).reshape(-1))
        adjoint._GEN_ROWS[k] = [(int(np.flatnonzero(m[r])[0]), complex(m[r, np.flatnonzero(m[r])[0]]))
                                for r in range(4)]
    yield
    for k in extra:
        for t in (adjoint._GEN, adjoint._GEN_C, adjoint._GEN_ROWS):
            t.pop(k, None)


@pytest.fixture(params=[-1, 0], ids=["register_runs", "pass_per_gate"])
def runs(request):
    from qaravan_gb300 import _lib
    _lib.check(_lib.lib().qgb_set_adjoint_runs(request.param), "set_adjoint_runs")
    yield request.param
    _lib.lib().qgb_set_adjoint_runs(-1)


@pytest.mark.parametrize("dtype,tol", [(torch.complex64, 2e-5), (torch.complex128, 1e-12)])
@pytest.mark.parametrize("n,tile", [(9, 6), (11, 8), (7, 7)])
def test_adjoint_sweep_matches_per_gate_steps(dtype, tol, n, tile, runs):
    from qaravan_gb300 import _lib
    from qaravan_gb300.adjoint import _GEN, _GEN_C, _adjoint_sweep_struct, _plan_reverse
    L = _lib.lib()
    code = _lib.dtype_code(dtype)
    rng = np.random.default_rng(n * 100 + tile)
    B, N = 3, 2 ** n
    # gates in circuit order: (sites, kind or 0); rotations get per-state angles
    gates = []
    for _ in range(40):
        if rng.random() < 0.5:
            q = int(rng.integers(n))
            gates.append(([q], int(rng.integers(1, 4)) if rng.random() < 0.7 else 0))
        else:
            a, b = rng.choice(n, size=2, replace=False)
            gates.append(([int(a), int(b)], int(rng.integers(4, 9)) if rng.random() < 0.6 else 0))
    G = len(gates)
    mats = np.zeros((B, G, 16), dtype=np.complex128)
    for s in range(B):
        for g, (sites, kind) in enumerate(gates):
            d = 2 ** len(sites)
            if kind:
                t = rng.uniform(-3, 3)
                m = np.cos(t) * np.eye(d) - 1j * np.sin(t) * _GEN[kind]
            elif g % 3 == 0:  # fixed permutation gates: X, CNOT (either control), SWAP, X on one site of two
                m = _PERMS[0] if d == 2 else _PERMS[1 + (g // 3) % 4]
            else:
                m = _haar(d, rng)
            mats[s, g, :d * d] = m.reshape(-1)
    md = torch.as_tensor(mats.reshape(-1)).to(dtype).cuda()
    phi0 = rng.normal(size=(B, N)) + 1j * rng.normal(size=(B, N))
    lam0 = rng.normal(size=(B, N)) + 1j * rng.normal(size=(B, N))
    st = _lib.stream_ptr()
    # per-gate reference
    p1 = torch.as_tensor(phi0.reshape(-1)).to(dtype).cuda()
    l1 = torch.as_tensor(lam0.reshape(-1)).to(dtype).cuda()
    g1 = torch.zeros(G * B, dtype=torch.float64, device="cuda")
    nb = L.qgb_reduce_scratch_bytes(n, 32, B)
    scr = torch.empty(nb // 8 + 1, dtype=torch.float64, device="cuda")
    isz = md.element_size()
    for g in reversed(range(G)):
        sites, kind = gates[g]
        args = (p1.data_ptr(), l1.data_ptr(), code, n, _lib.int_array(sites), len(sites), md.data_ptr() + g * 16 * isz,
                16 * G)
        if kind:
            rc = L.qgb_adjoint_step_rotation(*args, _GEN_C[kind], B, N, g1.data_ptr() + g * B * 8, scr.data_ptr(), nb, st)
        else:
            rc = L.qgb_adjoint_step_batched(*args, B, N, None, scr.data_ptr(), nb, st)
        assert rc == 0, L.qgb_last_error()
    # tile passes
    p2 = torch.as_tensor(phi0.reshape(-1)).to(dtype).cuda()
    l2 = torch.as_tensor(lam0.reshape(-1)).to(dtype).cuda()
    g2 = torch.full((G * B,), np.nan, dtype=torch.float64, device="cuda")
    items = [(g, [n - 1 - q for q in gates[g][0]]) for g in reversed(range(G))]
    plan = _plan_reverse(items, n, tile)
    assert len(plan) > 1 or tile == n
    sb = L.qgb_adjoint_sweep_scratch_bytes(n, min(tile, n), 64, B)
    s2 = torch.empty(sb // 8 + 1, dtype=torch.float64, device="cuda")
    for lo, high, ops in plan:
        sw = _adjoint_sweep_struct(lo, high, [(b, g * 16, g if gates[g][1] else -1, gates[g][1]) for g, b in ops])
        rc = L.qgb_adjoint_sweep_step(p2.data_ptr(), l2.data_ptr(), code, n, C.byref(sw), md.data_ptr(), 16 * G, B, N,
                                      g2.data_ptr(), s2.data_ptr(), sb, st)
        assert rc == 0, L.qgb_last_error()
    assert _lib.lib().qgb_check_status(st) == 0
    scale = max(np.abs(phi0).max(), np.abs(lam0).max())
    assert (p1 - p2).abs().max().item() < tol * scale * 4
    assert (l1 - l2).abs().max().item() < tol * scale * 4
    rot = np.array([g for g in range(G) if gates[g][1]])
    a1 = g1.cpu().numpy().reshape(G, B)[rot]
    a2 = g2.cpu().numpy().reshape(G, B)[rot]
    assert np.isfinite(a2).all()
    assert np.max(np.abs(a1 - a2)) < tol * 20 * np.max(np.abs(a1))


@pytest.mark.parametrize("dtype,tol", [(torch.complex64, 2e-5), (torch.complex128, 1e-11)])
def test_batched_ansatz_tile_passes_match_per_gate_passes(dtype, tol, runs):
    from qaravan_gb300 import workloads
    from qaravan_gb300.adjoint import BatchedAnsatz
    n, layers, P = 14, 4, 5
    terms = [(1.0, "i" * q + "zz" + "i" * (n - q - 2)) for q in range(n - 1)] + \
            [(0.8, "i" * q + "x" + "i" * (n - q - 1)) for q in range(n)]
    x = np.stack([workloads.hea_params(n, layers, 40 + s).reshape(-1) for s in range(P)])
    a = BatchedAnsatz.hea(n, layers, dtype=dtype)
    b = BatchedAnsatz.hea(n, layers, dtype=dtype)
    b.__init__(n, b.gates, nparams=b.nparams, dtype=dtype, tile_bits=0)
    assert a._rev and not b._rev
    ea, ga = a.energy_and_grad(x, terms)
    eb, gb = b.energy_and_grad(x, terms)
    assert torch.max(torch.abs(ea - eb)).item() < tol * 10
    assert (torch.max(torch.abs(ga - gb)) / torch.max(torch.abs(gb))).item() < tol
