"""The fused forward of BatchedAnsatz replayed on the CPU: the block plan and
the per-set fusion tables (plan_fused_forward, fused_tables) are composed and
applied in numpy exactly as qgb_fuse_blocks and qgb_apply_sweep read them,
and the result equals every set's gates applied one by one through the
oracle's op_action."""
import numpy as np
import pytest

from oracle import ref


def _hea_gates(n, layers):
    from qaravan_gb300.gates import CNOT
    gates = []
    for l in range(layers):
        for q in range(n):
            gates.append(("RY", [q], 2 * (l * n + q)))
            gates.append(("RZ", [q], 2 * (l * n + q) + 1))
        for q in range(n - 1):
            g = CNOT([q + 1, q], n)
            gates.append(("fixed", list(g.indices), np.asarray(g.matrix, dtype=np.complex128)))
    return gates


def _gate_matrix(g, params):
    from qaravan_gb300.adjoint import _GEN, _KIND
    name, idx, p = g
    if name == "fixed":
        return p
    gen = _GEN[_KIND[name]]
    th = params[p]
    return np.cos(th) * np.eye(gen.shape[0]) - 1j * np.sin(th) * gen


def _embed(m, pos, k):
    """The block-matrix embedding qgb_fuse_blocks forms: op bit j on block bit
    pos[j], 0 = most significant."""
    kop = len(pos)
    D = 1 << k
    e = np.zeros((D, D), dtype=np.complex128)
    mask = sum(1 << (k - 1 - p) for p in pos)
    for r in range(D):
        for c in range(D):
            if (r & ~mask) != (c & ~mask):
                continue
            sr = sum(((r >> (k - 1 - p)) & 1) << (kop - 1 - j) for j, p in enumerate(pos))
            sc = sum(((c >> (k - 1 - p)) & 1) << (kop - 1 - j) for j, p in enumerate(pos))
            e[r, c] = m[sr, sc]
    return e


@pytest.mark.parametrize("n,layers,width,nsets", [(9, 3, 3, 3), (14, 2, 3, 2), (15, 2, 4, 2), (10, 2, 2, 2),
                                                  (13, 2, 5, 1)])
def test_fused_forward_tables_replay(n, layers, width, nsets):
    from qaravan_gb300.adjoint import fused_tables, plan_fused_forward
    from qaravan_gb300.engine import _FUSE_BLOCK, _FUSE_ENTRY
    gates = _hea_gates(n, layers)
    G = len(gates)
    bits = [[n - 1 - q for q in idx] for _, idx, _ in gates]
    fixed = [(g, gt[2]) for g, gt in enumerate(gates) if gt[0] == "fixed"]
    fplan = plan_fused_forward(n, bits, fixed, width, 8)
    assert fplan is not None and fplan["blocks"] < G
    assert plan_fused_forward(n, bits, fixed, 6, 8) is None  # wider than the complex64 sweeps take
    host, ent_start = fused_tables(fplan, nsets, G)
    nb = nsets * len(fplan["blocks1"])
    blocks = host[:nb * _FUSE_BLOCK.itemsize].view(_FUSE_BLOCK)
    ents = host[ent_start:].view(_FUSE_ENTRY)
    rng = np.random.default_rng(n + layers)
    params = rng.uniform(-np.pi, np.pi, size=(nsets, 2 * n * layers))
    # the [set][gate][16] matrix buffer qgb_param_matrices fills (fixed gates from the template)
    opm = np.zeros((nsets, G, 16), dtype=np.complex128)
    for s in range(nsets):
        for g, gt in enumerate(gates):
            m = _gate_matrix(gt, params[s])
            opm[s, g, :m.size] = m.reshape(-1)
    flat_opm = opm.reshape(-1)
    fused = np.zeros(nsets * fplan["total"], dtype=np.complex128)
    for b in blocks:
        k = int(b["k"])
        M = np.eye(1 << k, dtype=np.complex128)
        for e in ents[b["op_begin"]:b["op_end"]]:
            kop = int(e["k"])
            m = flat_opm[e["mat"]:e["mat"] + 4 ** kop].reshape(1 << kop, 1 << kop)
            M = _embed(m, [int(p) for p in e["pos"][:kop]], k) @ M
        fused[b["out"]:b["out"] + 4 ** k] = M.reshape(-1)
    for s in range(nsets):
        sv = ref.initial_sv(n).astype(np.complex128).reshape([2] * n)
        for L, high, ops in fplan["sweeps"]:
            flat_of = list(range(L)) + list(high)
            for pos, off in ops:
                k = len(pos)
                m = fused[s * fplan["total"] + off:s * fplan["total"] + off + 4 ** k].reshape(1 << k, 1 << k)
                sv = ref.op_action(m, [n - 1 - flat_of[p] for p in pos], sv)
        exp = ref.initial_sv(n).astype(np.complex128).reshape([2] * n)
        for gt in gates:
            exp = ref.op_action(_gate_matrix(gt, params[s]), gt[1], exp)
        assert np.max(np.abs(sv - exp)) < 1e-12


def test_fused_forward_only_while_its_matrix_buffer_stays_small():
    """The fused forward keeps every set's complex128 gate matrices (256 bytes per
    gate and set): at most 2 GiB, or the states' own size."""
    import torch
    from qaravan_gb300.adjoint import BatchedAnsatz
    ba = BatchedAnsatz.__new__(BatchedAnsatz)  # host fields only: no device needed
    ba._fused, ba.gates, ba.dtype = {"blocks": 1}, [None] * 2360, torch.complex64
    ba.n = 20
    assert ba._use_fused(64) and ba._use_fused(4096)
    ba.n = 10
    assert ba._use_fused(1024) and not ba._use_fused(65535)
    ba._fused = None
    assert not ba._use_fused(1)
