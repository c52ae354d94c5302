"""Device-side fusion, checked on the CPU: the symbolic fusion makes the same
decisions as the host fusion, its recipes compose to the same block matrices,
and the packed tables the executor uploads decode (with the kernel's index
arithmetic, restated here in numpy) to those matrices."""
import numpy as np
import pytest

from oracle import ref
from qaravan_gb300 import compiler, workloads
from qaravan_gb300.density_matrix import dm_ops_for_gate
from qaravan_gb300.statevector import gates_to_ops


def _sv_ops(n, depth, seed):
    return gates_to_ops(workloads.brickwork_gates(n, depth, seed), n)


def _dm_ops(n, depth, seed):
    circ = workloads.noisy_brickwork_circuit(n, depth, seed, p=2e-3)
    ops = []
    for layer in circ.layers:
        for g in layer:
            ops.extend(dm_ops_for_gate(g, n))
    return ops


def _mixed_ops(seed):
    """Unsorted, non-adjacent and 3-/4-bit ops on 9 bits."""
    rng = np.random.default_rng(seed)
    ops = []
    for _ in range(60):
        k = int(rng.choice([1, 2, 2, 3, 4]))
        bits = [int(b) for b in rng.choice(9, size=k, replace=False)]
        ops.append(compiler.Op(bits, workloads.haar_unitary(2 ** k, rng)))
    return ops


@pytest.mark.parametrize("ops_fn,width", [(lambda: _sv_ops(12, 5, 1), 2), (lambda: _sv_ops(12, 5, 2), 4),
                                          (lambda: _sv_ops(14, 6, 3), 6), (lambda: _dm_ops(4, 3, 4), 4),
                                          (lambda: _dm_ops(4, 3, 5), 6), (lambda: _mixed_ops(6), 5),
                                          (lambda: _mixed_ops(7), 6)])
def test_symbolic_fusion_matches_host_fusion(ops_fn, width):
    ops = ops_fn()
    host = compiler.fuse(ops, width)
    sym = compiler.fuse_symbolic(ops, width)
    assert [b.bits for b in host] == [b.bits for b in sym]
    assert sum(b.n_ops for b in sym) == len(ops) >= sum(1 for _ in sym)
    mats = [np.asarray(o.matrix, dtype=np.complex128) for o in ops]
    for hb, sb in zip(host, sym):
        r = compiler.Recipe(list(sb.bits), [(i, list(ops[i].bits)) for i in sb.ops])
        assert np.max(np.abs(compiler.recipe_matrix(r, mats) - hb.matrix)) < 1e-12


def _decode_tables(host_bytes, starts, nblocks, nent, out_elems):
    """The kernel's composition, restated: identity, then each entry's matrix
    embedded through its pos[] list and applied from the left."""
    from qaravan_gb300.engine import _FUSE_BLOCK, _FUSE_ENTRY
    opm = host_bytes[starts[0]:starts[1]].view(np.complex128)
    blocks = host_bytes[starts[1]:starts[1] + nblocks * _FUSE_BLOCK.itemsize].view(_FUSE_BLOCK)
    ents = host_bytes[starts[2]:starts[2] + max(nent, 1) * _FUSE_ENTRY.itemsize].view(_FUSE_ENTRY)
    out = np.zeros(out_elems, np.complex128)
    for b in blocks:
        K = int(b["k"])
        D = 2 ** K
        m0 = np.eye(D, dtype=np.complex128)
        for e in range(int(b["op_begin"]), int(b["op_end"])):
            kop = int(ents["k"][e])
            pos = [int(p) for p in ents["pos"][e, :kop]]
            G = opm[int(ents["mat"][e]):int(ents["mat"][e]) + 4 ** kop].reshape(2 ** kop, 2 ** kop)
            rowbits = [sum(((s >> (kop - 1 - j)) & 1) << (K - 1 - pos[j]) for j in range(kop)) for s in range(2 ** kop)]
            opmask = sum(1 << (K - 1 - p) for p in pos)
            m1 = np.zeros_like(m0)
            for r in range(D):
                so = sum(((r >> (K - 1 - pos[j])) & 1) << (kop - 1 - j) for j in range(kop))
                rb = r & ~opmask
                m1[r] = sum(G[so, si] * m0[rb | rowbits[si]] for si in range(2 ** kop))
            m0 = m1
        out[int(b["out"]):int(b["out"]) + D * D] = m0.reshape(-1)
    return out


def test_executor_tables_decode_to_the_block_matrices(monkeypatch):
    """Packs a device-fused plan the way the executor does (without a GPU) and
    decodes the tables with the kernel's arithmetic."""
    import torch
    from qaravan_gb300 import engine
    ops = _mixed_ops(11)
    plan = compiler.compile_ops(ops, 9, mode="fused", width=5, device_fusion=True)
    captured = {}

    class FakeLib:
        def qgb_fuse_block_bytes(self):
            return engine._FUSE_BLOCK.itemsize

        def qgb_fuse_entry_bytes(self):
            return engine._FUSE_ENTRY.itemsize

        def qgb_fuse_blocks(self, out, code, out_elems, blocks, nblocks, ents, nent, opm, nop, stream):
            captured.update(out_elems=out_elems, nblocks=nblocks, nent=nent, starts=(opm, blocks, ents))
            return 0

    monkeypatch.setattr(engine._lib, "lib", lambda: FakeLib())
    monkeypatch.setattr(engine._lib, "stream_ptr", lambda *a: 0)
    ex = engine.Executor.__new__(engine.Executor)
    ex.dtype, ex.code, ex.device = torch.complex128, 1, torch.device("cpu")
    offs = ex._fuse_on_device(plan)
    host = ex._pinned.numpy()
    base = ex._fuse_tables.data_ptr()
    starts = [s - base for s in captured["starts"]]
    out = _decode_tables(host, starts, captured["nblocks"], captured["nent"], captured["out_elems"])
    for i, m in enumerate(plan.matrices):
        want = compiler.recipe_matrix(m, plan.op_matrices)
        got = out[offs[i]:offs[i] + want.size].reshape(want.shape)
        assert np.max(np.abs(got - want)) < 1e-12


def test_device_fused_plans_match_oracle():
    n = 10
    gates = workloads.brickwork_gates(n, 4, 3)
    ops = gates_to_ops(gates, n)
    for mode, width, tile in (("fused", 4, 0), ("fused", 6, 0), ("sweep", 3, 9)):
        plan = compiler.compile_ops(ops, n, mode=mode, width=width, tile_bits=tile, low_bits=3, device_fusion=True)
        assert plan.device_fused
        host = compiler.Plan(plan.nbits, plan.steps, [compiler.recipe_matrix(m, plan.op_matrices)
                                                      for m in plan.matrices], plan.n_gates)
        from test_compiler_cpu import run_plan_numpy
        v0 = np.zeros(2 ** n, complex)
        v0[0] = 1
        assert np.max(np.abs(run_plan_numpy(host, v0) - ref.run_sv(gates, n))) < 1e-12


def test_plan_cache_reuses_structure_with_new_matrices():
    """A second compile of the same structure (bits, unitarity, options) reuses the
    fusion decisions; its recipes compose the new matrices exactly like a fresh
    host fusion. A change of bits or of unitarity misses the cache."""
    from qaravan_gb300.compiler import Op, compile_ops, fuse, recipe_matrix
    rng = np.random.default_rng(11)
    n = 9

    def haar(d):
        q, r = np.linalg.qr(rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d)))
        return q * (np.diag(r) / np.abs(np.diag(r)))

    bits = [[int(a)] if rng.random() < 0.4 else [int(a), int((a + 1 + rng.integers(n - 1)) % n)]
            for a in rng.integers(n, size=60)]
    ops1 = [Op(b, haar(2 ** len(b))) for b in bits]
    ops2 = [Op(b, haar(2 ** len(b))) for b in bits]
    p1 = compile_ops(ops1, n, mode="fused", width=4, device_fusion=True)
    p2 = compile_ops(ops2, n, mode="fused", width=4, device_fusion=True)
    assert p2.steps is p1.steps and p2.matrices is p1.matrices
    host = fuse(ops2, 4)
    assert len(host) == len(p2.matrices)
    for blk, rec in zip(host, p2.matrices):
        assert list(blk.bits) == list(rec.bits)
        assert np.max(np.abs(recipe_matrix(rec, p2.op_matrices) - blk.matrix)) < 1e-12
    ops3 = [Op(o.bits, o.matrix * (1.5 if i == 7 else 1.0)) for i, o in enumerate(ops2)]  # op 7 not unitary
    p3 = compile_ops(ops3, n, mode="fused", width=4, device_fusion=True)
    assert p3.steps is not p1.steps
    ops4 = [Op(list(reversed(o.bits)), o.matrix) for o in ops2]
    assert compile_ops(ops4, n, mode="fused", width=4, device_fusion=True).steps is not p1.steps
