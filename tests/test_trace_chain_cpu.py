"""Host logic of the density-matrix trace chain without a GPU.

A complex64 density matrix on the tensor cores loses ~1e-7 of its trace per
pass (round-toward-zero accumulation). Channels keep the trace, so the
executor measures it where the ops applied so far are whole channels (both
halves of every unitary gate) and scales the next tensor-core pass by
reference / measured trace. These tests check which cuts the compiler marks as
whole, which op sequences keep the trace, and the order of the executor's
calls (the library replaced by a recorder, so no kernel runs)."""
import numpy as np
import pytest
import torch

from qaravan_gb300 import _lib, engine, workloads
from qaravan_gb300.compiler import DenseStep, NormalizeStep, Plan, compile_ops, trace_preserving, whole_cuts
from qaravan_gb300.density_matrix import dm_ops_for_gate
from qaravan_gb300.gates import ID, Reset
from qaravan_gb300.noise import amplitude_damping, depolarizing


def _noisy_ops(n, depth, seed):
    ops = []
    for g in workloads.brickwork_gates(n, depth, seed):
        ops += dm_ops_for_gate(g, n)
        for q in g.indices:
            for ch in (depolarizing(1e-3), amplitude_damping(5e-4)):
                ops += dm_ops_for_gate(ID(2, 0.0, [q], nm=ch), n)
    return ops


def test_channels_and_gate_halves_keep_the_trace_projectors_do_not():
    n = 3
    ops = _noisy_ops(n, 1, 4)
    assert all(trace_preserving(o) for o in ops)
    proj = dm_ops_for_gate(Reset([1], "0"), n)
    assert len(proj) == 2 and not any(trace_preserving(o) for o in proj)


def test_whole_cuts_of_fused_blocks_pair_every_gate():
    n = 7
    ops = _noisy_ops(n, 6, 11)
    plan = compile_ops(ops, 2 * n, mode="fused", width=6, device_fusion=True)
    assert plan.trace_kept
    dense = [s for s in plan.steps if isinstance(s, DenseStep)]
    assert any(s.whole for s in dense)
    # replay the block membership: at each cut marked whole every pair has both halves applied
    applied = set()
    for s in dense:
        for mi, _ in plan.matrices[s.mat].entries:
            applied.add(mi)
        pairs = {}
        for i in applied:
            p = ops[i].pair
            if p is not None:
                pairs[p] = pairs.get(p, 0) + 1
        assert s.whole == all(c == 2 for c in pairs.values())
    assert dense[-1].whole


def test_whole_cuts_toggle_on_half_gates():
    ops = _noisy_ops(3, 1, 2)
    flags = whole_cuts(ops, [[i] for i in range(len(ops))])
    for i, o in enumerate(ops):
        if o.pair is not None and (i + 1 < len(ops) and ops[i + 1].pair == o.pair):
            assert not flags[i]  # only the ket half applied
    assert flags[-1]


def test_trace_kept_only_when_every_loss_is_renormalised():
    n = 7
    ops = _noisy_ops(n, 2, 3)
    assert compile_ops(ops + dm_ops_for_gate(Reset([2], "0"), n) + [None], 2 * n, mode="fused", width=6,
                       device_fusion=True).trace_kept
    assert not compile_ops(ops + dm_ops_for_gate(Reset([2], "0"), n), 2 * n, mode="fused", width=6,
                           device_fusion=True).trace_kept


class _Recorder:
    def __init__(self, dense_impl=2):
        self.calls = []
        self.dense_impl = dense_impl

    def __getattr__(self, name):
        def call(*args):
            self.calls.append((name, args))
            return self.dense_impl if name == "qgb_get_dense_impl" else 0
        return call


def _run(monkeypatch, plan, dense_impl=2, chain=True):
    rec = _Recorder(dense_impl)
    monkeypatch.setattr(_lib, "_lib", rec)
    monkeypatch.setattr(_lib, "require_cuda", lambda t: None)
    monkeypatch.setattr(_lib, "stream_ptr", lambda device=None: 0)
    ex = engine.Executor(plan, torch.complex64, "cpu", mode_normalize="dm")
    monkeypatch.setattr(ex, "normalize", lambda state, batch=1, stride=0: 3)
    engine.set_trace_chain(chain)
    try:
        ex.run(torch.zeros(2 ** plan.nbits, dtype=torch.complex64))
    finally:
        engine.set_trace_chain(True)
    keep = ("qgb_op_action", "qgb_op_action_scaled", "qgb_dm_trace_factor", "qgb_op_action_unitary_chain")
    return [(name, args) for name, args in rec.calls if name in keep]


def _plan():
    m6, m2 = np.eye(64, dtype=np.complex128), np.eye(4, dtype=np.complex128)
    p = Plan(nbits=14, trace_kept=True)
    a, b = p.add_matrix(m6), p.add_matrix(m2)
    D = DenseStep
    p.steps = [D(list(range(6)), a, True, False), D(list(range(6, 12)), a, False, False), D([0, 1], b, False, True),
               D(list(range(6)), a, False, False), D(list(range(6)), a, False, False), D(list(range(6)), a, True, True),
               D(list(range(6)), a, False, False), D([2, 3], b, False, True), NormalizeStep(),
               D(list(range(6)), a, False, True)]
    return p


def test_executor_trace_chain_order(monkeypatch):
    calls = _run(monkeypatch, _plan())
    seq = [(n, a[4]) if n == "qgb_dm_trace_factor" else (n,) for n, a in calls]
    assert seq == [
        ("qgb_dm_trace_factor", 1),  # reference at the start
        ("qgb_op_action",), ("qgb_op_action",), ("qgb_op_action",),  # tc, tc, CUDA-core 2-bit block (whole)
        ("qgb_op_action",), ("qgb_op_action",),  # tc passes 3 and 4, cuts not whole
        ("qgb_op_action",),  # tc pass 5, whole cut: 4 or more passes since the reference
        ("qgb_dm_trace_factor", 0),
        ("qgb_op_action_scaled",),  # the next tensor-core pass takes the factor
        ("qgb_op_action",),
        ("qgb_dm_trace_factor", 1),  # after renormalisation: a new reference
        ("qgb_op_action",),
    ]
    # the scaled pass reads chain[1]: 8 bytes past the chain buffer the factor kernel writes
    buf = calls[0][1][3]
    scaled = [a for n, a in calls if n == "qgb_op_action_scaled"][0]
    assert scaled[6] == buf + 8
    # no norm chain for density matrices under the trace chain
    assert not any(n == "qgb_op_action_unitary_chain" for n, _ in calls)


def test_executor_trace_chain_off_on_cuda_cores_or_when_disabled(monkeypatch):
    for impl, chain in ((0, True), (2, False)):
        names = [n for n, _ in _run(monkeypatch, _plan(), dense_impl=impl, chain=chain)]
        assert "qgb_dm_trace_factor" not in names and "qgb_op_action_scaled" not in names
    p = _plan()
    p.trace_kept = False
    names = [n for n, _ in _run(monkeypatch, p)]
    assert "qgb_dm_trace_factor" not in names


def test_superoperator_cache_gives_the_same_ops_read_only():
    """Noise carriers of one op sequence share a superoperator built once per
    (noise model, time, decoupling flag, site order): the ops equal the ones
    built carrier by carrier, and the shared matrix cannot be written."""
    from qaravan_gb300.gates import ID
    from qaravan_gb300.noise import QubitNoise, depolarizing
    n = 4
    chans = [depolarizing(0.02), QubitNoise(80.0, 60.0, 1.0, 5.0)]
    from qaravan_gb300.noise import PauliNoise
    carriers = [ID(2, 1.0, [q], nm=ch) for q in range(n) for ch in chans] + \
               [ID(2, 5.0, [q], nm=chans[1]) for q in range(n)] + \
               [ID(2, 1.0, [3, 1], nm=PauliNoise(["ii", "xz", "yy"], [0.97, 0.02, 0.01]))]  # unsorted sites
    cache: dict = {}
    shared = [o for g in carriers for o in dm_ops_for_gate(g, n, cache)]
    fresh = [o for g in carriers for o in dm_ops_for_gate(g, n)]
    assert len(shared) == len(fresh)
    for a, b in zip(shared, fresh):
        assert a.bits == b.bits and a.kind == b.kind == "channel"
        assert np.array_equal(a.matrix, b.matrix)
    assert len(cache) == 4  # depolarising, T1/T2 at two gate times, the two-site Pauli channel
    with pytest.raises(ValueError):
        shared[0].matrix[0, 0] = 0.0
