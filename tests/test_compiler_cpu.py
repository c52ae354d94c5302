"""The fusion compiler and sweep planner preserve the circuit's action
(checked on the CPU by executing compiled plans with the oracle's op_action)."""
import numpy as np
import pytest

from oracle import ref
from qaravan_gb300 import compiler, workloads
from qaravan_gb300.density_matrix import dm_ops_for_gate
from qaravan_gb300.statevector import gates_to_ops


def run_plan_numpy(plan, vec):
    """Execute a Plan with the oracle's op_action (sites = nbits-1-bit)."""
    nb = plan.nbits
    v = vec.copy()
    for s in plan.steps:
        if isinstance(s, compiler.DenseStep):
            v = ref.op_action(plan.matrices[s.mat], [nb - 1 - b for b in s.bits], v)
        elif isinstance(s, compiler.SweepStep):
            tile_to_bit = list(range(s.low_bits)) + list(s.high_bits)
            for pos, mi in s.ops:
                bits = [tile_to_bit[p] for p in pos]
                v = ref.op_action(plan.matrices[mi], [nb - 1 - b for b in bits], v)
        else:
            v = v / np.linalg.norm(v)
    return v


@pytest.mark.parametrize("mode,width,tile", [("gate", 2, 0), ("fused", 2, 0), ("fused", 4, 0), ("fused", 6, 0),
                                             ("sweep", 2, 8), ("sweep", 3, 9), ("sweep", 4, 10), ("sweep", 5, 8)])
def test_plans_match_oracle(mode, width, tile):
    n = 10
    gates = workloads.brickwork_gates(n, 4, 3)
    ops = gates_to_ops(gates, n)
    plan = compiler.compile_ops(ops, n, mode=mode, width=width, tile_bits=tile, low_bits=3)
    v0 = np.zeros(2 ** n, complex)
    v0[0] = 1
    out = run_plan_numpy(plan, v0)
    exp = ref.run_sv(gates, n)
    assert np.max(np.abs(out - exp)) < 1e-12
    if mode == "sweep":
        for s in plan.steps:
            assert s.low_bits + len(s.high_bits) <= tile


def test_fusion_absorbs_single_qubit_layers():
    n = 12
    ops = gates_to_ops(workloads.brickwork_gates(n, 5, 1), n)
    blocks = compiler.fuse(ops, 2)
    assert len(blocks) == 5 * (n - 1)  # every SU(2) folded into an SU(4)


def test_reset_segments_and_unsorted_gates():
    from conftest import golden
    from gateio import unpack_gates
    z = golden("sv_mixed7.npz")
    gates = unpack_gates(z)
    n = int(z["n"])
    seq = [g for layer in ref.construct_layers(gates) for g in layer]
    ops = gates_to_ops(seq, n)
    assert any(o is None for o in ops)
    for mode, w in (("gate", 2), ("fused", 4), ("sweep", 4)):
        plan = compiler.compile_ops(ops, n, mode=mode, width=w, tile_bits=7)
        v0 = ref.initial_sv(n, str(z["init"])).reshape(-1)
        assert np.max(np.abs(run_plan_numpy(plan, v0) - z["sv"])) < 1e-12


def test_dm_op_lowering_matches_reference_superops():
    """Gate -> (ket M, bra conj M) and channel superops, incl. unsorted indices."""
    from conftest import golden
    from gateio import unpack_gates
    z = golden("dm_mixed5.npz")
    n = int(z["n"])
    gates = unpack_gates(z)
    offs = z["superop_offs"]
    ops = []
    for i, g in enumerate(gates):
        if z["is_noise"][i]:
            s = z["superops"][offs[i]:offs[i + 1]].reshape(4 ** g.span, 4 ** g.span)

            class _NM:
                def __init__(self, s):
                    self.s = s

                def get_superop(self, *a):
                    return self.s
            g.name = "ID"
            g.nm = _NM(s)
            g.time, g.dd = 0.0, False
        ops.extend(dm_ops_for_gate(g, n))
    plan = compiler.compile_ops(ops, 2 * n, mode="sweep", width=4, tile_bits=8)
    v0 = np.zeros(4 ** n, complex)
    v0[0] = 1
    out = run_plan_numpy(plan, v0).reshape(2 ** n, 2 ** n)
    assert np.max(np.abs(out - z["dm"])) < 1e-12


@pytest.mark.parametrize("n,depth,dev", [(14, 4, True), (16, 6, False), (17, 5, True)])
def test_tensor_core_sweep_plan_replays_to_the_circuit(n, depth, dev):
    """The "tcsweep" plan (up to four 5-qubit blocks per 13-bit tile, low bits
    >= 4), replayed block by block through the oracle's op_action, gives the
    circuit's state; narrower blocks are widened with identity bits of the tile."""
    from oracle import ref
    from qaravan_gb300 import workloads
    from qaravan_gb300.compiler import Recipe, TcSweepStep, compile_ops, recipe_matrix
    from qaravan_gb300.statevector import gates_to_ops
    gates = workloads.brickwork_gates(n, depth, 40 + n)
    plan = compile_ops(gates_to_ops(gates, n), n, mode="tcsweep", width=5, device_fusion=dev)
    st = ref.initial_sv(n)
    for s in plan.steps:
        assert isinstance(s, TcSweepStep)
        assert s.low_bits >= 4 and s.low_bits + len(s.high_bits) == 13 and 1 <= len(s.blocks) <= 4
        tile = list(range(s.low_bits)) + list(s.high_bits)
        for pos, mi in s.blocks:
            assert len(pos) == 5 and len(set(pos)) == 5 and all(0 <= p < 13 for p in pos)
            m = plan.matrices[mi]
            mat = recipe_matrix(m, plan.op_matrices) if isinstance(m, Recipe) else m
            st = ref.op_action(mat, [n - 1 - tile[p] for p in pos], st)
    assert np.max(np.abs(st.reshape(-1) - ref.run_sv(gates, n).reshape(-1))) < 1e-12


def test_tensor_core_sweep_plan_of_the_28_qubit_brickwork():
    from qaravan_gb300 import workloads
    from qaravan_gb300.compiler import TcSweepStep, compile_ops
    from qaravan_gb300.statevector import gates_to_ops
    n = 28
    plan = compile_ops(gates_to_ops(workloads.brickwork_gates(n, 20, 2028), n), n, mode="tcsweep", width=5,
                       device_fusion=True)
    assert all(isinstance(s, TcSweepStep) for s in plan.steps)
    assert plan.n_sweeps == 35 and sum(len(s.blocks) for s in plan.steps) == 102
    # below 14 qubits (one tile) the mode falls back to one pass per fused block
    small = compile_ops(gates_to_ops(workloads.brickwork_gates(13, 2, 1), 13), 13, mode="tcsweep", width=5)
    assert not any(isinstance(s, TcSweepStep) for s in small.steps)
