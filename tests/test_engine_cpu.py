"""Host logic of the plan executor without a GPU: which C entry each step
takes and the numbering of the norm chain (consecutive unitary blocks of one
state form a chain; any other step restarts it; batches use the row-wise
entry). The library is replaced by a recorder, so no kernel runs."""
import numpy as np
import torch

from qaravan_gb300 import _lib, engine
from qaravan_gb300.compiler import DenseStep, NormalizeStep, Plan, SweepStep


class _Recorder:
    def __init__(self):
        self.calls = []

    def __getattr__(self, name):
        def call(*args):
            self.calls.append((name, args))
            return 0
        return call


def _plan():
    u = np.eye(4, dtype=np.complex128)
    p = Plan(nbits=14)
    m = p.add_matrix(u)
    p.steps = [DenseStep([0, 1], m, True), DenseStep([2, 3], m, True), DenseStep([4, 5], m, True),
               SweepStep(10, [], [((0, 1), m)]), DenseStep([0, 1], m, True), DenseStep([2, 3], m, False),
               DenseStep([4, 5], m, True), DenseStep([6, 7], m, True), NormalizeStep(), DenseStep([0, 1], m, True)]
    return p


def _run(monkeypatch, mode, batch=1):
    rec = _Recorder()
    monkeypatch.setattr(_lib, "_lib", rec)
    monkeypatch.setattr(_lib, "require_cuda", lambda t: None)
    monkeypatch.setattr(_lib, "stream_ptr", lambda device=None: 0)
    ex = engine.Executor(_plan(), torch.complex64, "cpu")
    monkeypatch.setattr(ex, "normalize", lambda state, batch=1, stride=0: 3)
    engine.set_norm_restore(mode)
    try:
        state = torch.zeros(batch * 2 ** 14, dtype=torch.complex64)
        ex.run(state, batch=batch, stride=2 ** 14 if batch > 1 else 0)
    finally:
        engine.set_norm_restore("chain")
    return [(name, args) for name, args in rec.calls if name.startswith("qgb_op_action") or name == "qgb_apply_sweep"]


def test_norm_chain_links_restart_after_other_steps(monkeypatch):
    calls = _run(monkeypatch, "chain")
    names = [c[0] for c in calls]
    assert names == ["qgb_op_action_unitary_chain"] * 3 + ["qgb_apply_sweep", "qgb_op_action_unitary_chain",
                                                            "qgb_op_action"] + ["qgb_op_action_unitary_chain"] * 3
    links = [args[10] for name, args in calls if name == "qgb_op_action_unitary_chain"]
    # 0 1 2 | sweep | 0 | plain (non-unitary) | 0 1 | normalize | 0
    assert links == [0, 1, 2, 0, 0, 1, 0]
    bufs = {args[9] for name, args in calls if name == "qgb_op_action_unitary_chain"}
    assert len(bufs) == 1  # one chain buffer per executor


def test_row_mode_off_mode_and_batches(monkeypatch):
    names = [c[0] for c in _run(monkeypatch, "row")]
    assert "qgb_op_action_unitary_chain" not in names and names.count("qgb_op_action_unitary") == 7
    names = [c[0] for c in _run(monkeypatch, "off")]
    assert names.count("qgb_op_action") == 8
    names = [c[0] for c in _run(monkeypatch, "chain", batch=3)]  # the chain follows one state: batches restore rows
    assert "qgb_op_action_unitary_chain" not in names and names.count("qgb_op_action_unitary") == 7
