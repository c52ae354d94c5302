"""Host logic of the persistent trajectory launch without a GPU: the tile-sweep
planner (every gate exactly once, inside its sweep's tile, never moved past a
gate it shares a site with) and the autotuner's decision rule and cache."""
import json

import numpy as np
import pytest
import torch

from qaravan_gb300 import autotune, workloads
from qaravan_gb300.trajectories import TRAJ_MAX_OPS, plan_traj_sweeps


def _check_plan(bits, n, tile, low_min):
    plan = plan_traj_sweeps(bits, n, tile, low_min)
    seen = [g for _, _, taken in plan for g in taken]
    assert sorted(seen) == list(range(len(bits)))
    order = {g: (s, i) for s, (_, _, taken) in enumerate(plan) for i, g in enumerate(taken)}
    for L, high, taken in plan:
        m = min(tile, n)
        assert L + len(high) == m and len(taken) <= TRAJ_MAX_OPS
        assert high == sorted(high) and all(h >= L for h in high)
        tile_bits = set(range(L)) | set(high)
        for g in taken:
            assert set(bits[g]) <= tile_bits
    # gates sharing a bit keep their order
    for a in range(len(bits)):
        for b in range(a + 1, len(bits)):
            if set(bits[a]) & set(bits[b]):
                assert order[a] < order[b]
    return plan


@pytest.mark.parametrize("n,tile,low_min", [(20, 13, 5), (20, 12, 5), (20, 14, 5), (10, 6, 5), (10, 5, 4),
                                             (6, 13, 5), (24, 11, 4)])
def test_plan_of_tfi_trotter_and_brickwork(n, tile, low_min):
    for circ_gates in (workloads.tfi_trotter_circuit(n, 0.05, 3).gate_list, workloads.brickwork_gates(n, 2, 1)):
        bits = [[n - 1 - int(q) for q in g.indices] for g in circ_gates]
        plan = _check_plan(bits, n, tile, low_min)
        if n <= tile:
            assert len(plan) == -(-len(bits) // TRAJ_MAX_OPS)


def test_tfi_20_qubits_takes_few_sweeps_per_step():
    n, steps = 20, 40
    gl = workloads.tfi_trotter_circuit(n, 0.05, steps).gate_list
    bits = [[n - 1 - int(q) for q in g.indices] for g in gl]
    plan = plan_traj_sweeps(bits, n, 13, 5)
    assert len(plan) <= 3 * steps  # versus 39 gates per step gate by gate


def test_select_takes_the_fastest_measured_candidate():
    times = {"a": 3.0, "b": 1.0, "c": None, "d": 1.0}
    best, timings = autotune.select(["a", "b", "c", "d"], times.get)
    assert best == "b"  # ties keep the earlier candidate; a candidate that cannot run is skipped
    assert [c for c, _ in timings] == ["a", "b", "d"]
    with pytest.raises(RuntimeError):
        autotune.select(["c"], times.get)


def test_tuning_caches_and_choose_reads_the_cache(tmp_path, monkeypatch):
    monkeypatch.setenv("QGB_AUTOTUNE_CACHE", str(tmp_path / "at.json"))
    monkeypatch.delenv("QGB_AUTOTUNE", raising=False)
    fake = {("fused", 5, 14): 0.5, ("fused", 6, 14): 0.9}
    best, _ = autotune.tune_sv(22, torch.complex64, measure=lambda c: fake.get(tuple(c), 2.0))
    assert best == ("fused", 5, 14)
    assert autotune.choose_sv(22, torch.complex64) == ("fused", 5, 14)
    data = json.loads((tmp_path / "at.json").read_text())
    assert data["sv:c64:22"]["choice"] == ["fused", 5, 14]
    best, _ = autotune.tune_traj(20, torch.complex64, measure=lambda t: {12: 0.2}.get(t, 0.4))
    assert best == 12 and autotune.choose_traj(20, torch.complex64) == 12
    best, _ = autotune.tune(18, torch.complex128, measure=lambda c: 1.0 if c != (13, 3) else 0.1)
    assert best == (13, 3) and autotune.choose(18, torch.complex128) == (13, 3)


def test_choose_tunes_on_first_sight_only_when_enabled(tmp_path, monkeypatch):
    monkeypatch.setenv("QGB_AUTOTUNE_CACHE", str(tmp_path / "at.json"))
    calls = []

    def fake_tune(n, dtype, **kw):
        calls.append(n)
        autotune.store("traj", n, dtype, 11, [(11, 0.1)])
        return 11, [(11, 0.1)]
    monkeypatch.setattr(autotune, "tune_traj", fake_tune)
    monkeypatch.delenv("QGB_AUTOTUNE", raising=False)
    assert autotune.choose_traj(20, torch.complex64) == 13  # default, nothing measured
    assert calls == []
    monkeypatch.setenv("QGB_AUTOTUNE", "1")
    assert autotune.choose_traj(20, torch.complex64) == 11
    assert autotune.choose_traj(20, torch.complex64) == 11  # cached: measured once
    assert calls == [20]


@pytest.mark.parametrize("m,rmax", [(13, 4), (12, 3), (3, 4), (2, 3), (1, 4)])
def test_runs_cover_every_gate_within_r_bits_in_a_valid_order(m, rmax):
    from qaravan_gb300.trajectories import plan_runs
    rng = np.random.default_rng(m * 10 + rmax)
    pos = []
    for _ in range(60):
        if m >= 2 and rng.random() < 0.5:
            a, b = rng.choice(m, size=2, replace=False)
            pos.append([int(a), int(b)])
        else:
            pos.append([int(rng.integers(m))])
    runs = plan_runs(pos, m, rmax)
    R = min(rmax, m)
    order = [i for _, members in runs for i in members]
    assert sorted(order) == list(range(len(pos)))
    where = {i: k for k, i in enumerate(order)}
    for bits, members in runs:
        assert len(bits) == R and len(set(bits)) == R and all(0 <= b < m for b in bits)
        for i in members:
            assert set(pos[i]) <= set(bits)
    for a in range(len(pos)):
        for b in range(a + 1, len(pos)):
            if set(pos[a]) & set(pos[b]):
                assert where[a] < where[b]


def test_tfi_runs_hold_several_gates():
    from qaravan_gb300.trajectories import plan_runs
    n = 20
    gl = workloads.tfi_trotter_circuit(n, 0.05, 4).gate_list
    bits = [[n - 1 - int(q) for q in g.indices] for g in gl]
    plan = plan_traj_sweeps(bits, n, 13, 5)
    nruns = 0
    for L, high, taken in plan:
        tpos = {b: b for b in range(L)}
        for h, b in enumerate(high):
            tpos[b] = L + h
        nruns += len(plan_runs([[tpos[b] for b in bits[g]] for g in taken], L + len(high), 4))
    assert nruns * 2.5 < len(gl)  # several gates per shared-memory pass
