"""The replica path of bench.py (one process per GPU, no data-path collective)
with world_size 2 on the gloo backend: barrier, the max-over-ranks timing, and
the reference arm printing from rank 0 only."""
import json
import os
import socket
import subprocess
import sys


from conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker_script():
    return r'''
import os, sys, json
sys.path.insert(0, os.environ["QGB_ROOT"])
import bench
rank, world = bench.dist_init()
bench.barrier(world)
t = bench.max_over_ranks(float(rank + 1) * 0.25, world)
print(json.dumps({"rank": rank, "world": world, "max": t}), flush=True)
import torch.distributed as dist
dist.destroy_process_group()
'''


def _run_ranks(code, extra_env=None, args=()):
    port = _free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port), QGB_ROOT=ROOT, CUDA_VISIBLE_DEVICES="")
        env.update(extra_env or {})
        procs.append(subprocess.Popen([sys.executable, *(["-c", code] if code else []), *args], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, cwd=ROOT))
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=240)
        assert p.returncode == 0, err[-2000:]
        outs.append(out)
    return outs


def test_barrier_and_max_over_ranks_on_gloo():
    outs = _run_ranks(_worker_script())
    recs = [json.loads(o.strip().splitlines()[-1]) for o in outs]
    assert sorted(r["rank"] for r in recs) == [0, 1]
    assert all(r["world"] == 2 and r["max"] == 0.5 for r in recs)  # both ranks see the slowest rank's time


def test_reference_arm_prints_from_rank_zero_only():
    outs = _run_ranks(None, args=[os.path.join(ROOT, "bench.py"), "--impl", "reference", "--qubits", "12",
                                  "--steps", "1", "--warmup", "1", "--gpus", "2"])
    lines = [[ln for ln in o.splitlines() if ln.startswith("{")] for o in outs]
    assert len(lines[0]) == 1 and lines[1] == []
    rec = json.loads(lines[0][0])
    assert rec["impl"] == "reference" and rec["value"] > 0 and rec["cpu_baseline"]["kind"] in ("port", "reference")


def test_cpu_baseline_is_the_reference_arm_in_a_child_process():
    """The bench line's cpu_baseline comes from the reference arm run as a fresh
    process (the same measurement as `bench.py --impl reference`), plus the numpy
    complex128 and 12-qubit figures measured in place."""
    import bench
    gates = bench.workload_gates(14, 1)
    out = bench.cpu_baseline(gates, 14, 1)
    assert out["kind"] == "port" and out["unit"] == "gates/s" and out["value"] > 0 and out["cores"] >= 1
    assert "child process" in out["sample"]
    assert out["numpy_c128"]["gates_per_s"] > 0 and out["config1_12q_depth20_c128"]["gates"] == 460
