"""Benchmark: gates/s of a 28-qubit depth-20 Haar brickwork circuit on one GB300.

Workload (the reference's large plain-statevector configuration): 28 qubits
on an open chain, 20 depth units of seeded Haar SU(2) on every site followed
by Haar SU(4) on the even then odd nearest-neighbour pairs = 1100 gates,
complex64 state of 2 GiB (larger than the 129 MB L2, so no flush is needed
between steps). One step = initialise |0...0> and apply the whole circuit.

* ``value``: gates/s with the state resident in HBM (device-timed, CUDA events).
* ``e2e``: the same metric through the public API with host inputs: build
  ``StatevectorSim`` from host NumPy gate matrices (compile + pinned H2D of
  the fused matrices), run, and read one float64 observable back (D2H).
* ``roofline``: the dominant kernel (the fused tile sweep) -- algorithmic
  bytes per launch (one read + one write of the 2^28 x 8 B state) over its
  mean CUDA-event duration, against the measured HBM copy bandwidth.
* ``cpu_baseline``: the reference's algorithm (``op_action`` = ncon via
  tensordot + transpose, complex128, ``oracle/``) on a bounded sample of the
  same circuit's gates on the host cores.

``--impl reference`` times that CPU implementation alone (the reference is
pure Python; its algorithm is run through the oracle with all host threads).
Multi-GPU: replicas only (each rank runs its own copy, no collective).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "gates/sec & HBM GB/s vs peak at 28q; adjoint grads/sec vs autograd, same GPU"
N_QUBITS, DEPTH, SEED = 28, 20, 2028


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _profile_traffic():
    """dram bytes per sweep launch from the committed ncu summary (None if absent)."""
    path = os.path.join(ROOT, "profiles", "sweep_kernel_28q.txt")
    try:
        for line in open(path):
            if line.startswith("traffic_bytes_per_full_launch:"):
                return float(line.split(":")[1])
    except OSError:
        pass
    return None


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def workload_gates(n=N_QUBITS, depth=DEPTH, seed=SEED):
    from qaravan_gb300 import workloads
    return workloads.brickwork_gates(n, depth, seed)


def cpu_baseline(gates, n, budget_s=12.0, min_gates=2, max_gates=8):
    """Reference algorithm (oracle op_action, complex128) on a bounded prefix of the circuit."""
    import torch
    from oracle import ref
    threads = os.cpu_count() or 1
    torch.set_num_threads(threads)
    state = ref.initial_sv(n)
    done, t0 = 0, time.perf_counter()
    for g in gates[:max_gates]:
        state = ref.op_action(g.matrix, g.indices, state)
        done += 1
        if done >= min_gates and time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    del state
    return {"value": done / dt, "unit": "gates/s", "cores": threads, "kind": "port",
            "sample": f"first {done} gates ({sum(len(g.indices) == 1 for g in gates[:done])} SU(2), "
                      f"{sum(len(g.indices) == 2 for g in gates[:done])} SU(4)) of the {n}-qubit circuit, "
                      f"complex128 tensordot+transpose (reference op_action via oracle/), {dt:.1f} s"}


def dist_init():
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
    return rank, world


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gpu_arm(args):
    import torch
    from qaravan_gb300 import build as qbuild
    qbuild.build()
    from qaravan_gb300 import StatevectorSim, _lib
    from qaravan_gb300.circuits import Circuit
    from qaravan_gb300.compiler import plan_flops

    rank, world = dist_init()
    n = args.qubits
    gates = workload_gates(n, args.depth)
    circ = Circuit(gates, n=n)
    dtype = torch.complex64 if args.dtype == "c64" else torch.complex128
    sim = StatevectorSim(circ, dtype=dtype, mode=args.mode, fusion_width=args.width, tile_bits=args.tile,
                         low_bits=args.low)
    ex = sim.compile()
    state = torch.empty(2 ** n, dtype=dtype, device="cuda")
    L = _lib.lib()
    code = _lib.dtype_code(dtype)

    def step(events=None):
        _lib.check(L.qgb_init_basis(state.data_ptr(), code, n, 0, 1, 0, _lib.stream_ptr()), "init")
        ex.run(state, events=events)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    barrier(world)
    ev_steps = []
    with ClockSampler(torch.cuda.current_device()) as clocks:
        torch.cuda.synchronize()
        start = torch.cuda.Event(enable_timing=True)
        stop = torch.cuda.Event(enable_timing=True)
        start.record()
        for _ in range(args.steps):
            evs = []
            step(evs)
            ev_steps.append(evs)
        stop.record()
        torch.cuda.synchronize()
    barrier(world)
    ms_total = start.elapsed_time(stop)
    ms_total = max_over_ranks(ms_total, world)
    ms_step = ms_total / args.steps
    gates_per_step = ex.plan.n_gates
    value = world * gates_per_step * args.steps / (ms_total / 1e3)

    # dominant kernel: per-launch durations from the events recorded around each launch
    durs = {}
    for evs in ev_steps:
        for kind, a, b in evs:
            durs.setdefault(kind, []).append(a.elapsed_time(b))
    dom = max(durs, key=lambda k: sum(durs[k])) if durs else None
    itemsize = 8 if dtype == torch.complex64 else 16
    alg_bytes = 2 * (2 ** n) * itemsize
    peak, peak_kind = _peaks()
    roof = None
    if dom:
        mean_ms = statistics.mean(durs[dom])
        achieved = alg_bytes / (mean_ms / 1e3) / 1e9
        tr = _profile_traffic() if (n == N_QUBITS and dtype == torch.complex64 and args.mode == "sweep") else None
        roof = {"bound": "hbm", "kernel": f"qgb::{'sweep' if dom == 'sweep' else 'dense_reg'}_kernel",
                "achieved": round(achieved, 1), "peak": peak, "peak_source": f"hbm_gbs of {peak_kind}",
                "unit": "GB/s", "frac": round(achieved / peak, 4), "traffic": tr,
                "alg_bytes_per_launch": alg_bytes, "mean_launch_ms": round(mean_ms, 4),
                "launches_per_step": len(durs[dom]) // args.steps,
                "share_of_step": round(sum(durs[dom]) / ms_total, 4) if world == 1 else None}
    passes, flops_per_amp = plan_flops(ex.plan)

    # end to end through the public API with host inputs
    e2e = None
    if not args.no_e2e:
        host_circ = Circuit(gates, n=n)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        h2d = 0
        for _ in range(args.e2e_steps):
            s2 = StatevectorSim(host_circ, dtype=dtype, mode=args.mode, fusion_width=args.width,
                                tile_bits=args.tile, low_bits=args.low)
            s2.run()
            h2d = s2._exec.h2d_bytes
            r = s2.pauli_expectation("z" + "i" * (n - 1))
            del s2
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        dt = max_over_ranks(dt, world)
        e2e = {"value": round(world * gates_per_step * args.e2e_steps / dt, 2), "unit": "gates/s",
               "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": 8,
               "note": "StatevectorSim(host circuit).run() incl. compile + pinned H2D of fused matrices, "
                       "then pauli_expectation('zi...i').item()", "check_value": r}

    if rank != 0:
        return
    cpu = None if args.no_cpu else cpu_baseline(gates, n, budget_s=args.cpu_budget)
    launches = args.steps * (1 + ex.launches)
    out = {
        "metric": METRIC, "value": round(value, 2), "unit": "gates/s", "n_gates": gates_per_step,
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_step, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c64" if dtype == torch.complex64 else "c128", "data": "synthetic (seeded Haar brickwork)",
        "config": {"workload": f"{n}-qubit open-chain Haar brickwork, depth {args.depth} "
                               f"({gates_per_step} gates), {'complex64' if dtype == torch.complex64 else 'complex128'}",
                   "qubits": n, "depth": args.depth, "seed": SEED, "mode": args.mode, "fusion_width": args.width,
                   "tile_bits": args.tile, "hbm_passes_per_step": passes, "flops_per_amp_per_step": flops_per_amp,
                   "l2": "state (2^n x itemsize) larger than L2; no flush needed",
                   "parallelism": f"replicas x{world}"},
        "hbm_gbs_effective": round(passes * alg_bytes / (ms_step / 1e3) / 1e9, 1),
        "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks.summary(),
        "gpu_launches": launches,
    }
    print(json.dumps(out), flush=True)


def reference_arm(args):
    """The reference's CPU algorithm (complex128 op_action via tensordot), all host threads."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    n = args.qubits
    gates = workload_gates(n, args.depth)
    from oracle import ref
    import torch
    threads = os.cpu_count() or 1
    torch.set_num_threads(threads)
    sample = gates[: args.ref_gates]
    state = ref.initial_sv(n)
    for g in sample[:1] * args.warmup:
        state = ref.op_action(g.matrix, g.indices, state)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        for g in sample:
            state = ref.op_action(g.matrix, g.indices, state)
        times.append(time.perf_counter() - t0)
    total = sum(times)
    value = args.steps * len(sample) / total
    cpu = {"value": round(value, 4), "unit": "gates/s", "cores": threads, "kind": "port",
           "sample": f"{len(sample)} gates (SU(2) + SU(4)) of the {n}-qubit brickwork per step, complex128, "
                     f"reference op_action restated in oracle/"}
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": "gates/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * total / args.steps, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
        "data": "synthetic (seeded Haar brickwork)",
        "config": {"workload": f"{n}-qubit open-chain Haar brickwork, depth {args.depth}", "qubits": n,
                   "depth": args.depth, "seed": SEED},
        "cpu_baseline": cpu, "e2e": {"value": round(value, 4), "unit": "gates/s", "h2d_bytes_per_step": 0,
                                     "d2h_bytes_per_step": 0}}), flush=True)


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--qubits", type=int, default=N_QUBITS)
    p.add_argument("--depth", type=int, default=DEPTH)
    p.add_argument("--dtype", default="c64", choices=["c64", "c128"])
    p.add_argument("--mode", default="sweep", choices=["gate", "fused", "sweep"])
    p.add_argument("--width", type=int, default=4)
    p.add_argument("--tile", type=int, default=14)
    p.add_argument("--low", type=int, default=None)
    p.add_argument("--e2e-steps", type=int, default=3)
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--cpu-budget", type=float, default=12.0)
    p.add_argument("--ref-gates", type=int, default=2)
    args = p.parse_args()
    if args.impl == "reference":
        reference_arm(args)
    else:
        gpu_arm(args)


if __name__ == "__main__":
    main()
