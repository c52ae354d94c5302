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
* ``roofline``: the dominant kernel (by default the tensor-core 6-qubit block
  kernel, dense_tc_kernel<6>) -- algorithmic bytes per launch (one read + one
  write of the 2^28 x 8 B state) over its mean CUDA-event duration, against
  the measured HBM copy bandwidth.
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


def _profile_traffic(kernel):
    """DRAM bytes per launch of `kernel` at the full workload, from the committed ncu
    summary profiles/roofline_traffic.txt (lines "<kernel>: <bytes>"; None if absent)."""
    path = os.path.join(ROOT, "profiles", "roofline_traffic.txt")
    try:
        for line in open(path):
            if line.startswith(kernel + ":"):
                return float(line.split(":", 1)[1].split()[0])
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


def depth_unit(gates, n):
    """The circuit's first depth unit: SU(2) on every site, then SU(4) on the even
    and odd nearest-neighbour pairs (n + n - 1 gates, 55 at 28 qubits). Every
    depth unit of the brickwork has this shape, so its time extrapolates to the
    whole circuit by the gate count."""
    return gates[:2 * n - 1]


def _cpu_threads():
    import torch
    threads = os.cpu_count() or 1
    torch.set_num_threads(threads)
    return threads


def cpu_baseline(gates, n, depth, numpy_gates=4):
    """The reference's CPU path on the host cores, all threads: the reference arm
    of this script (its torch backend in complex64 -- the benchmark's own dtype --
    over the circuit's first depth unit, 5 steps of 11 gates after 3 warm-up
    gates) run as a fresh child process, so that this figure and the reference
    arm's line are one measurement on a clean process (timed here, after the GPU
    sections, the same gates ran at about half that rate); beside it the numpy
    complex128 path on a few gates of that unit, and the 12-qubit depth-20
    complex128 circuit run whole (median of 5)."""
    import subprocess
    import sys
    from oracle import ref
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "LOCAL_RANK", "WORLD_SIZE", "MASTER_ADDR",
                                                            "MASTER_PORT", "LOCAL_WORLD_SIZE", "GROUP_RANK")}
    env["CUDA_VISIBLE_DEVICES"] = ""
    cmd = [sys.executable, os.path.abspath(__file__), "--impl", "reference", "--steps", "5", "--warmup", "3",
           "--qubits", str(n), "--depth", str(depth)]
    res = subprocess.run(cmd, env=env, capture_output=True, text=True, timeout=900, check=True)
    line = [ln for ln in res.stdout.splitlines() if ln.startswith("{")][-1]
    out = dict(json.loads(line)["cpu_baseline"])
    out["sample"] += "; measured by the reference arm of this script (--impl reference) in a child process"
    # numpy complex128 (the reference's default backend) on the first gates of the same unit
    unit = depth_unit(gates, n)
    state = ref.initial_sv(n)
    t0 = time.perf_counter()
    for g in unit[:numpy_gates]:
        state = ref.op_action(g.matrix, g.indices, state)
    dt = time.perf_counter() - t0
    del state
    out["numpy_c128"] = {"gates_per_s": round(numpy_gates / dt, 4),
                         "sample": f"first {numpy_gates} gates of the same depth unit, numpy complex128"}
    # configuration 1: 12 qubits, depth 20, complex128, the whole circuit (median of 5 runs)
    from qaravan_gb300 import workloads
    g12 = workloads.brickwork_gates(12, 20, 12)
    times = []
    for _ in range(5):
        t0 = time.perf_counter()
        ref.run_sv(g12, 12)
        times.append(time.perf_counter() - t0)
    out["config1_12q_depth20_c128"] = {"gates": len(g12), "median_s": round(statistics.median(times), 5),
                                       "gates_per_s": round(len(g12) / statistics.median(times), 1)}
    return out


def _event_ms(fn, warmup=1, steps=1):
    import torch
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(steps):
        fn()
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / steps


def fma_peaks():
    """Measured rate of the float32 and float64 FMA pipes (qgb_fma_probe: 8
    independent FMA chains per thread, 8 CTAs of 256 threads per SM), TFLOP/s."""
    import torch
    from qaravan_gb300 import _lib
    L = _lib.lib()
    out = torch.empty(152 * 32, dtype=torch.float64, device="cuda")
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    res = {}
    for name, prec, iters in (("fp32_tflops", 0, 200000), ("fp64_tflops", 1, 20000), ("fp32x2_tflops", 2, 200000)):
        def run():
            _lib.check(L.qgb_fma_probe(prec, iters, 8, out.data_ptr(), _lib.stream_ptr()), "fma_probe")
        ms = _event_ms(run, 1, 3)
        res[name] = round((2 if prec == 2 else 1) * 2 * 8 * iters * 256 * 8 * sms / (ms / 1e3) / 1e12, 2)
    return res


def c128_roofline(plan, n, ms, double_float, peaks):
    """Roofline of a complex128 sweep plan: float64 kernels against the measured
    FP64 FMA rate (8 flops per complex multiply-add); double-float kernels
    against the measured FP32 rate, counting the FP32 pipe's work -- one
    double-float complex multiply-add is 4 real terms of 1 multiply, 3 FMAs and
    8 adds, 48 FP32 instructions, each counted as the probe counts an FMA (2
    flops) -- so that `frac` is the FP32 pipe's busy fraction."""
    from qaravan_gb300.compiler import plan_flops
    flops64 = plan_flops(plan)[1] * 2 ** n  # 8 per complex multiply-add
    out = {"tflops_fp64_equivalent": round(flops64 / (ms / 1e3) / 1e12, 3)}
    if double_float:
        achieved = 2 * 48 * (flops64 / 8) / (ms / 1e3) / 1e12
        out["roofline"] = {"bound": "fp32", "achieved": round(achieved, 2), "peak": peaks["fp32_tflops"],
                           "unit": "TFLOP/s", "frac": round(achieved / peaks["fp32_tflops"], 3),
                           "counting": "48 FP32 instructions per complex multiply-add, 2 flops each",
                           "peak_source": "qgb_fma_probe float32 FMA rate measured in this run"}
    else:
        achieved = flops64 / (ms / 1e3) / 1e12
        out["roofline"] = {"bound": "fp64", "achieved": round(achieved, 3), "peak": peaks["fp64_tflops"],
                           "unit": "TFLOP/s", "frac": round(achieved / peaks["fp64_tflops"], 3),
                           "peak_source": "qgb_fma_probe float64 FMA rate measured in this run"}
    return out


def section_c128(n, gates, steps=3):
    """The benchmark circuit in complex128 through StatevectorSim's default
    complex128 path (double-float tile sweeps), timed over `steps` runs after a
    warm-up, with its roofline; its final state against the float64 kernels'."""
    import torch
    from qaravan_gb300 import StatevectorSim, _lib
    from qaravan_gb300.circuits import Circuit
    L = _lib.lib()
    circ = Circuit(gates, n=n)
    code = _lib.dtype_code(torch.complex128)
    out = {}
    states = {}
    for arith, name in ((1, "double_float"), (0, "float64")):
        _lib.check(L.qgb_set_c128_arith(arith))
        ex = StatevectorSim(circ, dtype=torch.complex128).compile()
        st = torch.empty(2 ** n, dtype=torch.complex128, device="cuda")

        def step():
            _lib.check(L.qgb_init_basis(st.data_ptr(), code, n, 0, 1, 0, _lib.stream_ptr()), "init")
            ex.run(st)
        ms = _event_ms(step, 1, steps if arith == 1 else 1)
        out[name] = {"gates_per_s": round(len(gates) / (ms / 1e3), 1), "ms": round(ms, 2),
                     "hbm_passes": ex.plan.n_sweeps}
        out[name].update(c128_roofline(ex.plan, n, ms, arith == 1, out.setdefault("fma_peaks", fma_peaks())))
        states[name] = st
        del ex
    _lib.check(L.qgb_set_c128_arith(1))
    d = (states["double_float"] - states["float64"]).abs()
    out["max_abs_amplitude_diff_double_float_vs_float64"] = float(d.max().item())
    out["max_abs_amplitude"] = float(states["float64"].abs().max().item())
    out["norm_error_double_float"] = float(abs(torch.linalg.vector_norm(states["double_float"]).item() - 1.0))
    out["speedup_double_float_vs_float64"] = round(out["float64"]["ms"] / out["double_float"]["ms"], 2)
    del states, d
    torch.cuda.empty_cache()
    return out


def section_variants(n, gates):
    """Unfused (one HBM pass per gate), fused dense blocks of width 2..6 on the
    CUDA cores and (4..6) on the tensor cores, shared-memory tile sweeps, and
    the complex128 sweep path, on the same 28-qubit circuit (one timed run each)."""
    import torch
    from qaravan_gb300 import StatevectorSim, _lib, engine
    from qaravan_gb300.circuits import Circuit
    circ = Circuit(gates, n=n)
    out = {}
    L = _lib.lib()
    before = L.qgb_get_dense_impl()
    for name, dtype, mode, width, tile, impl in [
            ("c64_unfused", torch.complex64, "gate", 2, 14, 0),
            ("c64_fused_w2", torch.complex64, "fused", 2, 14, 0),
            ("c64_fused_w4_cudacores", torch.complex64, "fused", 4, 14, 0),
            ("c64_fused_w6_cudacores", torch.complex64, "fused", 6, 14, 0),
            ("c64_fused_w4_tensorcores", torch.complex64, "fused", 4, 14, 2),
            ("c64_fused_w5_tensorcores", torch.complex64, "fused", 5, 14, 2),
            ("c64_fused_w6_tensorcores", torch.complex64, "fused", 6, 14, 2),
            ("c64_fused_w6_tensorcores_row_norm_restore", torch.complex64, "fused", 6, 14, 4),
            ("c64_fused_w6_tensorcores_no_norm_restore", torch.complex64, "fused", 6, 14, 3),
            ("c64_tcsweep_w5", torch.complex64, "tcsweep", 5, 13, 2),
            ("c64_sweep_w3_t12", torch.complex64, "sweep", 3, 12, 0),
            ("c64_sweep_w4_t14", torch.complex64, "sweep", 4, 14, 0),
            ("c128_sweep_w3_t13_fp64", torch.complex128, "sweep", 3, 13, 0),
            ("c128_sweep_w2_t12_df", torch.complex128, "sweep", 2, 12, 1),
            ("c128_sweep_w3_t12_df", torch.complex128, "sweep", 3, 12, 1),
            ("c128_sweep_w3_t13_df", torch.complex128, "sweep", 3, 13, 1),
            ("c128_sweep_w4_t13_df", torch.complex128, "sweep", 4, 13, 1)]:
        try:
            if dtype == torch.complex128:  # impl: the complex128 arithmetic (0 float64, 1 double-float)
                _lib.check(L.qgb_set_c128_arith(impl))
                impl = 0
            _lib.check(L.qgb_set_dense_impl(min(impl, 2)))
            engine.set_norm_restore({3: "off", 4: "row"}.get(impl, "chain"))
            ex = StatevectorSim(circ, dtype=dtype, mode=mode, fusion_width=width, tile_bits=tile).compile()
            st = torch.empty(2 ** n, dtype=dtype, device="cuda")
            code = _lib.dtype_code(dtype)

            def step():
                _lib.check(_lib.lib().qgb_init_basis(st.data_ptr(), code, n, 0, 1, 0, _lib.stream_ptr()), "init")
                ex.run(st)
            ms = _event_ms(step, 1, 1)
            out[name] = {"gates_per_s": round(len(gates) / (ms / 1e3), 1), "ms": round(ms, 2),
                         "hbm_passes": ex.plan.n_sweeps}
            if dtype == torch.complex128:
                out[name].update(c128_roofline(ex.plan, n, ms, name.endswith("_df"),
                                               out.setdefault("fma_peaks", fma_peaks())))
            del st, ex
        except Exception as e:  # a variant that does not fit is reported, not fatal
            out[name] = {"error": str(e)[:200]}
        torch.cuda.empty_cache()
    _lib.check(L.qgb_set_dense_impl(before))
    _lib.check(L.qgb_set_c128_arith(1))
    engine.set_norm_restore("chain")
    return out


def _torch_backend_apply(m, idx, s):
    """The reference torch backend's op_action (tensorQ/statevector_sim.py:124-140:
    the operator's input legs contracted with the state's legs `idx` by one
    tensordot, the output legs moved back into place), restated on torch
    tensors of the state's device."""
    import torch
    n, k = s.ndim, len(idx)
    t = torch.tensordot(m.reshape([2] * 2 * k), s, dims=(list(range(k, 2 * k)), list(idx)))
    order = list(idx) + [a for a in range(n) if a not in idx]
    return t.permute(*[order.index(a) for a in range(n)])


def section_torch_backend_gpu(gates, n):
    """The reference's torch backend on this GPU (StatevectorSim(backend="torch",
    device="cuda"): per gate a complex64 cast and copy of the matrix to the
    device and one permute + tensordot, tensorQ/statevector_sim.py:19-29,50-52,
    124-140), restated here: the circuit's first depth unit at 28 qubits, and
    one brick layer (25 SU(4) gates) at 26 qubits, the reference's own GPU
    benchmark (examples/gpu_acceleration.ipynb, 4.5 s on a T4)."""
    import torch
    out = {}
    for name, nq, gl in (("depth_unit_28q", n, depth_unit(gates, n)),
                         ("brick_layer_26q", 26, [g for g in workload_gates(26, 1)[26:] if len(g.indices) == 2])):
        host = [np.asarray(g.matrix, dtype=np.complex128) for g in gl]

        def run():
            st = torch.zeros([2] * nq, dtype=torch.complex64, device="cuda")
            st.view(-1)[0] = 1
            for m, g in zip(host, gl):
                st = _torch_backend_apply(torch.tensor(m).to("cuda", torch.complex64), g.indices, st)
            return st
        ms = _event_ms(run, 1, 1)
        out[name] = {"qubits": nq, "gates": len(gl), "ms": round(ms, 2),
                     "gates_per_s": round(len(gl) / (ms / 1e3), 1)}
        torch.cuda.empty_cache()
    return out


def section_config1(seed=12):
    """The 12-qubit depth-20 brickwork (460 gates) on the GPU through
    StatevectorSim, complex128 (its parity configuration) and complex64,
    each a whole run (compile cached, state initialisation included)."""
    import torch
    from qaravan_gb300 import StatevectorSim, workloads
    from qaravan_gb300.circuits import Circuit
    gl = workloads.brickwork_gates(12, 20, seed)
    out = {"gates": len(gl)}
    for name, dtype in (("c128", torch.complex128), ("c64", torch.complex64)):
        circ = Circuit(gl, n=12)
        ex = StatevectorSim(circ, dtype=dtype).compile()
        st = torch.empty(2 ** 12, dtype=dtype, device="cuda")
        from qaravan_gb300 import _lib
        code = _lib.dtype_code(dtype)

        def step():
            _lib.check(_lib.lib().qgb_init_basis(st.data_ptr(), code, 12, 0, 1, 0, _lib.stream_ptr()), "init")
            ex.run(st)
        ms = _event_ms(step, 3, 20)
        out[name] = {"ms": round(ms, 4), "gates_per_s": round(len(gl) / (ms / 1e3), 1),
                     "hbm_passes": ex.plan.n_sweeps}
    return out


def _torch_reference_energy(n, layers, params, terms, device):
    """The reference's torch-backend path on this GPU, for the autograd comparison:
    gate matrices by torch.linalg.matrix_exp (core/param_gates.py:51-80), cast to
    complex64 on the device (to_backend, tensorQ/statevector_sim.py:19-24),
    op_action as permute + tensordot (tensorQ/statevector_sim.py:124-140), and
    torch autograd through every op. <H> by Pauli-X flips and Z signs."""
    import torch
    from qaravan_gb300.gates import CNOT
    Y = torch.tensor([[0, -1j], [1j, 0]], dtype=torch.complex128)
    Zm = torch.tensor([[1, 0], [0, -1]], dtype=torch.complex128)
    th = torch.tensor(params, dtype=torch.float64, requires_grad=True)
    st = torch.zeros([2] * n, dtype=torch.complex64, device=device)
    st.view(-1)[0] = 1

    apply = _torch_backend_apply
    for l in range(layers):
        for q in range(n):
            st = apply(torch.linalg.matrix_exp(-1j * th[l, q, 0] * Y).to(device, torch.complex64), [q], st)
            st = apply(torch.linalg.matrix_exp(-1j * th[l, q, 1] * Zm).to(device, torch.complex64), [q], st)
        for q in range(n - 1):
            g = CNOT([q + 1, q], n)
            st = apply(torch.tensor(g.matrix, dtype=torch.complex64, device=device), g.indices, st)
    e = 0
    p = (st.abs() ** 2).to(torch.float64)
    for c, s in terms:
        if 'x' in s:
            q = s.index('x')
            e = e + c * torch.real(torch.vdot(st.reshape(-1), torch.flip(st, dims=[q]).reshape(-1))).to(torch.float64)
        else:
            q = s.index('z')
            sign = torch.ones([2] * n, dtype=torch.float64, device=device)
            idx = [slice(None)] * n
            idx[q] = 1
            sign[tuple(idx)] *= -1
            if s.count('z') == 2:
                idx = [slice(None)] * n
                idx[q + 1] = 1
                sign[tuple(idx)] *= -1
            e = e + c * (p * sign).sum()
    return e, th


def section_adjoint(n=24, layers=40, base_layers=4):
    """Adjoint gradient of the TFI energy of the hardware-efficient ansatz (complex64)
    vs plain forward + torch autograd of the reference's torch path, same GPU."""
    import torch
    from qaravan_gb300 import StatevectorSim, workloads
    from qaravan_gb300.adjoint import adjoint_energy
    from qaravan_gb300.hamiltonians import TFI
    terms = TFI(n, 1, 1).pauli_sum()
    out = {"qubits": n, "layers": layers, "params": 2 * n * layers, "dtype": "c64"}

    def adjoint_run(L):
        th = torch.tensor(workloads.hea_params(n, L, 1), dtype=torch.float64, requires_grad=True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sim = StatevectorSim(workloads.hea_circuit(n, L, th), dtype=torch.complex64)
        e = adjoint_energy(sim, terms)
        e.backward()
        torch.cuda.synchronize()
        return time.perf_counter() - t0, float(e.item()), th.grad.numpy().copy()

    adjoint_run(layers)  # warm-up: plans and caches of this circuit structure, as a training loop has them
    torch.cuda.reset_peak_memory_stats()
    base = torch.cuda.memory_allocated()
    t_full, e_full, _ = adjoint_run(layers)
    out["adjoint_s_per_gradient"] = round(t_full, 4)
    out["adjoint_grads_per_s"] = round(1.0 / t_full, 3)
    out["adjoint_peak_state_multiples"] = round((torch.cuda.max_memory_allocated() - base) / (2 ** n * 8), 2)
    out["energy"] = e_full
    # error of the complex64 gradient against the same adjoint gradient in complex128
    th = torch.tensor(workloads.hea_params(n, layers, 1), dtype=torch.float64, requires_grad=True)
    e128 = adjoint_energy(StatevectorSim(workloads.hea_circuit(n, layers, th), dtype=torch.complex128), terms)
    e128.backward()
    _, _, g64 = adjoint_run(layers)
    g128 = th.grad.numpy()
    out["max_rel_grad_err_vs_c128"] = float(np.abs(g64 - g128).max() / np.abs(g128).max())
    out["energy_err_vs_c128"] = abs(e_full - float(e128.item()))
    # the complex128 gradient against the exact parameter-shift rule on 8 seeded angles:
    # every angle enters one exp(-i theta P) gate, so dE/dtheta = E(theta + pi/4) - E(theta - pi/4)
    base_params = workloads.hea_params(n, layers, 1)
    rng = np.random.default_rng(77)
    shift_err = 0.0
    for flat in rng.choice(base_params.size, size=8, replace=False):
        idx = np.unravel_index(flat, base_params.shape)
        e_pm = []
        for sgn in (1, -1):
            p = base_params.copy()
            p[idx] += sgn * np.pi / 4
            e_pm.append(StatevectorSim(workloads.hea_circuit(n, layers, p), dtype=torch.complex128)
                        .pauli_sum_expectation(terms))
        shift_err = max(shift_err, abs((e_pm[0] - e_pm[1]) - g128[idx]))
    out["c128_grad_max_abs_err_vs_parameter_shift"] = float(shift_err)
    # the reference's torch path at a depth that fits, same depth for the adjoint (both warmed up)
    adjoint_run(base_layers)
    t_adj_b, e_adj_b, g_adj_b = adjoint_run(base_layers)
    params = workloads.hea_params(n, base_layers, 1)
    e_w, _ = _torch_reference_energy(n, 1, params[:1], terms, "cuda")  # warm-up of the torch path
    e_w.backward()
    del e_w
    torch.cuda.synchronize()
    torch.cuda.reset_peak_memory_stats()
    base = torch.cuda.memory_allocated()
    t0 = time.perf_counter()
    e_ref, th = _torch_reference_energy(n, base_layers, params, terms, "cuda")
    e_ref.backward()
    torch.cuda.synchronize()
    t_ref = time.perf_counter() - t0
    peak = torch.cuda.max_memory_allocated() - base
    g_ref = th.grad.numpy()
    free_total = torch.cuda.get_device_properties(0).total_memory
    out["torch_autograd"] = {
        "layers": base_layers, "s_per_gradient": round(t_ref, 4), "peak_gb": round(peak / 1e9, 2),
        "predicted_peak_gb_at_full_depth": round(peak * layers / base_layers / 1e9, 1),
        "fits_at_full_depth": bool(peak * layers / base_layers < free_total)}
    out["adjoint_at_same_depth_s"] = round(t_adj_b, 4)
    out["speedup_vs_autograd_same_depth"] = round(t_ref / t_adj_b, 2)
    out["max_rel_grad_diff_vs_autograd"] = float(abs(g_adj_b - g_ref).max() / max(abs(g_ref).max(), 1e-30))
    out["energy_diff_vs_autograd"] = abs(e_adj_b - float(e_ref.item()))
    return out


def section_adjoint_batch(n=20, layers=40, sets=64, single_sample=8):
    """Energies and angle gradients of 64 parameter sets of the 20-qubit
    hardware-efficient ansatz (TFI energy, complex64) in one batched sweep, vs the
    single-set adjoint run set by set and vs torch autograd through the
    reference's torch path (one set, full depth), same GPU."""
    import torch
    from qaravan_gb300 import StatevectorSim, workloads
    from qaravan_gb300.adjoint import BatchedAnsatz, adjoint_energy
    from qaravan_gb300.hamiltonians import TFI
    terms = TFI(n, 1, 1).pauli_sum()
    ba = BatchedAnsatz.hea(n, layers, dtype=torch.complex64)
    pset = np.stack([workloads.hea_params(n, layers, 100 + s) for s in range(sets)])
    flat = torch.tensor(pset.reshape(sets, -1), dtype=torch.float64, device="cuda")
    ba.energy_and_grad(flat, terms)  # warm-up
    torch.cuda.synchronize()
    torch.cuda.reset_peak_memory_stats()
    base = torch.cuda.memory_allocated()
    t0 = time.perf_counter()
    E, grad = ba.energy_and_grad(flat, terms)
    torch.cuda.synchronize()
    t_batch = time.perf_counter() - t0
    peak = torch.cuda.max_memory_allocated() - base
    E, grad = E.cpu().numpy(), grad.cpu().numpy()
    # the same batch with the forward as one tile-pass op per gate (no fused blocks)
    b_pg = BatchedAnsatz.hea(n, layers, dtype=torch.complex64, fused_width=0)
    b_pg.energy_and_grad(flat, terms)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    _, g_pg = b_pg.energy_and_grad(flat, terms)
    torch.cuda.synchronize()
    t_pg = time.perf_counter() - t0
    g_pg = g_pg.cpu().numpy()
    del b_pg

    def single(s):
        th = torch.tensor(pset[s], dtype=torch.float64, requires_grad=True)
        e = adjoint_energy(StatevectorSim(workloads.hea_circuit(n, layers, th), dtype=torch.complex64), terms)
        e.backward()
        return float(e.item()), th.grad.numpy().reshape(-1).copy()

    single(0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ref = [single(s) for s in range(single_sample)]
    torch.cuda.synchronize()
    t_single = (time.perf_counter() - t0) / single_sample
    gdiff = max(float(np.abs(grad[s] - g).max() / max(np.abs(g).max(), 1e-30)) for s, (_, g) in enumerate(ref))
    ediff = max(abs(E[s] - e) for s, (e, _) in enumerate(ref))
    e_w, _ = _torch_reference_energy(n, 1, pset[0][:1], terms, "cuda")  # warm-up of the torch path
    e_w.backward()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e_ref, th = _torch_reference_energy(n, layers, pset[0], terms, "cuda")
    e_ref.backward()
    torch.cuda.synchronize()
    t_auto = time.perf_counter() - t0
    g_auto = th.grad.numpy().reshape(-1)
    # error of the complex64 batch against the same sweep in complex128 (first 4 sets)
    b128 = BatchedAnsatz.hea(n, layers, dtype=torch.complex128)
    E128, g128 = b128.energy_and_grad(flat[:4], terms)
    E128, g128 = E128.cpu().numpy(), g128.cpu().numpy()
    err64 = max(float(np.abs(grad[s] - g128[s]).max() / np.abs(g128[s]).max()) for s in range(4))
    err64_single = max(float(np.abs(ref[s][1] - g128[s]).max() / np.abs(g128[s]).max()) for s in range(4))
    return {"qubits": n, "layers": layers, "parameter_sets": sets, "params_per_set": 2 * n * layers,
            "gates_per_set": len(ba.gates), "dtype": "c64",
            "batched_s": round(t_batch, 4), "gradients_per_s": round(sets / t_batch, 2),
            "forward": {"fused_blocks": ba._fused["blocks"] if ba._fused else None,
                        "fused_passes": ba._fused["passes"] if ba._fused else None,
                        "per_gate_forward_batched_s": round(t_pg, 4),
                        "max_rel_grad_diff_fused_vs_per_gate": float(np.abs(grad - g_pg).max() / np.abs(g_pg).max())},
            "peak_state_multiples_per_set": round(peak / (sets * 2 ** n * 8), 2),
            "single_set_adjoint_s": round(t_single, 4),
            "speedup_vs_single_set_adjoint": round(t_single * sets / t_batch, 2),
            "torch_autograd_one_set_s": round(t_auto, 4),
            "speedup_vs_torch_autograd": round(t_auto * sets / t_batch, 2),
            "max_rel_grad_diff_vs_single_set": gdiff, "max_energy_diff_vs_single_set": float(ediff),
            "max_rel_grad_err_vs_c128": err64, "max_energy_err_vs_c128": float(np.abs(E[:4] - E128).max()),
            "single_set_max_rel_grad_err_vs_c128": err64_single,
            "max_rel_grad_diff_vs_autograd_set0": float(np.abs(grad[0] - g_auto).max() / np.abs(g_auto).max()),
            "energy_diff_vs_autograd_set0": abs(float(E[0]) - float(e_ref.item()))}


def _is_diagonal(g):
    m = np.asarray(g.matrix)
    return bool(np.all(m == np.diag(np.diag(m))))


def section_trajectories(n=20, ntraj=1024, steps=40):
    """1024 noisy TFI Trotter trajectories (depolarising 1e-3 + amplitude damping 5e-4
    after every gate): the persistent launch (default, one kernel for the whole
    run, in a CUDA graph) and the gate-by-gate path; mean <Z_i>, <Z_i Z_i+1>."""
    import torch
    from qaravan_gb300 import workloads
    from qaravan_gb300.trajectories import TrajectorySim, z_terms
    circ = workloads.tfi_trotter_circuit(n, 0.05, steps)
    peak, peak_kind = _peaks()
    out = {"qubits": n, "trajectories": ntraj}
    means = {}
    for mode in ("persistent", "per_gate"):
        sim = TrajectorySim(circ, ntraj, p_dep=1e-3, gamma=5e-4, seed=2026, mode=mode)
        ms = _event_ms(lambda: sim.run(graph=True), 1, 2)
        mean, _ = sim.mean_expectations(z_terms(n))
        means[mode] = mean.cpu().numpy()
        ng = len(sim.gates)
        r = {"ms_per_run": round(ms, 2), "trajectories_per_s": round(ntraj / (ms / 1e3), 1),
             "trajectory_gates_per_s": round(ntraj * ng / (ms / 1e3), 1), "launches_per_run": sim.launches}
        if mode == "persistent":
            jumps = int(sim.jump_count.sum().item())
            passes = len(sim.sweep_plan)
            # every sweep reads and writes each trajectory's state once; a sweep holding a jump runs twice
            alg = (passes * ntraj + jumps) * 2 * 2 ** n * 8
            r.update({"tile_bits": sim.tile_bits, "sweeps": passes, "jumps": jumps,
                      "hbm_algorithmic_tb": round(alg / 1e12, 3),
                      "hbm_frac": round(alg / (ms / 1e3) / 1e9 / peak, 3),
                      "shared_memory_passes_per_trajectory": ng})
            # the FP32 pipe's share: gate products per amplitude (a dense k-site gate 2^k complex
            # multiply-adds, a diagonal one a complex product: 8 flops each) plus the damping
            # channel per gate site (its K0 scaling and |1> weight: 4 flops per amplitude)
            flops_amp = sum(8 * (1 if _is_diagonal(g) else 2 ** len(g.indices)) + 4 * len(g.indices)
                            for g in circ.gate_list)
            fl = flops_amp * 2 ** n * ntraj
            fp32 = fma_peaks()["fp32_tflops"]
            r["fp32"] = {"flops_per_amplitude": flops_amp, "achieved_tflops": round(fl / (ms / 1e3) / 1e12, 2),
                         "peak_tflops": fp32, "frac": round(fl / (ms / 1e3) / 1e12 / fp32, 3),
                         "peak_source": "qgb_fma_probe float32 FMA rate measured in this run",
                         "counting": "8 flops per complex multiply-add of the gate products, "
                                     "4 per amplitude and site for the damping channel; jumps' re-runs not counted"}
        else:
            alg = ng * 2 * ntraj * 2 ** n * 8
            r.update({"hbm_algorithmic_tb": round(alg / 1e12, 2), "hbm_frac": round(alg / (ms / 1e3) / 1e9 / peak, 3)})
        r["hbm_frac_of"] = f"hbm_gbs of {peak_kind}"
        out[mode] = r
        del sim
        torch.cuda.empty_cache()
    out["gates"] = len(circ.gate_list)
    out["mean_z_first"] = float(means["persistent"][0])
    out["mean_zz_first"] = float(means["persistent"][n])
    # the two unravellings sample the same mixture: their means agree to a few standard errors
    out["max_mean_diff_persistent_vs_per_gate"] = float(np.abs(means["persistent"] - means["per_gate"]).max())
    out["speedup_persistent_vs_per_gate"] = round(out["per_gate"]["ms_per_run"] / out["persistent"]["ms_per_run"], 2)
    return out


def section_dm_batch(count=256, seed=7):
    """256 noisy brickwork density matrices, 6-14 qubits, depth 10-40: the circuits of 8+ qubits in one
    persistent launch, the smaller ones in one batched launch (one CUDA graph)."""
    import torch
    from qaravan_gb300 import DensityMatrixSim, workloads
    from qaravan_gb300.batch import DensityMatrixBatch
    specs = workloads.uneven_dm_specs(count, seed)
    t0 = time.perf_counter()
    circs = [workloads.noisy_brickwork_circuit(n, d, s, p=1e-3) for n, d, s in specs]
    gen_s = time.perf_counter() - t0  # the synthetic input: seeded Haar gates and noise carriers
    t0 = time.perf_counter()
    sims = [DensityMatrixSim(c, dtype=torch.complex64) for c in circs]
    batch = DensityMatrixBatch(sims, dtype=torch.complex64)
    torch.cuda.synchronize()
    compile_s = time.perf_counter() - t0
    ms = _event_ms(lambda: batch.run(graph=True), 1, 1)
    res = batch.results()
    # algorithmic HBM bytes of the large circuits: every pass reads and writes vec(rho)
    # (the persistent launch's first pass of a circuit reads nothing; counted anyway)
    big = [(s, ex) for _, s, ex, *_ in batch.large] + [(s, ex) for _, s, ex, _ in batch.pers]
    passes = sum(ex.plan.n_sweeps for _, ex in big)
    alg = sum(ex.plan.n_sweeps * 2 * 4 ** s.num_sites * 8 for s, ex in big)
    peak, peak_kind = _peaks()
    out = {"circuits": count, "small_batched": len(batch.small), "persistent": len(batch.pers),
           "stream_parallel": len(batch.large), "launches_per_batch": batch.launches,
           "persistent_items": getattr(batch, "persistent_items", 0),
           "circuit_generation_s": round(gen_s, 2), "compile_s": round(compile_s, 2), "ms_per_batch": round(ms, 1),
           "circuits_per_s": round(count / (ms / 1e3), 2),
           "max_trace_error": float(max(abs(r["trace"] - 1) for r in res)),
           "state_gb": round(sum(4 ** n * 8 for n, _, _ in specs) / 1e9, 1),
           "large_passes": passes, "large_algorithmic_tb": round(alg / 1e12, 2),
           "hbm_frac": round(alg / (ms / 1e3) / 1e9 / peak, 3), "hbm_frac_of": f"hbm_gbs of {peak_kind}"}
    # accuracy against the same circuits in complex128 (CUDA-core sweeps, pinned to the
    # oracle at 1e-12): ten circuits of up to 10 qubits, two of 12 and one of 13
    pick, want = [], {10: 10, 12: 2, 13: 1}
    for i, (n, d, sd) in enumerate(specs):
        key = 10 if n <= 10 else n
        if want.get(key, 0) > 0:
            pick.append(i)
            want[key] -= 1
    perr, zerr, rerr = 0.0, 0.0, 0.0
    for i in pick:
        n, d, sd = specs[i]
        s128 = DensityMatrixSim(workloads.noisy_brickwork_circuit(n, d, sd, p=1e-3), dtype=torch.complex128)
        s128.run()
        z = s128.pauli_expectations([(1.0, 'i' * q + 'z' + 'i' * (n - q - 1)) for q in range(n)]).cpu().numpy()
        perr = max(perr, abs(res[i]["purity"] - s128.purity()))
        zerr = max(zerr, float(np.abs(res[i]["z"] - z).max()))
        rho = batch.density_matrix(i).to(torch.complex128)
        rerr = max(rerr, float((rho - s128.get_density_matrix()).abs().max().item()))
        del s128, rho
        torch.cuda.empty_cache()
    out["vs_complex128"] = {"circuits": [specs[i][:2] for i in pick], "max_purity_error": perr,
                            "max_z_error": zerr, "max_abs_entry_error": rerr}
    del batch, sims
    torch.cuda.empty_cache()
    return out


def dist_init():
    """One process per GPU (replicas): NCCL with a GPU, gloo on the CPU (the
    host-side replica logic is tested that way)."""
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        if torch.cuda.is_available():
            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
            dist.init_process_group("nccl")
        else:
            dist.init_process_group("gloo")
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
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
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
    ex_kmax = max([len(st.bits) for st in ex.plan.steps if hasattr(st, "bits")] +
                  [len(p) for st in ex.plan.steps if hasattr(st, "ops") for p, _ in st.ops] +
                  [len(p) for st in ex.plan.steps if hasattr(st, "blocks") for p, _ in st.blocks] + [2])
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
        kname = {"sweep": (f"sweep_ldst_kernel<float,{ex_kmax}>" if itemsize == 8 else
                           f"sweep_df_kernel<{ex_kmax}>"),
                 "dense": f"dense_reg_kernel<{'float' if itemsize == 8 else 'double'},{ex_kmax}>",
                 "tcsweep": "tc_sweep_kernel"}[dom]
        tc_mode = _lib.lib().qgb_get_dense_impl()
        if dom == "dense" and itemsize == 8 and n >= 13 and (ex_kmax >= 5 and tc_mode >= 1 or
                                                            ex_kmax == 4 and tc_mode == 2):
            kname = f"dense_tc_kernel<{ex_kmax}>"
        tr = _profile_traffic(f"{kname}@{n}q") if args.depth == DEPTH else None
        roof = {"bound": "hbm", "kernel": f"qgb::{kname}",
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
                       "then pauli_expectation('zi...i').item(); the fusion plan of the circuit's structure "
                       "is cached after the first run (cold_compile: the first run of a new structure)",
               "check_value": r}
        # the same call with every plan and table cache emptied: a circuit structure seen for the first time
        from qaravan_gb300 import compiler, engine
        compiler._PLAN_CACHE.clear()
        engine._LAYOUT_CACHE.clear()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s2 = StatevectorSim(Circuit(gates, n=n), dtype=dtype, mode=args.mode, fusion_width=args.width,
                            tile_bits=args.tile, low_bits=args.low)
        s2.run()
        s2.pauli_expectation("z" + "i" * (n - 1))
        torch.cuda.synchronize()
        cold = time.perf_counter() - t0
        del s2
        e2e["cold_compile"] = {"s": round(cold, 4), "gates_per_s": round(gates_per_step / cold, 2)}

    if rank != 0:
        return
    launches = args.steps * (1 + ex.launches)
    # accuracy of the timed path: the final state (the last timed step's) against the same circuit
    # run in complex128 (CUDA-core tile sweeps, the path pinned to the reference fixtures at 1e-12)
    accuracy = None
    if rank == 0 and dtype == torch.complex64 and not args.no_accuracy:
        _lib.check(_lib.lib().qgb_set_c128_arith(0))  # float64 arithmetic for the reference state
        ref_sim = StatevectorSim(circ, dtype=torch.complex128)
        ref_state = ref_sim.get_statevector().reshape(-1)
        _lib.check(_lib.lib().qgb_set_c128_arith(1))
        diff = (state.to(torch.complex128) - ref_state).abs()
        accuracy = {"reference": "same circuit in complex128 (float64 CUDA-core tile sweeps)",
                    "max_abs_amplitude_error": float(diff.max().item()),
                    "rms_amplitude_error": float(diff.square().mean().sqrt().item()),
                    "max_abs_amplitude": float(ref_state.abs().max().item()),
                    "norm_error": float(abs(torch.linalg.vector_norm(state.to(torch.complex128)).item() - 1.0))}
        del ref_sim, ref_state, diff
    del state, ex, sim
    torch.cuda.empty_cache()
    sections = {}
    all_sections = ["c128", "variants", "torch_backend_gpu", "config1", "adjoint", "adjoint_batch", "trajectories",
                    "dm_batch"]
    wanted = args.sections.split(",") if args.sections != "all" else all_sections
    for name, fn in [("c128", lambda: section_c128(n, gates)), ("variants", lambda: section_variants(n, gates)),
                     ("torch_backend_gpu", lambda: section_torch_backend_gpu(gates, n)),
                     ("config1", section_config1), ("adjoint", section_adjoint),
                     ("adjoint_batch", section_adjoint_batch),
                     ("trajectories", section_trajectories), ("dm_batch", section_dm_batch)]:
        if name in wanted:
            try:
                sections[name] = fn()
            except Exception as e:  # secondary sections never suppress the headline line
                sections[name] = {"error": f"{type(e).__name__}: {str(e)[:300]}"}
            torch.cuda.empty_cache()
    # the CPU baseline is rank 0's at N=1 only
    cpu = None if (args.no_cpu or world > 1) else cpu_baseline(gates, n, args.depth)
    out = {
        "metric": METRIC, "value": round(value, 2), "unit": "gates/s", "n_gates": gates_per_step,
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_step, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c64" if dtype == torch.complex64 else "c128", "data": "synthetic (seeded Haar brickwork)",
        "config": workload_config(n, args.depth, "complex64" if dtype == torch.complex64 else "complex128"),
        "execution": {"mode": args.mode, "fusion_width": args.width, "tile_bits": args.tile,
                      "hbm_passes_per_step": passes, "flops_per_amp_per_step": flops_per_amp,
                      "parallelism": f"replicas x{world}"},
        "hbm_gbs_effective": round(passes * alg_bytes / (ms_step / 1e3) / 1e9, 1),
        "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks.summary(),
        "gpu_launches": launches, "accuracy": accuracy, "sections": sections,
    }
    print(json.dumps(out), flush=True)


def workload_config(n, depth, dtype_name):
    """The benchmark configuration, identical in both arms."""
    return {"workload": f"{n}-qubit open-chain Haar brickwork, depth {depth} "
                        f"({depth * (2 * n - 1)} gates), {dtype_name}",
            "qubits": n, "depth": depth, "seed": SEED, "dtype": dtype_name,
            "l2": "state (2^n x itemsize) larger than L2; no flush needed"}


def reference_arm(args):
    """The reference's CPU path (its torch backend's op_action on the host cores,
    complex64, all threads) on the benchmark's circuit: each step applies the
    next ceil(55 / steps) gates of the circuit's first depth unit, so the timed
    steps together cover the whole 55-gate unit (every depth unit has its shape)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import torch
    from oracle import ref
    n = args.qubits
    gates = workload_gates(n, args.depth)
    threads = _cpu_threads()
    unit = depth_unit(gates, n)
    mats = [torch.tensor(np.asarray(g.matrix), dtype=torch.complex64) for g in unit]
    per_step = -(-len(unit) // max(args.steps, 1))
    state = torch.zeros([2] * n, dtype=torch.complex64)
    state.view(-1)[0] = 1
    for i in range(args.warmup):
        state = ref.op_action_torch(mats[i % len(unit)], unit[i % len(unit)].indices, state)
    times, applied, pos = [], 0, 0
    for _ in range(args.steps):
        t0 = time.perf_counter()
        for _ in range(per_step):
            state = ref.op_action_torch(mats[pos], unit[pos].indices, state)
            pos = (pos + 1) % len(unit)
        times.append(time.perf_counter() - t0)
        applied += per_step
    total = sum(times)
    value = applied / total
    cpu = {"value": round(value, 4), "unit": "gates/s", "cores": threads, "kind": "port",
           "sample": f"{applied} gates ({per_step} per step) of the first depth unit ({len(unit)} gates: {n} SU(2) + "
                     f"{n - 1} SU(4)) of the {n}-qubit brickwork, complex64, the reference torch backend's op_action "
                     f"(permute + tensordot on CPU tensors, restated in oracle/); the {len(gates)}-gate circuit "
                     f"extrapolates to {len(gates) / value:.3g} s"}
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": "gates/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * total / args.steps, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c64",
        "data": "synthetic (seeded Haar brickwork)", "config": workload_config(n, args.depth, "complex64"),
        "cpu_baseline": cpu, "e2e": {"value": round(value, 4), "unit": "gates/s", "h2d_bytes_per_step": 0,
                                     "d2h_bytes_per_step": 0}}), flush=True)


def _time_traj_gates(sim):
    """Per-gate mode: one run with CUDA events around every gate's launches on the launching
    stream: a list of (gate index, union bits, lowest union bit, ms). The
    union is the gate's sites plus the previous gate's (pending damping)."""
    import torch
    from qaravan_gb300 import _lib
    L = _lib.lib()
    n, T = sim.n, sim.ntraj
    code = _lib.dtype_code(sim.dtype)
    st = _lib.stream_ptr(sim.device)
    stream = torch.cuda.current_stream(sim.device)
    sv, isz = sim.state.data_ptr(), sim.mats.element_size()
    _lib.check(L.qgb_init_basis(sv, code, n, 0, T, 2 ** n, st), "init_basis")
    rows, prev, kprev, prev_sites = [], None, 0, []
    for i, g in enumerate(sim.gates):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        _lib.check(L.qgb_traj_step(sv, code, n, T, 2 ** n, sim._site_arrays[i], len(g.indices),
                                   sim.mats.data_ptr() + sim.offs[i] * isz, prev, kprev, sim.kraus.data_ptr(),
                                   sim.p_dep, sim.gamma, sim.seed, i, sim.partials.data_ptr(), None, None, st),
                   "traj_step")
        e1.record(stream)
        union = set(g.indices) | set(prev_sites)
        rows.append((i, len(union), n - 1 - max(union), e0, e1))
        prev, kprev, prev_sites = sim._site_arrays[i], len(g.indices), list(g.indices)
    torch.cuda.synchronize(sim.device)
    return [(i, k, lo, e0.elapsed_time(e1)) for i, k, lo, e0, e1 in rows]


def run_case(args):
    """Small committed workloads for profiler captures (one run each, no CUDA
    graph, so that a profiler sees every launch):
      adjoint_batch [qubits layers sets]: one batched energy-and-gradient
        evaluation of the hardware-efficient ansatz (default 18 4 64);
      trajectory_gates [qubits trajectories steps]: the noisy TFI trajectories
        gate by gate with CUDA events around every gate (default 20 1024 2);
      trajectories [qubits trajectories steps tile_bits]: the same workload in
        one persistent launch (default 18 256 2 13);
      dm_batch [circuits seed]: the uneven noisy density-matrix batch (default 32 7);
      dm_batch_n [circuits qubits depth]: a batch of equal circuits of one size in the
        persistent launch (default 6 12 20)."""
    import torch
    from qaravan_gb300 import build as qbuild
    qbuild.build()
    from qaravan_gb300 import workloads
    vals = [int(v) for v in args.case_args.split(",") if v.strip()] if args.case_args else []
    if args.case == "adjoint_batch":
        from qaravan_gb300.adjoint import BatchedAnsatz
        from qaravan_gb300.hamiltonians import TFI
        n, layers, sets = (vals + [18, 4, 64][len(vals):])[:3]
        ba = BatchedAnsatz.hea(n, layers)
        x = torch.tensor(np.stack([workloads.hea_params(n, layers, s).reshape(-1) for s in range(sets)]),
                         device="cuda")
        E, _ = ba.energy_and_grad(x, TFI(n, 1, 1).pauli_sum())
        torch.cuda.synchronize()
        print("energy[0]", float(E[0]), "reverse passes", len(ba._rev), "ops per pass", [s.n_ops for s in ba._rev])
    elif args.case == "trajectory_gates":
        from qaravan_gb300.trajectories import TrajectorySim
        n, T, steps = (vals + [20, 1024, 2][len(vals):])[:3]
        sim = TrajectorySim(workloads.tfi_trotter_circuit(n, 0.05, steps), T, p_dep=1e-3, gamma=5e-4, seed=2026,
                            mode="per_gate")
        sim.run()
        rows = _time_traj_gates(sim)
        alg = 2 * T * 2 ** n * 8
        total = sum(ms for *_, ms in rows)
        print(f"{n} qubits, {T} trajectories, {len(rows)} gates: {total / len(rows):.3f} ms/gate, "
              f"{alg / 1e9:.2f} GB algorithmic per gate")
    elif args.case == "trajectories":
        from qaravan_gb300.trajectories import TrajectorySim
        n, T, steps, tile = (vals + [18, 256, 2, 13][len(vals):])[:4]
        sim = TrajectorySim(workloads.tfi_trotter_circuit(n, 0.05, steps), T, p_dep=1e-3, gamma=5e-4, seed=2026,
                            tile_bits=tile)
        ms = _event_ms(sim.run, 1, 1)
        print(f"{n} qubits, {T} trajectories, {len(sim.gates)} gates, {len(sim.sweep_plan)} sweeps of "
              f"{tile}-bit tiles: {ms:.2f} ms, {int(sim.jump_count.sum().item())} jumps")
    elif args.case == "dm_batch":
        from qaravan_gb300 import DensityMatrixSim
        from qaravan_gb300.batch import DensityMatrixBatch
        count, seed = (vals + [32, 7][len(vals):])[:2]
        specs = workloads.uneven_dm_specs(count, seed)
        sims = [DensityMatrixSim(workloads.noisy_brickwork_circuit(n, d, s, p=1e-3), dtype=torch.complex64)
                for n, d, s in specs]
        batch = DensityMatrixBatch(sims, dtype=torch.complex64)
        batch.run()
        torch.cuda.synchronize()
        res = batch.results()
        print(f"{count} circuits: {len(batch.small)} in the batched launch, {len(batch.large)} stream-parallel; "
              f"max trace error {max(abs(r['trace'] - 1) for r in res):.2e}")
    elif args.case == "dm_batch_n":
        from qaravan_gb300 import DensityMatrixSim
        from qaravan_gb300.batch import DensityMatrixBatch
        count, n, depth = (vals + [6, 12, 20][len(vals):])[:3]
        sims = [DensityMatrixSim(workloads.noisy_brickwork_circuit(n, depth, 100 + j, p=1e-3), dtype=torch.complex64)
                for j in range(count)]
        batch = DensityMatrixBatch(sims, dtype=torch.complex64)
        ms = _event_ms(batch.run, 1, 1)
        res = batch.results()
        print(f"{count} circuits of {n} qubits, depth {depth}: {len(batch.pers)} persistent, "
              f"{batch.persistent_passes} passes, {batch.persistent_items} items, {ms:.2f} ms; "
              f"max trace error {max(abs(r['trace'] - 1) for r in res):.2e}")
    else:
        raise SystemExit(f"unknown case {args.case!r}")


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--qubits", type=int, default=N_QUBITS)
    p.add_argument("--depth", type=int, default=DEPTH)
    p.add_argument("--dtype", default="c64", choices=["c64", "c128"])
    p.add_argument("--mode", default="fused", choices=["gate", "fused", "sweep", "tcsweep"])
    p.add_argument("--width", type=int, default=6)
    p.add_argument("--tile", type=int, default=14)
    p.add_argument("--low", type=int, default=None)
    p.add_argument("--e2e-steps", type=int, default=3)
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-accuracy", action="store_true", help="skip the complex128 comparison of the final state")
    p.add_argument("--sections", default="all",
                   help="comma list of variants,torch_backend_gpu,config1,adjoint,adjoint_batch,trajectories,"
                        "dm_batch; 'none' for the headline only")
    p.add_argument("--case", default=None, help="run one profiling workload instead (see run_case)")
    p.add_argument("--case-args", default="", help="comma-separated integers for --case")
    args = p.parse_args()
    if args.case:
        run_case(args)
    elif args.impl == "reference":
        reference_arm(args)
    else:
        gpu_arm(args)


if __name__ == "__main__":
    main()
