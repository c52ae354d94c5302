"""Generate the golden fixtures by running the real reference (qaravan).

Run from the repository root, in a container where the reference source tree
is present (``QGB_REFERENCE_SRC``, default ``/root/reference/src``):

    python tests/golden/make_golden.py

The reference is imported through ``oracle.refload`` (stand-ins for its three
uninstallable imports; nothing is written into its tree). Every output below
comes from the reference's own public API: ``StatevectorSim``,
``DensityMatrixSim``, ``pauli_expectation_sv``, ``partial_overlap``,
``Noise.get_superop`` and the torch backend with autograd. Inputs are the
seeded workloads of ``qaravan_gb300.workloads`` converted to the reference's
own gate objects; the gates are stored exactly as the reference saw them
(after e.g. ``CNOTGate`` reordered its indices).
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from oracle import refload  # noqa: E402
from gateio import pack_gates  # noqa: E402
from qaravan_gb300 import workloads  # noqa: E402


def _save(name, **arrays):
    path = os.path.join(HERE, name)
    np.savez_compressed(path, **arrays)
    print(f"wrote {name}: {os.path.getsize(path) / 1024:.1f} KiB")


def to_ref_gates(R, gates):
    return [R.core.Gate(g.name, list(g.indices), np.asarray(g.matrix, dtype=np.complex128)) for g in gates]


def run_ref_sv(R, gates, n, init_state=None):
    circ = R.core.Circuit(gates, n=n)
    sim = R.tensorQ.StatevectorSim(circ, init_state=init_state)
    sim.run(progress_bar=False)
    return np.asarray(sim.get_statevector(), dtype=np.complex128), sim


def gen_sv_brickwork(R):
    n, depth, seed = 12, 20, 1234
    gates = to_ref_gates(R, workloads.brickwork_gates(n, depth, seed))
    sv, sim = run_ref_sv(R, gates, n)
    rng = np.random.default_rng(7)
    ops = []
    for _ in range(n):
        a = rng.standard_normal((2, 2)) + 1j * rng.standard_normal((2, 2))
        ops.append((a + a.conj().T) / 2)
    local = sim.local_expectation(ops)
    one_local = np.array([sim.one_local_expectation(ops[q], q) for q in range(n)])
    tfi = [(c, s) for c, s in _tfi_terms(n)]
    pexp = np.array([R.tensorQ.pauli_expectation_sv(sv, s) for _, s in tfi])
    _save("sv_brickwork12.npz", n=n, depth=depth, seed=seed, sv=sv, local_ops=np.array(ops),
          local=np.array(local), one_local=one_local, tfi_coeffs=np.array([c for c, _ in tfi]),
          tfi_strings=np.array([s for _, s in tfi]), tfi_exp=pexp, **pack_gates(gates))


def _tfi_terms(n):
    t = [(1.0, 'i' * i + 'zz' + 'i' * (n - i - 2)) for i in range(n - 1)]
    t += [(1.0, 'i' * i + 'x' + 'i' * (n - i - 1)) for i in range(n)]
    return t


def gen_sv_mixed(R):
    """Unsorted / non-adjacent / 3-site gates, fixed and parametrised gates,
    CNOT in both orientations, mid-circuit Reset, bitstring initial state."""
    c = R.core
    n = 7
    rng = np.random.default_rng(99)
    hu = lambda d: workloads.haar_unitary(d, rng)  # noqa: E731
    gates = [
        c.H(0), c.X(3), c.SX(5), c.Gate("u2", [4, 1], hu(4)), c.Gate("u2", [0, 6], hu(4)),
        c.CNOT([1, 0], n), c.CNOT([2, 3], n), c.Gate("u3", [5, 2, 3], hu(8)),
        c.Gate("u3", [6, 0, 4], hu(8)), c.RX([2], 0.37), c.RY([4], 1.1), c.RZ([6], -0.8),
        c.RZZ([1, 5], 0.45), c.CZ([3, 4]), c.SWAP([0, 5]), c.iSWAP([2, 6]),
        c.Reset([3], "1"), c.Gate("u1", [3], hu(2)), c.Gate("u2", [3, 2], hu(4)),
        c.Reset([0, 4], "01"), c.Gate("u4", [1, 6, 3, 0], hu(16)), c.H(4),
    ]
    init = "0110101"
    sv, _ = run_ref_sv(R, gates, n, init_state=init)
    _save("sv_mixed7.npz", n=n, init=init, sv=sv, **pack_gates(gates))


def gen_sv_decomp(R):
    """A circuit with U gates built from angles and from matrices, run with
    requires_decomp=True: the reference decomposes every U into RZ / SX gates
    (core/circuits.py:31-40, core/param_gates.py:144-156) inside the
    simulator's copy; a U built from a matrix stores it without the phase of
    its top-left entry (core/param_gates.py:131-133)."""
    c = R.core
    n = 4
    rng = np.random.default_rng(5)
    mats = [workloads.haar_unitary(2, rng) for _ in range(2)]
    angles = [(0.3, -1.1, 2.0), (1.7, 0.4, -0.6)]
    gates = [c.U([0], *angles[0]), c.U([2], mats[0]), c.CNOT([1, 0], n), c.U([1], *angles[1]), c.U([3], mats[1]),
             c.H(2), c.CNOT([3, 2], n)]
    sim = R.tensorQ.StatevectorSim(c.Circuit(gates, n=n, requires_decomp=True))
    sim.run(progress_bar=False)
    sv = np.asarray(sim.get_statevector(), dtype=np.complex128)
    plain = [c.U([0], *angles[0]), c.U([2], mats[0]), c.CNOT([1, 0], n), c.U([1], *angles[1]), c.U([3], mats[1]),
             c.H(2), c.CNOT([3, 2], n)]
    sv_plain, _ = run_ref_sv(R, plain, n)
    # the simulator's copy drops requires_decomp (core/circuits.py:163-169); Circuit.build()
    # on the circuit itself decomposes, and a prebuilt circuit runs as built
    built = c.Circuit([c.U([0], *angles[0]), c.U([2], mats[0]), c.CNOT([1, 0], n), c.U([1], *angles[1]),
                       c.U([3], mats[1]), c.H(2), c.CNOT([3, 2], n)], n=n, requires_decomp=True).build()
    sim_b = R.tensorQ.StatevectorSim(built)
    sim_b.run(progress_bar=False)
    sv_built = np.asarray(sim_b.get_statevector(), dtype=np.complex128)
    _save("sv_decomp4.npz", n=n, sv=sv, sv_plain=sv_plain, sv_built=sv_built, angles=np.array(angles),
          mats=np.array(mats), **pack_gates(sim.circ.gate_list, prefix="d"), **pack_gates(plain, prefix="u"),
          **pack_gates(built.gate_list, prefix="b"))


def gen_gates_misc(R):
    """CUGate matrices and stored indices (both control placements, 1- and
    2-site subgates) and embed_operator in its three forms, from the reference."""
    c = R.core
    rng = np.random.default_rng(17)
    sub1, sub2 = workloads.haar_unitary(2, rng), workloads.haar_unitary(4, rng)
    cases = [([1, 2], sub1), ([2, 1], sub1), ([1, 2, 3], sub2), ([2, 3, 1], sub2)]
    out = {}
    for i, (idx, sub) in enumerate(cases):
        g = c.CUGate(idx, c.Gate("u", list(range(int(np.log2(sub.shape[0])))), sub))
        out[f"cu{i}_in"] = np.array(idx)
        out[f"cu{i}_idx"] = np.array(g.indices)
        out[f"cu{i}_mat"] = np.asarray(g.matrix, dtype=np.complex128)
        out[f"cu{i}_sub"] = sub
        out[f"cu{i}_bottom"] = np.array(bool(g.bottom_heavy))
    a = workloads.haar_unitary(4, rng)
    out["emb_block"] = np.asarray(c.embed_operator(4, [1, 2], a), dtype=np.complex128)
    out["emb_block_op"] = a
    ops = [workloads.haar_unitary(2, rng) for _ in range(2)]
    out["emb_ops"] = np.array(ops)
    out["emb_dense"] = np.asarray(c.embed_operator(4, [0, 3], ops, dense=True), dtype=np.complex128)
    out["emb_dense_half"] = np.asarray(c.embed_operator(4, [0, 3], ops, dense=True, factor=True), dtype=np.complex128)
    out["emb_sparse"] = c.embed_operator(4, [2, 1], ops).toarray()
    out["emb_pauli"] = c.embed_operator(3, [0, 1, 2], "xyz").toarray()
    _save("gates_misc.npz", **out)


def gen_pretty(R):
    """The reference's pretty-printed statevector and density matrix (core/utils.py:52-89)."""
    u = R.core
    v = np.array([1, 0, 0.5j, 0, 0, 0, 0, 1]) / np.sqrt(2.25)
    rho = 0.6 * np.outer(v, v.conj()) + 0.4 * np.diag([0, 0, 0, 1, 0, 0, 0, 0])
    _save("pretty.npz", sv=v, dm=rho, sv_str=np.array(u.pretty_print_sv(v)), dm_str=np.array(u.pretty_print_dm(rho)))


def gen_noise_misc(R):
    """random_pauli_channel under a fixed global seed (strings, weights, str())
    and the Pauli-Lindblad superoperators, from the reference (core/noise.py)."""
    c = R.core
    np.random.seed(3)
    ch = c.random_pauli_channel(3, 5, 0.2)
    lb = c.PauliLindbladNoise(['xi', 'zz', 'yx'], [0.05, 0.1, 0.02])
    _save("noise_misc.npz", strings=np.array(ch.strings), probs=np.array(ch.probs), text=np.array(str(ch)),
          lb_superop=lb.make_superop(), lb_superop_1=lb.get_superop_for_string(1))


def gen_trotter_apps(R):
    """applications/trotter.py run by the reference itself: the statevector run
    (TFI, 6 sites, 5 steps, normalised magnetisation) and the noisy
    density-matrix run (4 sites, 4 steps, a 4-site Pauli channel after every
    layer), cached and uncached."""
    import importlib
    t = importlib.import_module("qaravan.applications.trotter")
    c = R.core
    ham = c.TFI(6, jz=1.0, h=0.7)
    sv = t.trotter_sv_sim(ham, 0.1, 5, t.magnetization(6))
    ham4 = c.TFI(4, jz=1.0, h=0.9)
    ch = c.PauliNoise(["iiii", "xiii", "iziz", "yyii", "iixx"], [0.92, 0.02, 0.03, 0.01, 0.02])
    dm = t.trotter_dm_sim(ham4, 0.1, 4, ch, t.magnetization(4))
    dm_u = t.trotter_dm_sim_uncached(ham4, 0.1, 4, ch, t.magnetization(4))
    _save("trotter_apps.npz", sv=np.array(sv), dm=np.array(dm), dm_uncached=np.array(dm_u))


def gen_sv_observables(R):
    """Pauli-string expectations, partial overlaps and outcome probabilities on
    a random 8-qubit state."""
    n = 8
    rng = np.random.default_rng(5)
    gates = to_ref_gates(R, workloads.brickwork_gates(n, 4, 77))
    sv, _ = run_ref_sv(R, gates, n)
    strings = [''.join(rng.choice(list('ixyz'), size=n)) for _ in range(24)]
    strings += ['z' * n, 'x' * n, 'y' * n, 'i' * n]
    pexp = np.array([R.tensorQ.pauli_expectation_sv(sv, s) for s in strings])
    sv2, _ = run_ref_sv(R, to_ref_gates(R, workloads.brickwork_gates(n, 3, 78)), n)
    po_sites = [[2], [0, 5], [7, 1, 3]]
    po = [R.tensorQ.partial_overlap(sv, sv2, skip=s) for s in po_sites]
    rdm = [R.tensorQ.rdm_from_sv(sv, s) for s in po_sites]
    _save("sv_observables8.npz", n=n, sv=sv, sv2=sv2, strings=np.array(strings), pexp=pexp,
          po_sites=np.array([s + [-1] * (3 - len(s)) for s in po_sites]),
          po0=po[0], po1=po[1], po2=po[2], rdm0=rdm[0], rdm1=rdm[1], rdm2=rdm[2])


def gen_dm_mixed(R):
    """Gates (sorted and unsorted indices) and channel superoperators applied
    through ``DensityMatrixSim.apply_gate``; expectations and purity."""
    c = R.core
    n = 5
    rng = np.random.default_rng(2024)
    hu = lambda d: workloads.haar_unitary(d, rng)  # noqa: E731
    qn = c.QubitNoise(50.0, 30.0, 1.0, 5.0)
    pn = c.PauliNoise(['ii', 'xz', 'yy', 'zi'], [0.85, 0.05, 0.04, 0.06])
    ops = [
        c.Gate("u1", [0], hu(2)), c.Gate("u2", [1, 2], hu(4)), c.Gate("u2", [4, 3], hu(4)),
        c.ID(2, 3.0, [2], nm=qn), c.Gate("u3", [0, 2, 4], hu(8)), c.ID(2, 0.0, [3, 1], nm=pn),
        c.CNOT([1, 0], n), c.Gate("u2", [3, 0], hu(4)), c.ID(2, 5.0, [4], nm=qn, dd=True),
        c.Gate("u1", [1], hu(2)), c.ID(2, 0.0, [0, 4], nm=pn),
    ]
    sim = R.tensorQ.DensityMatrixSim(c.Circuit([c.H(0)], n=n))
    sim.initialize_state()
    superops, locs = [], []
    for op in ops:
        sim.apply_gate(op)
        superops.append(np.asarray(op.to_superop(), dtype=np.complex128).reshape(4 ** op.span, 4 ** op.span))
        locs.append(list(op.indices))
    dm = np.asarray(sim.get_density_matrix(), dtype=np.complex128).copy()
    sim.ran = True
    rng2 = np.random.default_rng(3)
    lops = []
    for _ in range(n):
        a = rng2.standard_normal((2, 2)) + 1j * rng2.standard_normal((2, 2))
        lops.append((a + a.conj().T) / 2)
    one_local = np.array([sim.one_local_expectation(lops[q], q) for q in range(n)])
    g = rng2.standard_normal((2 ** n, 2 ** n)) + 1j * rng2.standard_normal((2 ** n, 2 ** n))
    gop = (g + g.conj().T) / 2
    glob = sim.global_expectation(gop)
    # local_expectation overwrites the simulator's state; evaluate it last, on a copy
    sim2 = R.tensorQ.DensityMatrixSim(c.Circuit([c.H(0)], n=n), init_state=dm.copy())
    sim2.initialize_state()
    sim2.ran = True
    sim2.run = lambda progress_bar=False: None
    local = sim2.local_expectation(lops)
    flat = np.concatenate([s.reshape(-1) for s in superops])
    offs = np.cumsum([0] + [s.size for s in superops])
    _save("dm_mixed5.npz", n=n, dm=dm, superops=flat, superop_offs=offs,
          locs=np.array([l + [-1] * (3 - len(l)) for l in locs]), nlocs=np.array([len(l) for l in locs]),
          is_noise=np.array([op.name == "ID" for op in ops]), local_ops=np.array(lops),
          one_local=one_local, global_op=gop, global_exp=np.array(glob), local=np.array(local),
          purity=np.array(np.trace(dm @ dm).real), **pack_gates(ops))


def gen_dm_kats(R):
    c, tq = R.core, R.tensorQ
    circ = c.Circuit([c.H(0), c.CNOT([1, 0], 3), c.CNOT([2, 1], 3)], 3)
    Z, X = c.pauli_Z, c.pauli_X
    out = {}
    sim = tq.DensityMatrixSim(circ, nm=c.QubitNoise(1000, 1000, 1, 5))
    sim.run(progress_bar=False)
    out["thermal_dm"] = np.asarray(sim.get_density_matrix(), dtype=np.complex128).copy()
    out["thermal_zzz"] = sim.local_expectation([Z, Z, Z])
    sim = tq.DensityMatrixSim(circ, nm=c.QubitNoise(1000, 1000, 1, 5))
    out["thermal_xxx"] = sim.local_expectation([X, X, X])
    pn = c.PauliNoise(['iii', 'xxx', 'yyy', 'zyz'], [0.9, 0.05, 0.02, 0.03])
    sim = tq.DensityMatrixSim(circ, nm=pn)
    sim.run(progress_bar=False)
    out["pauli_dm"] = np.asarray(sim.get_density_matrix(), dtype=np.complex128).copy()
    out["pauli_zzz"] = sim.local_expectation([Z, Z, Z])
    sim = tq.DensityMatrixSim(circ, nm=pn)
    out["pauli_xxx"] = sim.local_expectation([X, X, X])
    sv = tq.StatevectorSim(circ)
    out["ghz_sv"] = np.asarray(sv.get_statevector(), dtype=np.complex128)
    out["ghz_zzz"] = sv.local_expectation([Z, Z, Z])
    out["ghz_xxx"] = sv.local_expectation([X, X, X])
    # trajectory notebook KAT: H RZ(pi/4) H on 2 sites, normalised magnetisation
    c2 = c.Circuit([c.H(0), c.RZ(0, np.pi / 4), c.H(0)], 2)
    fs = c2.to_matrix() @ np.array([1, 0, 0, 0])
    op = (np.kron(Z, c.pauli_I) + np.kron(c.pauli_I, Z)) / (2 * np.sqrt(2))
    out["hrzh_exp"] = np.trace(op @ np.outer(fs, fs.conj())).real
    _save("dm_kats.npz", **{k: np.asarray(v) for k, v in out.items()})


def gen_traj_dm10(R, steps, p, gamma, name):
    """DM oracle for the noisy TFI trajectories: every Trotter gate followed,
    on each of its sites, by depolarising(p) and then amplitude damping(gamma)."""
    c, tq = R.core, R.tensorQ
    n = 10
    dep = c.PauliNoise(['i', 'x', 'y', 'z'], [1 - p, p / 3, p / 3, p / 3])
    ad = c.QubitNoise(1.0, np.inf, 1.0, 1.0)
    t_ad = -np.log(1 - gamma)  # 1 - exp(-t/t1) = gamma with t1 = 1
    gates = c.TFI(n, jz=1, h=1).trotter_circ(0.05, steps).gate_list
    sim = tq.DensityMatrixSim(c.Circuit([c.H(0)], n=n))
    sim.initialize_state()
    t0 = time.time()
    for g in gates:
        sim.apply_gate(g)
        for q in g.indices:
            sim.apply_gate(c.ID(2, 0.0, [q], nm=dep))
            sim.apply_gate(c.ID(2, t_ad, [q], nm=ad))
    dm = np.asarray(sim.get_density_matrix(), dtype=np.complex128)
    Z = c.pauli_Z
    diag = np.real(np.diag(dm))
    idx = np.arange(2 ** n)
    zi = np.array([np.sum(diag * (1 - 2 * ((idx >> (n - 1 - q)) & 1))) for q in range(n)])
    zz = np.array([np.sum(diag * (1 - 2 * (((idx >> (n - 1 - q)) ^ (idx >> (n - 2 - q))) & 1)))
                   for q in range(n - 1)])
    one_local = np.array([sim.one_local_expectation(Z, q) for q in range(n)])
    print(f"{name}: {len(gates)} gates in {time.time() - t0:.1f}s")
    _save(name, n=n, steps=steps, p=p, gamma=gamma, z=zi, zz=zz, one_local_z=one_local,
          purity=np.array(np.sum(np.abs(dm) ** 2)), **pack_gates(gates))


def gen_grad_hea(R):
    """Reference torch-backend autograd gradient of the TFI energy of a small
    hardware-efficient ansatz (complex64, as the reference's torch path)."""
    import torch
    c, tq = R.core, R.tensorQ
    n, layers = 6, 3
    params = workloads.hea_params(n, layers, 11)
    th = torch.tensor(params, dtype=torch.float64, requires_grad=True)
    gl = []
    for l in range(layers):
        for q in range(n):
            gl.append(c.RY([q], th[l, q, 0]))
            gl.append(c.RZ([q], th[l, q, 1]))
        for q in range(n - 1):
            gl.append(c.CNOT([q + 1, q], n))
    sim = tq.StatevectorSim(c.Circuit(gl, n=n), backend="torch")
    sim.run(progress_bar=False)
    sv = sim.get_statevector()
    terms = _tfi_terms(n)
    from functools import reduce
    P = {'i': np.eye(2), 'x': c.pauli_X, 'z': c.pauli_Z}
    H = sum(cf * reduce(np.kron, [P[ch] for ch in s]) for cf, s in terms)
    Ht = torch.tensor(H, dtype=torch.complex64)
    loss = torch.real(torch.vdot(sv, Ht @ sv))
    loss.backward()
    _save("grad_hea6.npz", n=n, layers=layers, params=params, energy=np.array(loss.item()),
          grad=th.grad.numpy(), sv=sv.detach().numpy().astype(np.complex128))


def gen_msp_env(R):
    """applications/compilation.py run by the reference itself on 4 qubits:
    environments of single gates, three sweeps of ``msp_via_environments``
    (final gate matrices and costs) and ``msp_cost`` with a matrix target and
    with output states. (The reference's ``unitary_embedding`` raises NameError:
    its module does not import scipy.)"""
    import contextlib
    import importlib
    import io
    comp = importlib.import_module("qaravan.applications.compilation")
    rng = np.random.default_rng(31)
    n, sk = 4, [[0, 1], [1, 2], [2, 3], [0, 1], [1, 2]]
    params = rng.uniform(0, 2 * np.pi, size=len(sk) * 6 + n * 3)
    in_strings = ["0000", "0110", "1011"]
    ins = [comp.string_to_sv(s) for s in in_strings]
    outs = []
    for _ in in_strings:
        v = rng.normal(size=2 ** n) + 1j * rng.normal(size=2 ** n)
        outs.append(v / np.linalg.norm(v))
    ansatz = comp.dressed_cnot_circ(sk, n, params)
    env_idx = [0, 1, 4, len(ansatz.gate_list) - 1]
    envs = np.array([comp.msp_environment(ins[1], ansatz, outs[1], i) for i in env_idx])
    with contextlib.redirect_stdout(io.StringIO()), contextlib.redirect_stderr(io.StringIO()):
        new, costs, term = comp.msp_via_environments(ins, comp.dressed_cnot_circ(sk, n, params), outs, num_sweeps=3)
    mats = np.zeros((len(new.gate_list), 16), dtype=np.complex128)
    for i, g in enumerate(new.gate_list):
        m = np.asarray(g.matrix, dtype=np.complex128).reshape(-1)
        mats[i, :m.size] = m
    sizes = np.array([np.asarray(g.matrix).size for g in new.gate_list])
    target = np.linalg.qr(rng.normal(size=(2 ** n, 2 ** n)) + 1j * rng.normal(size=(2 ** n, 2 ** n)))[0]
    cost_mat = comp.msp_cost(params, sk, ins, target)
    cost_states = comp.msp_cost(params, sk, ins, outs)
    _save("msp_env.npz", n=n, skeleton=np.array(sk), params=params, in_strings=np.array(in_strings),
          outs=np.array(outs), env_idx=np.array(env_idx), envs=envs, costs=np.array(costs), term=np.array(term),
          mats=mats, sizes=sizes, target=target,
          cost_mat=np.array(cost_mat), cost_states=np.array(cost_states))


def main():
    R = refload.load()
    np.random.seed(0)
    gen_sv_brickwork(R)
    gen_sv_mixed(R)
    gen_sv_observables(R)
    gen_dm_mixed(R)
    gen_dm_kats(R)
    gen_grad_hea(R)
    gen_traj_dm10(R, steps=10, p=0.02, gamma=0.03, name="traj_dm10_strong.npz")
    gen_traj_dm10(R, steps=40, p=1e-3, gamma=5e-4, name="traj_dm10.npz")
    gen_sv_decomp(R)
    gen_gates_misc(R)
    gen_pretty(R)
    gen_noise_misc(R)
    gen_trotter_apps(R)
    gen_msp_env(R)


if __name__ == "__main__":
    main()
