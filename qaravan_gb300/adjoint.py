"""Adjoint-method gradients behind ``torch.autograd``.

The reference differentiates circuits by running its torch backend under
autograd (``core/param_gates.py:21-49`` builds gate matrices with
``torch.linalg.matrix_exp``; ``applications/compilation.py:73-133`` calls
``loss.backward()``), which keeps every intermediate state on the tape: one
state per gate. Here the forward pass runs the fused CUDA plan and keeps only
the final state; the backward pass walks the gates in reverse, uncomputing the
state (``phi <- U^dagger phi``) and carrying the co-state
(``lam <- U^dagger lam``) in one kernel pass per gate, which also reduces the
gate's gradient block ``sum_rest lam[r, rest] conj(phi[c, rest])`` in float64
(``qgb_adjoint_step``). Memory: three states, independent of depth.

Conventions: for a real loss L, torch's gradient of a complex tensor z is
``2 dL/d conj(z)``; the state function receives ``g = 2 dL/d conj(psi)`` and
returns ``dL/dM = sum g[r] conj(phi[c])`` (the factor 2 is already in ``g``);
the energy function starts from ``lam = H psi`` and returns
``2 sum lam[r] conj(phi[c])``.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from .compiler import Op, compile_ops
from .engine import Executor, Scratch


def _gate_list(sim):
    from .statevector import circuit_ops
    gates = [g for g in circuit_ops(sim.circ, build=True, nm=getattr(sim, "nm", None))
             if not (g.name == "ID" and getattr(g, "nm", None) is not None)]
    for g in gates:
        if len(g.indices) > 2:
            raise NotImplementedError("the adjoint sweep handles gates on one or two sites")
        if g.name == "Reset":
            raise NotImplementedError("Reset is not differentiable")
    return gates


class _Runner:
    """Forward plan + reverse sweep for a fixed gate structure."""

    def __init__(self, sim, gates):
        self.sim = sim
        self.gates = gates
        self.n = sim.num_sites
        self.dtype = sim.dtype
        self.device = sim.device
        self.code = _lib.dtype_code(self.dtype)
        self.scratch = Scratch(self.device)
        self._sites = [_lib.int_array(g.indices) for g in gates]

    def host_matrices(self, mats):
        """All gate matrices as complex128 NumPy arrays (one host transfer)."""
        flat = torch.cat([m.detach().reshape(-1).to("cpu", torch.complex128) for m in mats]).numpy()
        out, o = [], 0
        for m in mats:
            k = m.numel()
            d = int(round(k ** 0.5))
            out.append(flat[o:o + k].reshape(d, d))
            o += k
        return out, flat

    def forward_state(self, mats, flat=None):
        n = self.n
        if flat is None:
            host, flat = self.host_matrices(mats)
        else:  # per-gate views of the flattened matrices
            o = 0
            host = []
            for m in mats:
                k = m.numel()
                d = int(round(k ** 0.5))
                host.append(flat[o:o + k].reshape(d, d))
                o += k
        self._flat = flat
        ops = [Op([n - 1 - q for q in g.indices], m) for g, m in zip(self.gates, host)]
        kcap = 5 if self.dtype == torch.complex64 else 4
        isz = torch.empty(0, dtype=self.dtype).element_size()
        if self.dtype == torch.complex64:
            # gradients are differences of large, nearly cancelling sums: the forward runs as
            # float32 CUDA-core tile sweeps of 4-qubit blocks (a few ms) rather than the split-fp16
            # tensor-core blocks, whose rounding left up to 9e-6 relative gradient error at 20
            # qubits, 40 layers (3e-6 with the CUDA cores, against complex128)
            plan = compile_ops(ops, n, mode="sweep", width=4, tile_bits=14, max_sweep_k=kcap, itemsize=isz,
                               device_fusion=True)
        else:
            plan = compile_ops(ops, n, mode=self.sim.mode, width=self.sim.fusion_width, tile_bits=self.sim.tile_bits,
                               low_bits=self.sim.low_bits, max_sweep_k=kcap, itemsize=isz, device_fusion=True)
        self.sim.initialize_state()  # |0..0>, a bitstring or a given array (copied), as the simulator starts
        psi = self.sim.state.detach().reshape(-1)
        self.sim.state = None  # psi is the only reference: no extra state-sized buffer
        Executor(plan, self.dtype, self.device).run(psi)
        return psi

    def reverse(self, psi, lam, mats, need):
        """Reverse sweep from (psi, lam). ``need[i]``: False (no gradient), True
        (the matrix block sum_rest lam[r] conj(phi[c])) or ("rotation", kind)
        for a rotation exp(-i theta P): the scalar Im <lam|P|phi> at the gate's
        output. Runs of gates without a matrix block go through tile passes
        (``qgb_adjoint_sweep_step``, many gates per read of the two states);
        a matrix block takes its own pass (``qgb_adjoint_step``). Returns per
        gate the complex128 block, the float, or None."""
        L = _lib.lib()
        n = self.n
        st = _lib.stream_ptr(self.device)
        phi = psi.detach().clone()
        lam = lam.contiguous()
        # every gate matrix in one pinned upload; per-gate element offsets
        flat = getattr(self, "_flat", None)
        if flat is None:
            _, flat = self.host_matrices(mats)
        dev = torch.from_numpy(flat).to(self.dtype).pin_memory().to(self.device, non_blocking=True)
        isz = dev.element_size()
        offs = np.cumsum([0] + [m.numel() for m in mats])
        grads_dev = torch.empty(len(self.gates), 32, dtype=torch.float64, device=self.device)
        tile = min(_tile_bits(self.dtype), n)
        nbytes = max(L.qgb_reduce_scratch_bytes(n, 32, 1), L.qgb_adjoint_sweep_scratch_bytes(n, tile, 64, 1))
        scr = self.scratch.get(nbytes)
        base, gbase = dev.data_ptr(), grads_dev.data_ptr()
        run = []

        def flush():
            if not run:
                return
            rows = np.array([(i, kind, bits[0], bits[1] if len(bits) > 1 else -1) for (i, kind), bits in run],
                            dtype=np.int64)
            key = (n, tile, rows.tobytes(), offs[rows[:, 0]].tobytes())
            sweeps = _REV_CACHE.pop(key, None)
            if sweeps is None:
                sweeps = [_adjoint_sweep_struct(lo, high, [(bits, int(offs[i]), i * 32 if kind else -1, kind)
                                                           for (i, kind), bits in ops])
                          for lo, high, ops in _plan_reverse(run, n, tile)]
            _REV_CACHE[key] = sweeps  # most recently used last
            while len(_REV_CACHE) > 16:
                _REV_CACHE.pop(next(iter(_REV_CACHE)))
            for sw in sweeps:
                _lib.check(L.qgb_adjoint_sweep_step(phi.data_ptr(), lam.data_ptr(), self.code, n, C.byref(sw), base,
                                                    0, 1, 0, gbase, scr.data_ptr(), nbytes, st), "adjoint_sweep_step")
            run.clear()

        for i in range(len(self.gates) - 1, -1, -1):
            k = len(self.gates[i].indices)
            want = need[i]
            if want is True:
                flush()
                _lib.check(L.qgb_adjoint_step(phi.data_ptr(), lam.data_ptr(), self.code, n, self._sites[i], k,
                                              base + int(offs[i]) * isz, gbase + i * 32 * 8, scr.data_ptr(), nbytes,
                                              st), "adjoint_step")
            else:
                run.append(((i, want[1] if want else 0), [n - 1 - q for q in self.gates[i].indices]))
        flush()
        host = grads_dev.cpu().numpy()
        out = []
        for i, g in enumerate(self.gates):
            want = need[i]
            if want is False:
                out.append(None)
            elif want is True:
                d = 2 ** len(g.indices)
                v = host[i, :2 * d * d]
                out.append((v[0::2] + 1j * v[1::2]).reshape(d, d))
            else:
                out.append(float(host[i, 0]))
        return out


def _grad_like(m, arr):
    return torch.from_numpy(arr).to(device=m.device, dtype=m.dtype if m.is_complex() else torch.complex128)


# Rotations exp(-i theta P) with P a Pauli or a Pauli pair (core/param_gates.py:51-103):
# kind -> P as a dense matrix (rows = the gate's index order).
_KIND = {"RX": 1, "RY": 2, "RZ": 3, "RXX": 4, "RYY": 5, "RZZ": 6}
_PX = np.array([[0, 1], [1, 0]], dtype=np.complex128)
_PY = np.array([[0, -1j], [1j, 0]], dtype=np.complex128)
_PZ = np.array([[1, 0], [0, -1]], dtype=np.complex128)
_GEN = {1: _PX, 2: _PY, 3: _PZ, 4: np.kron(_PX, _PX), 5: np.kron(_PY, _PY), 6: np.kron(_PZ, _PZ)}
_GEN_C = {k: _lib.double_array(np.stack([m.real, m.imag], axis=-1).reshape(-1)) for k, m in _GEN.items()}
# per kind: (column, value) of the one nonzero of each generator row
_GEN_ROWS = {k: [(int(np.flatnonzero(m[r])[0]), complex(m[r, np.flatnonzero(m[r])[0]])) for r in range(m.shape[0])]
             for k, m in _GEN.items()}


# tile-pass descriptions of a reverse sweep per structure (gates, sites, derivative slots,
# matrix offsets): a training loop re-plans nothing
_REV_CACHE: dict = {}


def _tile_bits(dtype):
    """Tile of the adjoint sweeps: state and co-state double-buffered in shared
    memory (4 x 2^m amplitudes: 64 KiB at m = 11 for complex64, three CTAs per
    SM, the fastest of m = 10-12 measured on 64 sets of 20 qubits; 128 KiB at
    m = 11 for complex128)."""
    return 11


def _plan_reverse(items, nbits, tile_bits):
    """Group the reverse sweep's gates into tile passes. ``items``: (payload, flat
    bits in matrix order) in the order the sweep meets them. Gates on disjoint
    bits may change order, which leaves every rotation derivative unchanged
    (the moved gate commutes with the generator). Returns (L, high, [(payload,
    bits)]) per pass."""
    from types import SimpleNamespace
    from .compiler import plan_sweeps
    blocks = [SimpleNamespace(bits=list(b), payload=p) for p, b in items]
    return [(L, high, [(blk.payload, blk.bits) for blk in taken])
            for L, high, taken in plan_sweeps(blocks, nbits, tile_bits)]


def _adjoint_sweep_struct(L, high, ops):
    """``qgb_adjoint_sweep`` for one pass; ``ops``: (flat bits in matrix order,
    matrix element offset, output slot or -1, rotation kind when the slot is set)."""
    sw = _lib.AdjointSweep()
    sw.low_bits = L
    sw.n_high = len(high)
    for i, b in enumerate(high):
        sw.high_bits[i] = b
    tpos = {b: b for b in range(L)}
    tpos.update({b: L + h for h, b in enumerate(high)})
    sw.n_ops = len(ops)
    for i, (bits, off, out, kind) in enumerate(ops):
        sw.op_k[i] = len(bits)
        for j, b in enumerate(bits):
            sw.op_pos[i][j] = tpos[b]
        sw.op_mat[i] = int(off)
        sw.op_out[i] = int(out)
        if out >= 0:
            for r, (c, v) in enumerate(_GEN_ROWS[int(kind)]):
                sw.op_gen_col[i][r] = c
                sw.op_gen_val[i][r][0] = v.real
                sw.op_gen_val[i][r][1] = v.imag
    return sw


def _forward_sweep_struct(L, high, ops):
    """``qgb_sweep`` for one forward pass; ``ops``: (flat bits in matrix order, matrix element offset)."""
    sw = _lib.Sweep()
    sw.low_bits = L
    sw.n_high = len(high)
    for i, b in enumerate(high):
        sw.high_bits[i] = b
    tpos = {b: b for b in range(L)}
    tpos.update({b: L + h for h, b in enumerate(high)})
    sw.n_ops = len(ops)
    for i, (bits, off) in enumerate(ops):
        sw.op_k[i] = len(bits)
        for j, b in enumerate(bits):
            sw.op_pos[i][j] = tpos[b]
        sw.op_mat[i] = int(off)
    return sw


def _forward_sweep_struct_pos(L, high, ops):
    """``qgb_sweep`` for one pass; ``ops``: (tile positions in matrix order, matrix element offset)."""
    sw = _lib.Sweep()
    sw.low_bits = L
    sw.n_high = len(high)
    for i, b in enumerate(high):
        sw.high_bits[i] = b
    sw.n_ops = len(ops)
    for i, (pos, off) in enumerate(ops):
        sw.op_k[i] = len(pos)
        for j, p in enumerate(pos):
            sw.op_pos[i][j] = p
        sw.op_mat[i] = int(off)
    return sw


def _rotation_angle(g):
    """The torch angle of a rotation gate whose matrix is still the one built
    from it, else None."""
    kind = _KIND.get(getattr(g, "name", None))
    angles = getattr(g, "angles", None)
    if kind is None or not isinstance(angles, tuple) or len(angles) != 1:
        return None
    a = angles[0]
    if not (torch.is_tensor(a) and a.numel() == 1 and getattr(g, "built_from_angles", lambda: False)()):
        return None
    return a


def _stack_angles(angles):
    """All rotation angles as one float64 host vector for autograd. When every
    angle is a one-element view of the same contiguous tensor (``th[l, q, k]``,
    as a parameter tensor is usually indexed), one gather from that tensor
    replaces a stack of per-angle selects, so the backward is one scatter rather
    than one autograd node per angle; the values and gradients are the same."""
    if not angles:
        return torch.zeros(0, dtype=torch.float64)
    base = angles[0]._base
    if (base is not None and base.is_contiguous()
            and all(a._base is base and a.numel() == 1 and a.dtype == base.dtype for a in angles)):
        idx = torch.tensor([a.storage_offset() - base.storage_offset() for a in angles], dtype=torch.long,
                           device=base.device)
        out = base.reshape(-1).index_select(0, idx)
        return (out.cpu() if out.is_cuda else out).to(torch.float64)
    vals = [a.reshape(()).to(torch.float64) for a in angles]
    try:
        out = torch.stack(vals)  # one copy to the host when the angles share a device
    except RuntimeError:
        return torch.stack([v.cpu() for v in vals])
    return out.cpu() if out.is_cuda else out


class _Inputs:
    """How the gates enter autograd. A rotation gate exp(-i theta P) built from
    a torch angle contributes its angle (all such angles stacked into one
    float64 vector): dL/dtheta = Re sum conj(G) dM/dtheta (G = dL/dM) equals
    2 Im <lam|P|phi> at the gate's output (M commutes with P), which the
    rotation form of the reverse step reduces directly, so autograd never walks
    back through ``matrix_exp``. Every other gate contributes its matrix."""

    def __init__(self, gates, closed_form=False):
        self.mats, self.flat = _matrices(gates, closed_form)
        self.rot, angles = [], []
        for i, g in enumerate(gates):
            a = _rotation_angle(g)
            if a is not None:
                self.rot.append(i)
                angles.append(a)
        rs = set(self.rot)
        self.other = [i for i in range(len(gates)) if i not in rs]
        self.angles = _stack_angles(angles)
        self.kinds = np.array([_KIND[gates[i].name] for i in self.rot], dtype=np.int64)

    def args(self):
        return (self.angles, *[self.mats[i] for i in self.other])

    def need(self, needs_input_grad, first):
        """Per gate, what the reverse sweep computes (``_Runner.reverse``), from
        the Function's ``needs_input_grad`` (angles at ``first``, other matrices
        after): ("rotation", kind), True for a matrix block, or False."""
        need = [False] * len(self.mats)
        if needs_input_grad[first]:
            for i, k in zip(self.rot, self.kinds):
                need[i] = ("rotation", int(k))
        for j, i in enumerate(self.other):
            need[i] = bool(needs_input_grad[first + 1 + j])
        return need

    def grads(self, blocks, scale, needs_input_grad, first):
        """Gradients for ``args()`` from the sweep's outputs times ``scale`` (the
        factor that turns a block into dL/dM): a rotation's Im <lam|P|phi> times
        ``scale`` is Re sum conj(dL/dM) dM/dtheta, its angle's gradient."""
        g_ang = None
        if needs_input_grad[first] and self.rot:
            out = np.array([scale * blocks[i] for i in self.rot], dtype=np.float64)
            g_ang = torch.from_numpy(out).to(self.angles.device)
        rest = [None if blocks[i] is None else _grad_like(self.mats[i], scale * blocks[i]) for i in self.other]
        return (g_ang, *rest)


class _StateFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, runner, inputs, *args):
        psi = runner.forward_state(inputs.mats, inputs.flat)
        ctx.runner, ctx.inputs = runner, inputs
        ctx.save_for_backward(psi)
        return psi

    @staticmethod
    def backward(ctx, g_psi):
        (psi,) = ctx.saved_tensors
        runner, inputs = ctx.runner, ctx.inputs
        need = inputs.need(ctx.needs_input_grad, 2)
        lam = g_psi.detach().to(runner.dtype).contiguous().clone()
        blocks = runner.reverse(psi, lam, inputs.mats, need)
        return (None, None, *inputs.grads(blocks, 1.0, ctx.needs_input_grad, 2))


class _EnergyFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, runner, terms, inputs, *args):
        from .statevector import pauli_expectations
        psi = runner.forward_state(inputs.mats, inputs.flat)
        e = pauli_expectations(psi, runner.n, terms).sum()
        ctx.runner, ctx.terms, ctx.inputs = runner, terms, inputs
        ctx.save_for_backward(psi)
        return e

    @staticmethod
    def backward(ctx, g_e):
        (psi,) = ctx.saved_tensors
        runner, terms, inputs = ctx.runner, ctx.terms, ctx.inputs
        L = _lib.lib()
        n = runner.n
        lam = torch.empty_like(psi)
        strings = "".join(s.lower() for _, s in terms).encode()
        coeff = _lib.double_array([c for c, _ in terms])
        _lib.check(L.qgb_pauli_apply(psi.data_ptr(), lam.data_ptr(), runner.code, n, strings, coeff, len(terms), 1, 0,
                                     _lib.stream_ptr(runner.device)), "pauli_apply")
        need = inputs.need(ctx.needs_input_grad, 3)
        blocks = runner.reverse(psi, lam, inputs.mats, need)
        return (None, None, None, *inputs.grads(blocks, 2.0 * float(g_e), ctx.needs_input_grad, 3))


_GEN_T = {k: torch.from_numpy(m) for k, m in _GEN.items()}


def _matrices(gates, closed_form=False):
    """Every gate's matrix as a torch tensor, and all of them flattened into one
    complex128 host array (row-major, gate after gate). With ``closed_form``,
    rotation gates whose matrix has not been built yet (torch angles, see
    ``ParamGate``) get cos(theta) I - i sin(theta) P from their construction-time
    angles, all of a kind in one vectorised step, instead of one ``matrix_exp``
    each; the two differ by the series truncation of ``matrix_exp`` (about
    2e-10), far below complex64 rounding, so the complex64 paths use it."""
    mats = [None] * len(gates)
    sizes = np.array([4 ** len(g.indices) for g in gates], dtype=np.int64)
    offs = np.concatenate([[0], np.cumsum(sizes)])
    flat = np.empty(int(offs[-1]), dtype=np.complex128)
    if closed_form:
        by_kind = {}
        for i, g in enumerate(gates):
            kind = _KIND.get(getattr(g, "name", None))
            if kind is not None and getattr(g, "matrix_pending", lambda: False)() and _rotation_angle(g) is not None:
                by_kind.setdefault(kind, []).append(i)
        for kind, idx in by_kind.items():
            if all(gates[i].angles_unchanged() for i in idx):
                # the live angles hold the construction-time values: one gather when they
                # are views of one parameter tensor
                th = _stack_angles([gates[i].angles[0] for i in idx]).detach()
            else:
                vals = [gates[i].angle_values()[0].reshape(()).to(torch.float64) for i in idx]
                try:
                    th = torch.stack(vals).cpu()  # one copy when the angles share a device
                except RuntimeError:
                    th = torch.stack([v.cpu() for v in vals])
            gen = _GEN_T[kind]
            eye = torch.eye(gen.shape[0], dtype=torch.complex128)
            m = torch.cos(th)[:, None, None] * eye - 1j * torch.sin(th)[:, None, None] * gen
            dd = gen.shape[0] ** 2
            ia = np.asarray(idx)
            flat[(offs[ia][:, None] + np.arange(dd)[None, :]).reshape(-1)] = m.numpy().reshape(-1)
            for i, v in zip(idx, m.unbind(0)):
                mats[i] = v
    shared: dict = {}  # one tensor per distinct host matrix object (fixed gates repeat theirs)
    for i, g in enumerate(gates):
        if mats[i] is None:
            gm = g.matrix
            if torch.is_tensor(gm):
                mats[i] = gm
                flat[offs[i]:offs[i + 1]] = gm.detach().reshape(-1).to("cpu", torch.complex128).numpy()
            else:
                hit = shared.get(id(gm))
                if hit is None or hit[0] is not gm:
                    a = np.asarray(gm, dtype=np.complex128)
                    hit = shared[id(gm)] = (gm, torch.as_tensor(a), a.reshape(-1))
                mats[i] = hit[1]
                flat[offs[i]:offs[i + 1]] = hit[2]
    return mats, flat


def run_with_adjoint(sim):
    """Differentiable ``StatevectorSim.run``: the returned state carries an
    adjoint backward to every gate matrix (or rotation angle) that requires grad."""
    gates = _gate_list(sim)
    inputs = _Inputs(gates, closed_form=sim.dtype == torch.complex64)
    return _StateFn.apply(_Runner(sim, gates), inputs, *inputs.args())


def adjoint_energy(sim, terms):
    """Differentiable ``sum_t c_t <psi|P_t|psi>`` (float64) of ``sim``'s circuit."""
    gates = _gate_list(sim)
    inputs = _Inputs(gates, closed_form=sim.dtype == torch.complex64)
    return _EnergyFn.apply(_Runner(sim, gates), list(terms), inputs, *inputs.args())


# ------------------------------------------------------------ parameter-set batches


def plan_fused_forward(n, gate_bits, fixed, width, itemsize):
    """The forward pass of a parametrised gate structure as fused blocks of
    ``width`` qubits in tile sweeps. The block structure is planned once (the
    fusion compiler on the gate bits ``gate_bits`` -- flat bits in matrix order
    per gate -- with the fixed gates' matrices ``fixed`` ((gate, matrix) pairs)
    and unit placeholders for the rotations, which are unitary at every angle);
    each call then composes every parameter set's block matrices on the device
    (``qgb_fuse_blocks``, float64 products) from that set's gate matrices, laid
    out [set][gate][16]. Returns the tables of one set -- ``blocks1`` (block
    matrix at element ``out`` of the set's ``total``), ``ents1`` (gate g's matrix
    at element 16 g) -- and the sweeps as (low bits, high bits, [(tile positions,
    block offset)]), or None when the plan is not all device-fused tile sweeps
    (blocks wider than the sweep kernels take: 5 qubits for complex64, 4 for
    complex128)."""
    from .compiler import Recipe, SweepStep
    from .engine import _FUSE_BLOCK, _FUSE_ENTRY
    G = len(gate_bits)
    fixed_m = dict(fixed)
    ops = [Op(gate_bits[g], fixed_m[g] if g in fixed_m else np.eye(2 ** len(gate_bits[g]), dtype=np.complex128))
           for g in range(G)]
    plan = compile_ops(ops, n, mode="sweep", width=width, tile_bits=13,
                       max_sweep_k=min(width, 5 if itemsize <= 8 else 4), itemsize=itemsize, device_fusion=True)
    if not plan.matrices or not all(isinstance(m, Recipe) for m in plan.matrices) or \
            not all(isinstance(st, SweepStep) for st in plan.steps):
        return None
    offs, total, ents1 = [], 0, []
    blocks1 = np.zeros(len(plan.matrices), dtype=_FUSE_BLOCK)
    for i, r in enumerate(plan.matrices):
        offs.append(total)
        pos_of = {b: j for j, b in enumerate(r.bits)}
        blocks1[i] = (total, len(r.bits), len(ents1), len(ents1) + len(r.entries), 0)
        for mi, obits in r.entries:
            ents1.append((len(obits), [pos_of[b] for b in obits] + [0] * (6 - len(obits)), 0, mi * 16))
        total += 4 ** len(r.bits)
    ents1 = np.array(ents1, dtype=_FUSE_ENTRY)
    sweeps = [(st.low_bits, list(st.high_bits), [(list(pos), offs[mi]) for pos, mi in st.ops]) for st in plan.steps]
    tmpl = np.zeros((G, 16), dtype=np.complex128)
    for g, m in fixed:
        tmpl[g, :m.size] = m.reshape(-1)
    return {"blocks1": blocks1, "ents1": ents1, "total": total, "sweeps": sweeps, "template": tmpl,
            "passes": len(plan.steps), "blocks": len(plan.matrices)}


def fused_tables(fplan, nsets, ngates):
    """The block and entry tables of ``nsets`` parameter sets, one host byte
    buffer: set s's blocks write at ``s * total`` and read its gate matrices at
    ``s * ngates * 16``. Returns (buffer, byte offset of the entries)."""
    blocks = np.tile(fplan["blocks1"], nsets)
    ents = np.tile(fplan["ents1"], nsets)
    nb1, ne1 = len(fplan["blocks1"]), len(fplan["ents1"])
    s = np.repeat(np.arange(nsets, dtype=np.int64), nb1)
    blocks["out"] += s * fplan["total"]
    blocks["op_begin"] += (s * ne1).astype(np.int32)
    blocks["op_end"] += (s * ne1).astype(np.int32)
    ents["mat"] += np.repeat(np.arange(nsets, dtype=np.int64), ne1) * (ngates * 16)
    pad = (-blocks.nbytes) % 16
    return np.concatenate([blocks.view(np.uint8), np.zeros(pad, np.uint8), ents.view(np.uint8)]), blocks.nbytes + pad


class BatchedAnsatz:
    """Energies and angle gradients of one parametrised circuit structure for
    many parameter sets at once (the reference differentiates one set at a time
    through torch autograd, ``applications/compilation.py:73-133``).

    ``gates``: ``(name, indices, p)`` per gate in execution order, ``name`` one of
    RX RY RZ RXX RYY RZZ with angle parameter index ``p``, or ``("fixed",
    indices, matrix)``. Gate matrices of every set are built on the device from
    the parameter tensor (``qgb_param_matrices``: ``expm(-i theta P)`` as in
    ``core/param_gates.py``); the forward pass applies each gate to all sets in
    one launch with per-set matrices; the reverse sweep (``lam = H psi``, then
    one step per gate over all sets: ``qgb_adjoint_step_rotation`` for a
    rotation, which also reduces its angle derivative 2 Im <lam|P|phi>, and
    ``qgb_adjoint_step_batched`` for a fixed gate) carries all sets together;
    ``qgb_param_grads`` sums the derivatives of the gates of each parameter.
    With ``tile_bits`` > 0 (the default) both directions run as tile passes,
    many gates per read of the states: the forward as blocks of
    ``fused_width`` qubits (default 4) composed per set on the device and
    applied through ``qgb_apply_sweep`` with every set's own block matrices
    (``fused_width=0``, or very many sets of small states: one op per gate),
    the reverse through ``qgb_adjoint_sweep_step``; ``tile_bits=0`` runs one
    pass per gate.
    Memory: three states per set."""

    def __init__(self, n, gates, nparams=None, dtype=torch.complex64, device="cuda", tile_bits=None,
                 fused_width=4):
        self.n = int(n)
        self.dtype, self.device = dtype, torch.device(device)
        if self.device.type != "cuda":
            raise _lib.QgbError("qaravan_gb300 runs on CUDA devices only")
        self.code = _lib.dtype_code(dtype)
        self.gates = [(g[0], [int(q) for q in g[1]], g[2]) for g in gates]
        kinds, pidx, fixed = [], [], []
        for i, (name, idx, p) in enumerate(self.gates):
            if len(idx) > 2:
                raise NotImplementedError("the adjoint sweep handles gates on one or two sites")
            if name == "fixed":
                kinds.append(0)
                pidx.append(0)
                fixed.append((i, np.asarray(p, dtype=np.complex128)))
            else:
                if _KIND[name] >= 4 and len(idx) != 2 or _KIND[name] < 4 and len(idx) != 1:
                    raise ValueError(f"{name} on {len(idx)} sites")
                kinds.append(_KIND[name])
                pidx.append(int(p))
        self.nparams = int(nparams) if nparams is not None else max([p for k, p in zip(kinds, pidx) if k] + [-1]) + 1
        self._kinds = torch.tensor(kinds, dtype=torch.int32, device=self.device)
        self._pidx = torch.tensor(pidx, dtype=torch.int32, device=self.device)
        self._fixed = fixed
        # one gate-matrix row per gate: the fixed gates' matrices in place, rotations
        # left for qgb_param_matrices; copied to every parameter set in one step
        tmpl = np.zeros((len(gates), 16), dtype=np.complex128)
        for i, m in fixed:
            tmpl[i, :m.size] = m.reshape(-1)
        self._template = torch.from_numpy(tmpl).to(self.dtype).to(self.device)
        by_param = [[] for _ in range(self.nparams)]
        for g, (k, p) in enumerate(zip(kinds, pidx)):
            if k:
                by_param[p].append(g)
        ptr = np.cumsum([0] + [len(b) for b in by_param]).astype(np.int32)
        self._csr_ptr = torch.from_numpy(ptr).to(self.device)
        flat = np.array([g for b in by_param for g in b] or [0], dtype=np.int32)
        self._csr_gate = torch.from_numpy(flat).to(self.device)
        self._sites = [_lib.int_array(idx) for _, idx, _ in self.gates]
        self._need = [k != 0 for k in kinds]
        self._gens = [_GEN_C[k] if k else None for k in kinds]
        self._kinds_h = kinds
        self.scratch = Scratch(self.device)
        # tile passes (tile_bits=0: one pass per gate). Forward: the sweep kernel with
        # every set's own matrices; reverse: the adjoint sweep, derivative slot = gate index.
        self.tile_bits = _tile_bits(dtype) if tile_bits is None else int(tile_bits)
        self._fwd, self._rev = [], []
        self._fused = None
        if self.tile_bits > 0:
            bits = [[self.n - 1 - q for q in idx] for _, idx, _ in self.gates]
            if fused_width:
                isz = torch.empty(0, dtype=self.dtype).element_size()
                self._fused = plan_fused_forward(self.n, bits, fixed, int(fused_width), isz)
            if self._fused is not None:
                L = _lib.lib()
                if L.qgb_fuse_block_bytes() != self._fused["blocks1"].itemsize or \
                        L.qgb_fuse_entry_bytes() != self._fused["ents1"].itemsize:
                    raise _lib.QgbError("fusion table layout mismatch with the library")
                self._fused["template_dev"] = torch.from_numpy(self._fused["template"]).to(self.device)
                self._fused["sweep_structs"] = [_forward_sweep_struct_pos(lo, high, ops)
                                                for lo, high, ops in self._fused["sweeps"]]
            # one tile-pass op per gate: the forward without fusion, and the fallback for very many sets
            fwd_tile = min(self.tile_bits + 1, self.n)  # one state only: twice the tile of the reverse pass
            for lo, high, ops in _plan_reverse([(g, bits[g]) for g in range(len(bits))], self.n, fwd_tile):
                self._fwd.append(_forward_sweep_struct(lo, high, [(b, g * 16) for g, b in ops]))
            tile = min(self.tile_bits, self.n)
            for lo, high, ops in _plan_reverse([(g, bits[g]) for g in reversed(range(len(bits)))], self.n, tile):
                self._rev.append(_adjoint_sweep_struct(lo, high, [(b, g * 16, g if kinds[g] else -1, kinds[g])
                                                                  for g, b in ops]))

    def _use_fused(self, P):
        """Whether ``P`` sets take the fused forward: it composes every set's blocks
        from the sets' complex128 gate matrices (256 bytes per gate and set), a
        buffer kept at most 2 GiB or the size of the states themselves -- for very
        many sets of small states the per-gate forward runs instead."""
        if self._fused is None:
            return False
        need = P * len(self.gates) * 256
        states = P * (2 ** self.n) * torch.empty(0, dtype=self.dtype).element_size()
        return need <= max(1 << 31, states)

    def _fused_tables(self, P):
        """Device copy of the fused forward's tables for ``P`` sets (kept for the
        next call with the same ``P``)."""
        f = self._fused
        if f.get("sets") != P:
            host, f["ent_start"] = fused_tables(f, P, len(self.gates))
            f["tables"] = torch.from_numpy(host).to(self.device)
            f["sets"] = P
        return f["tables"]

    def _forward_fused(self, psi, params, P, st):
        """Composes every set's block matrices and applies the fused sweeps to the
        ``P`` states in ``psi`` (|0> on entry)."""
        L = _lib.lib()
        f = self._fused
        G, N = len(self.gates), 2 ** self.n
        tables = self._fused_tables(P)
        opm = f["template_dev"].unsqueeze(0).expand(P, G, 16).contiguous()
        _lib.check(L.qgb_param_matrices(self._kinds.data_ptr(), self._pidx.data_ptr(), G, params.data_ptr(),
                                        self.nparams, P, opm.data_ptr(), _lib.QGB_C128, 16, 16 * G, st),
                   "param_matrices")
        fused = torch.empty(P * f["total"], dtype=self.dtype, device=self.device)
        _lib.check(L.qgb_fuse_blocks(fused.data_ptr(), self.code, fused.numel(), tables.data_ptr(),
                                     P * len(f["blocks1"]), tables.data_ptr() + f["ent_start"],
                                     P * len(f["ents1"]), opm.data_ptr(), opm.numel(), st), "fuse_blocks")
        for sw in f["sweep_structs"]:
            _lib.check(L.qgb_apply_sweep(psi.data_ptr(), self.code, self.n, C.byref(sw), fused.data_ptr(),
                                         f["total"], P, N, st), "apply_sweep")

    @classmethod
    def hea(cls, n, layers, dtype=torch.complex64, device="cuda", fused_width=4):
        """The hardware-efficient ansatz of the adjoint benchmark: per layer RY(theta)
        then RZ(phi) on every qubit, then a CNOT ladder; parameter index
        2 * (l * n + q) + (0 theta, 1 phi), the flattening of ``workloads.hea_params``."""
        from .gates import CNOT
        gates = []
        for l in range(layers):
            for q in range(n):
                gates.append(("RY", [q], 2 * (l * n + q)))
                gates.append(("RZ", [q], 2 * (l * n + q) + 1))
            for q in range(n - 1):
                g = CNOT([q + 1, q], n)  # the gate object of workloads.hea_circuit (its own site order)
                gates.append(("fixed", list(g.indices), np.asarray(g.matrix, dtype=np.complex128)))
        return cls(n, gates, nparams=2 * layers * n, dtype=dtype, device=device, fused_width=fused_width)

    def _matrices(self, params, P):
        G = len(self.gates)
        mats = self._template.unsqueeze(0).expand(P, G, 16).contiguous()
        _lib.check(_lib.lib().qgb_param_matrices(self._kinds.data_ptr(), self._pidx.data_ptr(), G, params.data_ptr(),
                                                 self.nparams, P, mats.data_ptr(), self.code, 16, 16 * G,
                                                 _lib.stream_ptr(self.device)), "param_matrices")
        return mats

    def energy_and_grad(self, params, terms):
        """``params``: (P, nparams) float64 (device or host). Returns float64 device
        tensors ``E`` (P,) = sum_t c_t <psi|P_t|psi> and ``dE/dparams`` (P, nparams)."""
        from .statevector import pauli_expectations
        L = _lib.lib()
        n, N = self.n, 2 ** self.n
        params = torch.as_tensor(params, dtype=torch.float64).to(self.device).contiguous()
        P = params.shape[0]
        if P < 1 or P > 65535:
            raise ValueError("1 to 65535 parameter sets")
        mats = self._matrices(params, P)
        st = _lib.stream_ptr(self.device)
        isz = mats.element_size()
        psi = torch.empty(P * N, dtype=self.dtype, device=self.device)
        _lib.check(L.qgb_init_basis(psi.data_ptr(), self.code, n, 0, P, N, st), "init")
        base = mats.data_ptr()
        set_stride = 16 * len(self.gates)
        if self._use_fused(P):
            self._forward_fused(psi, params, P, st)
        elif self._fwd:
            for sw in self._fwd:
                _lib.check(L.qgb_apply_sweep(psi.data_ptr(), self.code, n, C.byref(sw), base, set_stride, P, N, st),
                           "apply_sweep")
        else:
            for g, (_, idx, _) in enumerate(self.gates):
                _lib.check(L.qgb_op_action(psi.data_ptr(), self.code, n, self._sites[g], len(idx), base + g * 16 * isz,
                                           set_stride, P, N, st), "op_action")
        terms = list(terms)
        E = pauli_expectations(psi, n, terms, batch=P, stride=N).reshape(P, -1).sum(dim=1)
        lam = torch.empty_like(psi)
        strings = "".join(s.lower() for _, s in terms).encode()
        coeff = _lib.double_array([c for c, _ in terms])
        _lib.check(L.qgb_pauli_apply(psi.data_ptr(), lam.data_ptr(), self.code, n, strings, coeff, len(terms), P, N, st),
                   "pauli_apply")
        phi = psi  # uncomputed in place
        gvals = torch.zeros(len(self.gates) * P, dtype=torch.float64, device=self.device)  # [gate][set]
        nbytes = L.qgb_reduce_scratch_bytes(n, 32, P)
        if self._rev:
            nbytes = max(nbytes, L.qgb_adjoint_sweep_scratch_bytes(n, min(self.tile_bits, n), 64, P))
        scr = self.scratch.get(nbytes)
        for sw in self._rev:
            _lib.check(L.qgb_adjoint_sweep_step(phi.data_ptr(), lam.data_ptr(), self.code, n, C.byref(sw), base,
                                                set_stride, P, N, gvals.data_ptr(), scr.data_ptr(), nbytes, st),
                       "adjoint_sweep_step")
        for g in (range(len(self.gates) - 1, -1, -1) if not self._rev else ()):
            idx = self.gates[g][1]
            op = base + g * 16 * isz
            if self._need[g]:
                _lib.check(L.qgb_adjoint_step_rotation(phi.data_ptr(), lam.data_ptr(), self.code, n, self._sites[g],
                                                       len(idx), op, set_stride, self._gens[g], P, N,
                                                       gvals.data_ptr() + g * P * 8, scr.data_ptr(), nbytes, st),
                           "adjoint_step_rotation")
            else:
                _lib.check(L.qgb_adjoint_step_batched(phi.data_ptr(), lam.data_ptr(), self.code, n, self._sites[g],
                                                      len(idx), op, set_stride, P, N, None, scr.data_ptr(), nbytes,
                                                      st), "adjoint_step_batched")
        grad = torch.empty(P, self.nparams, dtype=torch.float64, device=self.device)
        # dE/dtheta = 2 Im <lam|P|phi> per gate (lam = H psi), summed over the gates of each parameter
        _lib.check(L.qgb_param_grads(self._csr_ptr.data_ptr(), self._csr_gate.data_ptr(), self.nparams, P,
                                     gvals.data_ptr(), 2.0, grad.data_ptr(), st), "param_grads")
        return E, grad
