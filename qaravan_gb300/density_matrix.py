"""``DensityMatrixSim`` on GB300: vec(rho) run by the same gate engine.

Mirrors ``tensorQ/density_matrix_sim.py:8-89``. The state is vec(rho): ``4^n``
complex entries, row (ket) site ``q`` on flat bit ``2n-1-q`` and column (bra)
site ``q`` on bit ``n-1-q`` -- the C-order flattening of the reference's
rank-2n tensor (ket axes first, ``:12-36``). A unitary ``M`` on sites ``S``
becomes ``M`` on the ket bits and ``conj(M)`` on the bra bits (the
reference's superoperator ``kron(conj M, M)``, ``core/gates.py:43-44``, split
into two cheaper ops); a noise carrier contributes its channel
superoperator ``sum kron(conj K, K)`` (``core/noise.py:10-13``) as one dense
op on the 2k bits. As in the reference's ``generate_gate_indices``
(``:91-99``), an op's input legs follow its ``indices`` and its output legs
ascending site order; for unsorted indices this is reproduced by permuting
the operator's rows.
"""
from __future__ import annotations

import itertools

import numpy as np
import torch

from . import _lib
from .compiler import Op, compile_ops
from .engine import Executor, Scratch
from .statevector import _to_np, circuit_ops, inner_product


_PAIR_IDS = itertools.count()  # ties the ket and bra halves of one gate


def _sorted_rows(mat, idx):
    """Rows of an operator whose output legs follow sorted(idx), re-indexed to idx order."""
    k = len(idx)
    srt = sorted(idx)
    if list(idx) == srt:
        return mat
    d = mat.shape[0]
    reps = d // (2 ** k)  # 1 for a gate, 2^k for a superop (bra block, ket block)
    r_new = np.arange(d)
    perm = np.zeros(d, dtype=np.int64)
    nb = int(round(np.log2(d)))
    for r in r_new:
        out = 0
        # each block of k bits (bra then ket for a superop) is reordered
        for blk in range(nb // k):
            chunk = (r >> (nb - (blk + 1) * k)) & ((1 << k) - 1)
            # chunk bits are in idx order (bit k-1-j <-> idx[j]); source row uses sorted order
            src = 0
            for p, s in enumerate(srt):
                j = list(idx).index(s)
                src |= ((chunk >> (k - 1 - j)) & 1) << (k - 1 - p)
            out |= src << (nb - (blk + 1) * k)
        perm[r] = out
    del reps
    return mat[perm, :]


def _pauli_mix_op(nm, idx, n):
    """A Pauli channel on sites ``idx`` too wide for a dense superoperator block,
    as a Pauli mixture on vec(rho): rho -> sum_k w_k P_k rho P_k^dagger is
    sum_k w_k (P_k on the ket sites) (conj(P_k) = (-1)^#Y P_k on the bra sites).
    w_k = conj(sqrt p_k) sqrt p_k with the reference's Kraus operators
    sqrt(p_k) P_k (core/noise.py:90-129, emath square root: |p_k|)."""
    terms = []
    for p, s in zip(nm.probs, nm.strings):
        r = np.emath.sqrt(p)
        w = float((np.conj(r) * r).real)
        chars = ["i"] * (2 * n)
        for j, q in enumerate(idx):
            chars[q] = s[j]  # ket site q: vec bit 2n-1-q
            chars[n + q] = s[j]  # bra site q: vec bit n-1-q
        terms.append((w * (-1) ** s.lower().count("y"), "".join(chars)))
    return Op([], None, kind="pauli_mix", terms=terms)


def dm_ops_for_gate(g, n, cache=None):
    """Ops on vec(rho) for one reference op (gate, Reset projector or noise carrier).

    ``cache`` (optional dict, valid while the noise models are not modified):
    noise superoperators already built in this op sequence, keyed by the noise
    model, gate time, dynamical-decoupling flag and site order, shared
    read-only between the carriers that use them."""
    idx = [int(q) for q in g.indices]
    ket = [2 * n - 1 - q for q in idx]
    bra = [n - 1 - q for q in idx]
    if g.name == "ID" and getattr(g, "nm", None) is not None:
        if 2 * len(idx) > 6 and hasattr(g.nm, "strings") and hasattr(g.nm, "probs"):
            return [_pauli_mix_op(g.nm, idx, n)]
        dd = getattr(g, "dd", False)
        key = (id(g.nm), g.time, bool(dd), tuple(np.argsort(idx)))
        m = cache.get(key) if cache is not None else None
        if m is None:
            s = np.asarray(g.nm.get_superop(g.time, dd), dtype=np.complex128)
            m = np.array(_sorted_rows(s.reshape(4 ** len(idx), 4 ** len(idx)), idx))
            if cache is not None:
                m.flags.writeable = False
                cache[key] = (m, g.nm)  # the model kept alive with its key
        else:
            m = m[0]
        return [Op(bra + ket, m, kind="channel")]
    if type(g).__name__ == "SuperOp":  # its matrix is the superoperator (tensorQ/density_matrix_sim.py:40)
        s = np.asarray(g.matrix, dtype=np.complex128).reshape(4 ** len(idx), 4 ** len(idx))
        return [Op(bra + ket, _sorted_rows(s, idx), kind="channel")]
    m = _sorted_rows(_to_np(g.matrix), idx)
    pair = next(_PAIR_IDS)
    return [Op(ket, m, pair=pair), Op(bra, np.conj(m), pair=pair)]


class DensityMatrixSim:
    def __init__(self, circ, init_state=None, nm=None, device="cuda", dtype=torch.complex64,
                 mode="auto", fusion_width=None, tile_bits=13, low_bits=None):
        self.circ = circ.copy() if hasattr(circ, "copy") else circ
        self.num_sites = circ.num_sites
        self.local_dim = getattr(circ, "local_dim", 2)
        if self.local_dim != 2:
            raise NotImplementedError("qaravan_gb300 supports qubits only (local_dim 2)")
        self.nm = nm
        self.init_state = init_state
        self.device = torch.device(device)
        if self.device.type != "cuda":
            raise _lib.QgbError("qaravan_gb300 runs on CUDA devices only")
        self.dtype = dtype
        # auto: complex64 vec(rho) of >= 13 bits -> 6-qubit fused blocks on the tensor cores (2.7x
        # faster than the CUDA-core tile sweep at 13 sites); otherwise 4-bit blocks in tile sweeps
        if mode == "auto":
            tc = dtype == torch.complex64 and 2 * self.num_sites >= 13 and _lib.lib().qgb_get_dense_impl() >= 1
            mode = "fused" if tc else "sweep"
            if fusion_width is None:
                fusion_width = 6 if tc else 4
        if fusion_width is None:
            fusion_width = 4
        self.mode, self.fusion_width, self.tile_bits, self.low_bits = mode, fusion_width, tile_bits, low_bits
        self.state = None
        self.ran = False
        self._exec = None
        self._scratch = Scratch(self.device)

    def initialize_state(self):
        n = self.num_sites
        if self.init_state is None or isinstance(self.init_state, str):
            idx = 0 if self.init_state is None else int(self.init_state, 2)
            self.state = torch.empty(4 ** n, dtype=self.dtype, device=self.device)
            _lib.check(_lib.lib().qgb_init_basis(self.state.data_ptr(), _lib.dtype_code(self.dtype), 2 * n,
                                                 (idx << n) | idx, 1, 0, _lib.stream_ptr(self.device)),
                       "init_basis")
        else:
            t = self.init_state if torch.is_tensor(self.init_state) else torch.from_numpy(np.asarray(self.init_state))
            self.state = t.reshape(-1).to(dtype=self.dtype, device=self.device).contiguous().clone()
            if self.state.numel() != 4 ** n:
                raise ValueError("init_state must be a 2^n x 2^n matrix or a rank-2n tensor")

    def op_sequence(self):
        c = self.circ
        if self.nm is not None and hasattr(c, "build"):
            c = c.copy() if getattr(c, "built", False) is False else c
            c.build(self.nm)
        seq = circuit_ops(c)
        n = self.num_sites
        ops = []
        cache: dict = {}
        for g in seq:
            ops.extend(dm_ops_for_gate(g, n, cache))
            if g.name == "Reset" and getattr(g, "normalize", True):
                ops.append(None)
        return ops

    def compile(self):
        if self._exec is None:
            kcap = 5 if self.dtype == torch.complex64 else 4
            plan = compile_ops(self.op_sequence(), 2 * self.num_sites, mode=self.mode, width=self.fusion_width,
                               device_fusion=True,
                               tile_bits=self.tile_bits, low_bits=self.low_bits, max_sweep_k=kcap,
                               itemsize=torch.empty(0, dtype=self.dtype).element_size())
            self._exec = Executor(plan, self.dtype, self.device, mode_normalize="dm")
        return self._exec

    def run(self, progress_bar=False, debug=0):
        self.initialize_state()
        self.compile().run(self.state)
        self.ran = True
        return self.state

    def apply_gate(self, gate):
        """``DensityMatrixSim.apply_gate`` (``:38-42``) for one op."""
        if self.state is None:
            self.initialize_state()
        n = self.num_sites
        kcap = 5 if self.dtype == torch.complex64 else 4
        plan = compile_ops(dm_ops_for_gate(gate, n), 2 * n, mode="gate", max_sweep_k=kcap)
        Executor(plan, self.dtype, self.device, mode_normalize="dm").run(self.state)

    def get_density_matrix(self):
        if not self.ran and self.state is None:
            self.run()
        d = 2 ** self.num_sites
        return self.state.reshape(d, d)

    def __str__(self):
        """rho as a mixture of pure states (``tensorQ/density_matrix_sim.py:78-80``)."""
        from .measure import pretty_print_dm
        self._ensure_ran()
        d = 2 ** self.num_sites
        return pretty_print_dm(self.state.detach().reshape(d, d).cpu().numpy())

    def normalize_state(self):
        Executor(compile_ops([], 2 * self.num_sites), self.dtype, self.device, mode_normalize="dm").normalize(self.state)

    def _ensure_ran(self):
        if not self.ran:
            self.run()

    def _reduce(self, fn, nslots, *args):
        L = _lib.lib()
        n = self.num_sites
        out = torch.empty(nslots, dtype=torch.float64, device=self.device)
        nbytes = L.qgb_reduce_scratch_bytes(2 * n, nslots, 1)
        buf = self._scratch.get(nbytes)
        _lib.check(fn(self.state.data_ptr(), _lib.dtype_code(self.dtype), n, *args, out.data_ptr(), buf.data_ptr(),
                      nbytes, _lib.stream_ptr(self.device)), fn.__name__)
        return out

    def local_expectation(self, local_ops):
        """Re Tr((x)_i O_i rho) (``:49-58``); the state is left unchanged."""
        self._ensure_ran()
        return self._product({i: local_ops[i] for i in range(self.num_sites)})

    def one_local_expectation(self, op, site):
        """Re Tr(O_site rho) (``:60-70``)."""
        self._ensure_ran()
        return self._product({site: op})

    def _product(self, site_ops):
        n = self.num_sites
        arr = np.zeros((n, 2, 2), dtype=np.complex128)
        arr[:] = np.eye(2)
        for q, o in site_ops.items():
            arr[q] = _to_np(o)
        flat = np.stack([arr.real, arr.imag], axis=-1).reshape(-1)
        ops = _lib.double_array(flat)
        L = _lib.lib()
        out = self._reduce(L.qgb_dm_product_expectation, 1, ops, 1, 0)
        return float(out[0].item())

    def pauli_expectation(self, pauli_string):
        self._ensure_ran()
        return float(self.pauli_expectations([(1.0, pauli_string)])[0].item())

    def pauli_expectations(self, terms):
        terms = list(terms)
        L = _lib.lib()
        strings = "".join(s.lower() for _, s in terms).encode()
        coeff = _lib.double_array([c for c, _ in terms])
        return self._reduce(L.qgb_dm_pauli_expectation, len(terms), strings, coeff, len(terms), 1, 0)

    def global_expectation(self, global_op):
        """Re Tr(rho O) (``:72-76``) = <vec(O^dagger) | vec(rho)>."""
        self._ensure_ran()
        n = self.num_sites
        od = torch.as_tensor(np.ascontiguousarray(_to_np(global_op).conj().T)).to(self.dtype).to(self.device)
        return float(inner_product(od.reshape(-1), self.state, 2 * n)[0].item())

    def trace(self):
        L = _lib.lib()
        return float(self._reduce(L.qgb_dm_trace, 1, 1, 0)[0].item())

    def purity(self):
        """Tr(rho^2) = ||vec rho||^2 for Hermitian rho, accumulated in float64."""
        self._ensure_ran()
        L = _lib.lib()
        n = self.num_sites
        out = torch.empty(1, dtype=torch.float64, device=self.device)
        nbytes = L.qgb_reduce_scratch_bytes(2 * n, 1, 1)
        buf = self._scratch.get(nbytes)
        _lib.check(L.qgb_norm2(self.state.data_ptr(), _lib.dtype_code(self.dtype), 2 * n, 1, 0, out.data_ptr(),
                               buf.data_ptr(), nbytes, _lib.stream_ptr(self.device)), "norm2")
        return float(out[0].item())
