"""Environment tensors and environment-based state preparation on the GPU.

Mirrors ``tensorQ/environments.py:7-80``: the environment of gate ``i`` is the
partial overlap of the state before it and the state after it pulled back from
the target, ``partial_overlap(pre, post, skip=indices)``
(``tensorQ/statevector_sim.py:155-180``, skipped sites ascending); the
optimal unitary replacing the gate is ``yh^H x^H`` from its SVD, and the sweep
updates the two states by one gate each. Here both states stay on the device:
the environment is one ``qgb_partial_overlap`` pass (float64), the state
updates are ``qgb_op_action`` passes, and only the 2^k x 2^k environment
crosses to the host for its SVD. ``RunContext`` keeps the reference's
iteration control (``core/utils.py:144-232``) without checkpoint files.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib
from .circuits import two_local_circ
from .statevector import StatevectorSim, inner_product


class RunContext:
    """Iteration control of ``core/utils.py:144-232``: ``max_iter``, progress
    log, and the plateau / absolute stop rules; ``run_state`` may be given to
    resume in the same process (checkpoint files are not written)."""

    def __init__(self, progress_interval=10, max_iter=1000, resume=False, convergence_check=False, stop_ratio=1e-6,
                 stop_absolute=None, quiet=False, run_state=None):
        self.progress_interval, self.max_iter = progress_interval, max_iter
        self.resume = bool(resume and run_state is not None)
        self.convergence_check, self.stop_ratio, self.stop_absolute = convergence_check, stop_ratio, stop_absolute
        self.quiet = quiet
        self.run_state = run_state
        self.step = run_state.get("step", 0) if (self.resume and isinstance(run_state, dict)) else 0
        self.term_msg = ""

    def log(self, msg):
        if not self.quiet:
            print(msg, flush=True)

    def step_update(self, run_state):
        self.run_state = run_state
        self.step = run_state.get("step", self.step)
        if self.step % self.progress_interval == 0 and run_state.get("cost_list"):
            self.log(f"Step {self.step} with cost {run_state['cost_list'][-1]}")
        if self.step >= self.max_iter:
            self.term_msg = "Max iterations reached."
            self.log(self.term_msg)
            return True
        return self.check_convergence() if self.convergence_check else False

    def check_convergence(self):
        cl = self.run_state.get("cost_list")
        if len(cl) < 2:
            return False
        if abs(cl[-1] - cl[-2]) < self.stop_ratio * abs(cl[-2]):
            self.term_msg = f"Plateau detected with cost {cl[-1]} at step {self.step}"
            self.log(self.term_msg)
            return True
        if self.stop_absolute is not None and cl[-1] < self.stop_absolute:
            self.term_msg = f"Absolute stop condition met with cost {cl[-1]} at step {self.step}"
            self.log(self.term_msg)
            return True
        return False


class _Dev:
    """Device-side helpers for one state size and dtype."""

    def __init__(self, n, dtype, device):
        self.n, self.dtype, self.device = n, dtype, torch.device(device)
        self.code = _lib.dtype_code(dtype)
        self.nbytes = 0
        self.scratch = None
        self.out = None

    def _buffers(self, k, batch):
        """Scratch and output of a batched partial overlap on k sites, grown on demand."""
        nbytes = _lib.lib().qgb_partial_overlap_scratch_bytes(self.n, k, batch)
        if nbytes == 0:
            raise ValueError(f"partial overlap on {k} of {self.n} sites is not supported")
        if nbytes > self.nbytes:
            self.nbytes = nbytes
            self.scratch = torch.empty(nbytes // 8 + 1, dtype=torch.float64, device=self.device)
        if self.out is None or self.out.numel() < 2 * batch * 4 ** k:
            self.out = torch.empty(2 * batch * 4 ** k, dtype=torch.float64, device=self.device)

    def vec(self, v):
        t = v if torch.is_tensor(v) else torch.as_tensor(np.asarray(v))
        return t.reshape(-1).to(device=self.device, dtype=self.dtype).contiguous().clone()

    def op_action(self, mat, indices, state, batch=1):
        """In place: state <- mat on ``indices`` (``op_action``, ``statevector_sim.py:124-140``);
        ``batch`` contiguous vectors of 2^n amplitudes."""
        m = torch.as_tensor(np.asarray(mat)).to(device=self.device, dtype=self.dtype).contiguous()
        _lib.check(_lib.lib().qgb_op_action(state.data_ptr(), self.code, self.n, _lib.int_array(list(indices)),
                                            len(indices), m.data_ptr(), 0, batch, 2 ** self.n,
                                            _lib.stream_ptr(self.device)), "op_action")
        return state

    def partial_overlap(self, a, b, skip, batch=None):
        """Host complex128 ``partial_overlap(a, b, skip)``, skipped sites ascending; with
        ``batch`` set, one 2^k x 2^k matrix per pair of contiguous vectors."""
        sites = sorted(int(s) for s in skip)
        k = len(sites)
        nb = 1 if batch is None else batch
        self._buffers(k, nb)
        _lib.check(_lib.lib().qgb_partial_overlap(a.data_ptr(), b.data_ptr(), self.code, self.n, _lib.int_array(sites),
                                                  k, nb, 2 ** self.n, self.out.data_ptr(), self.scratch.data_ptr(),
                                                  self.nbytes, _lib.stream_ptr(self.device)), "partial_overlap")
        o = self.out[:2 * nb * 4 ** k].cpu().numpy()
        o = (o[0::2] + 1j * o[1::2]).reshape(nb, 2 ** k, 2 ** k)
        return o[0] if batch is None else o

    def overlap(self, a, b):
        """<a|b> (complex, host)."""
        r = inner_product(a, b, self.n).cpu().numpy()
        return complex(r[0], r[1])


def sv_environment(circ, left_sv, gate_idx, dtype=torch.complex128, device="cuda"):
    """Environment of gate ``gate_idx`` against ``left_sv`` and the gate's matrix
    (``environments.py:7-20``)."""
    mat, indices = circ[gate_idx].matrix, circ[gate_idx].indices
    n = circ.num_sites
    d = _Dev(n, dtype, device)
    sv1 = StatevectorSim(circ[:gate_idx], dtype=dtype, device=device).run().reshape(-1)
    sv2 = StatevectorSim(circ[gate_idx + 1:].dag(), init_state=d.vec(left_sv), dtype=dtype, device=device).run()
    return d.partial_overlap(sv1, sv2.reshape(-1), indices), mat


def environment_update(circ, gate_idx, pre_state, post_state, target_sv, init_sv, direction="decreasing", dev=None):
    """One environment step (``environments.py:22-46``): replace the gate by the
    best unitary for its environment and move the two device states by one
    gate. Returns ``(cost, pre_state, post_state)``."""
    d = dev if dev is not None else _Dev(circ.num_sites, pre_state.dtype, pre_state.device)
    indices = circ[gate_idx].indices
    env = d.partial_overlap(pre_state, post_state, indices)
    x, _, yh = np.linalg.svd(env)
    new_mat = yh.conj().T @ x.conj().T
    circ.update_gate(gate_idx, new_mat)
    if direction == "decreasing":
        if gate_idx == 1:
            pre_state.copy_(init_sv)
        else:
            g = circ[gate_idx - 1]
            d.op_action(np.asarray(g.matrix).conj().T, g.indices, pre_state)  # undo the gate before
        d.op_action(new_mat.conj().T, indices, post_state)
    else:
        d.op_action(new_mat, indices, pre_state)
        if gate_idx == len(circ) - 2:
            post_state.copy_(target_sv)
        else:
            g = circ[gate_idx + 1]
            d.op_action(g.matrix, g.indices, post_state)  # the gate after, pulled back
    return 1 - np.abs(np.trace(new_mat @ env)), pre_state, post_state


def environment_state_prep(target_sv, init_sv=None, circ=None, skeleton=None, context=None, quiet=True,
                           dtype=torch.complex128, device="cuda"):
    """Optimise a circuit to prepare ``target_sv`` by environment sweeps
    (``environments.py:48-80``); returns ``(circ, cost_list)``."""
    context = RunContext() if context is None else context
    if context.resume:
        circ = context.run_state["circ"]
        n = circ.num_sites
        d = _Dev(n, dtype, device)
        cost_list = context.run_state["cost_list"]
        pre_state = d.vec(context.run_state["pre_state"])
        post_state = d.vec(context.run_state["post_state"])
    else:
        if circ is None:
            circ = two_local_circ(skeleton)
        n = circ.num_sites
        d = _Dev(n, dtype, device)
        ansatz = StatevectorSim(circ, init_state=None if init_sv is None else d.vec(init_sv), dtype=dtype,
                                device=device).run().reshape(-1).clone()
        tgt = d.vec(target_sv)
        cost_list = [1 - abs(d.overlap(tgt, ansatz))]
        last = circ[-1]
        pre_state = d.op_action(np.asarray(last.matrix).conj().T, last.indices, ansatz)  # undo the last gate
        post_state = tgt.clone()
    tgt = d.vec(target_sv)
    if init_sv is None:
        init = torch.zeros(2 ** n, dtype=dtype, device=d.device)
        init[0] = 1
    else:
        init = d.vec(init_sv)
    for step in range(context.step, context.max_iter):
        for i in reversed(range(1, len(circ))):
            cost, pre_state, post_state = environment_update(circ, i, pre_state, post_state, tgt, init, "decreasing", d)
            cost_list.append(cost)
        for i in range(len(circ) - 1):
            cost, pre_state, post_state = environment_update(circ, i, pre_state, post_state, tgt, init, "increasing", d)
            cost_list.append(cost)
        run_state = {"step": step, "circ": circ, "cost_list": cost_list, "pre_state": pre_state,
                     "post_state": post_state}
        if context.step_update(run_state):
            break
    return circ, cost_list
