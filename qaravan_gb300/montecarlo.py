"""Monte-Carlo Pauli-channel trajectories, many samples at once on the GPU.

Mirrors ``MonteCarloSim`` (``tensorQ/monte_carlo_sim.py:3-35``) and
``trotter_mc_sim`` (``applications/trotter.py:61-78``): after every layer of
the (built) circuit, a noise layer sampled from ``nm`` -- a ``PauliNoise``
(``core/noise.py:90-164``) or ``PauliLindbladNoise`` (``:166-210``), whose
``sample`` returns the X/Y/Z gates of one Pauli string on sites
``0 .. nm.num_sites - 1``. The reference runs one CPU statevector per sample;
here ``expectation_samples`` runs ``num_samples`` states as one batch: each
circuit layer is one fused pass over the whole batch (same matrices for every
sample), each noise layer one ``qgb_pauli_layer`` pass applying every sample's
own string. Noise strings are drawn on the host from ``rng`` in the order
(sample, layer), the same stream ``circuit_sample`` consumes one sample at a
time. With ``inverse=True`` layers come from ``PauliLindbladNoise.inv_sample``
and each sample carries the product of its layers' quasi-probability
prefactors (probabilistic error cancellation).
"""
from __future__ import annotations

import copy

import numpy as np
import torch

from . import _lib
from .compiler import compile_ops
from .engine import Executor
from .gates import pauli_string_to_gates
from .noise import PauliLindbladNoise, PauliNoise
from .paulis import pauli_masks, pauli_multiply
from .statevector import gates_to_ops, pauli_expectations

_MAX_BATCH = 65535


def _string_masks(strings, n):
    """(xmask, zmask, n_y) of each Pauli string on sites 0.. of an n-site state."""
    out = np.zeros((len(strings), 3), dtype=np.int64)
    for i, s in enumerate(strings):
        out[i] = pauli_masks(s + 'i' * (n - len(s)))
    return out


class MonteCarloSim:
    def __init__(self, circ, init_state=None, nm=None, dtype=torch.complex64, device="cuda"):
        self.circ = circ.copy() if hasattr(circ, "copy") else copy.deepcopy(circ)
        self.num_sites = circ.num_sites
        self.init_state = init_state
        self.nm = nm
        self.dtype = dtype
        self.device = torch.device(device)
        if self.device.type != "cuda":
            raise _lib.QgbError("qaravan_gb300 runs on CUDA devices only")
        self._layer_execs = None

    # ------------------------------------------------------------ sampling
    def _layers(self):
        c = self.circ.copy() if hasattr(self.circ, "copy") else copy.deepcopy(self.circ)
        if not getattr(c, "built", False):
            c.decompose()
            c.construct_layers()
        return c.layers

    def sample_noise(self, num_samples, num_layers, rng=None, inverse=False):
        """Noise strings (num_samples x num_layers, n-site strings padded with 'i')
        and, for ``inverse``, each sample's prefactor."""
        rng = np.random.default_rng() if rng is None else rng
        nm, n = self.nm, self.num_sites
        S, L = int(num_samples), int(num_layers)
        pref = np.ones(S)
        if isinstance(nm, PauliNoise) and not inverse:
            idx = rng.choice(len(nm.strings), p=np.asarray(nm.probs, dtype=float), size=(S, L))
            strings = np.array(nm.strings, dtype=object)[idx]
        elif isinstance(nm, PauliLindbladNoise):
            fired = rng.random((S, L, len(nm.rates))) < np.asarray(nm.rates)
            strings = np.empty((S, L), dtype=object)
            for s in range(S):
                for l in range(L):
                    out = 'i' * nm.num_sites
                    for st, f in zip(nm.strings, fired[s, l]):
                        if f:
                            out, _ = pauli_multiply(out, st)
                    strings[s, l] = out
                    if inverse:
                        pref[s] *= nm.gamma * (-1) ** (out != 'i' * nm.num_sites)
        else:
            raise NotImplementedError("MonteCarloSim samples PauliNoise or PauliLindbladNoise (inverse: Lindblad only)")
        strings = np.vectorize(lambda x: x + 'i' * (n - len(x)), otypes=[object])(strings)
        return strings, pref

    def circuit_sample(self, rng=None):
        """One sampled circuit: every layer followed by a sampled noise layer
        (``monte_carlo_sim.py:14-28``)."""
        layers = self._layers()
        c = self.circ.copy() if hasattr(self.circ, "copy") else copy.deepcopy(self.circ)
        if self.nm is not None:
            strings, _ = self.sample_noise(1, len(layers), rng)
            noise = [pauli_string_to_gates(s) for s in strings[0]]
            layers = [x for pair in zip(layers, noise) for x in pair]
        c.layers = layers
        c.built = True
        return c

    # ------------------------------------------------------------ running
    def _execs(self):
        if self._layer_execs is None:
            isz = torch.empty(0, dtype=self.dtype).element_size()
            self._layer_execs = []
            for layer in self._layers():
                ops = gates_to_ops(layer, self.num_sites)
                plan = compile_ops(ops, self.num_sites, mode="fused", width=6, itemsize=isz, device_fusion=True)
                self._layer_execs.append(Executor(plan, self.dtype, self.device))
        return self._layer_execs

    def _init_states(self, S):
        n = self.num_sites
        st = torch.empty(S * 2 ** n, dtype=self.dtype, device=self.device)
        if self.init_state is None or isinstance(self.init_state, str):
            idx = 0 if self.init_state is None else int(self.init_state, 2)
            L = _lib.lib()
            for b0 in range(0, S, _MAX_BATCH):
                nb = min(_MAX_BATCH, S - b0)
                _lib.check(L.qgb_init_basis(st.data_ptr() + b0 * 2 ** n * st.element_size(), _lib.dtype_code(self.dtype),
                                            n, idx, nb, 2 ** n, _lib.stream_ptr(self.device)), "init_basis")
        else:
            v = torch.as_tensor(np.asarray(self.init_state) if not torch.is_tensor(self.init_state) else self.init_state)
            st.view(S, 2 ** n).copy_(v.reshape(1, -1).to(self.dtype))
        return st

    def _apply_layers(self, st, S, strings):
        n = self.num_sites
        L = _lib.lib()
        masks = torch.from_numpy(np.stack([_string_masks(strings[:, l], n) for l in range(strings.shape[1])]))
        xm = masks[:, :, 0].contiguous().to(self.device)
        zm = masks[:, :, 1].contiguous().to(self.device)
        ny = masks[:, :, 2].to(torch.int32).contiguous().to(self.device)
        for l, ex in enumerate(self._execs()):
            for b0 in range(0, S, _MAX_BATCH):
                nb = min(_MAX_BATCH, S - b0)
                part = st[b0 * 2 ** n:(b0 + nb) * 2 ** n]
                ex.run(part, batch=nb, stride=2 ** n)
                _lib.check(L.qgb_pauli_layer(part.data_ptr(), _lib.dtype_code(self.dtype), n,
                                             xm[l, b0:].data_ptr(), zm[l, b0:].data_ptr(), ny[l, b0:].data_ptr(),
                                             nb, 2 ** n, _lib.stream_ptr(self.device)), "pauli_layer")
        return st

    def _evaluate(self, st, S, obs):
        n = self.num_sites
        if isinstance(obs, (list, tuple)):  # Pauli sum [(coeff, 'ixyz...'), ...]
            vals = torch.zeros(S, dtype=torch.float64, device=self.device)
            for b0 in range(0, S, _MAX_BATCH):
                nb = min(_MAX_BATCH, S - b0)
                e = pauli_expectations(st[b0 * 2 ** n:(b0 + nb) * 2 ** n], n, obs, batch=nb, stride=2 ** n)
                vals[b0:b0 + nb] = e.reshape(nb, -1).sum(dim=1)
            return vals.cpu().numpy()
        o = torch.as_tensor(np.asarray(obs)).to(device=self.device, dtype=torch.complex128)
        psi = st.view(S, 2 ** n).to(torch.complex128)
        return torch.einsum("si,si->s", psi.conj(), psi @ o.T).real.cpu().numpy()

    def expectation_samples(self, obs, num_samples, rng=None, inverse=False):
        """Per-sample <obs> (``obs``: a dense 2^n x 2^n matrix, as the reference
        takes, or a Pauli sum ``[(coeff, string), ...]``); with ``inverse``,
        returns ``(values, prefactors)``."""
        S = int(num_samples)
        layers = self._layers()
        strings, pref = self.sample_noise(S, len(layers), rng, inverse)
        st = self._apply_layers(self._init_states(S), S, strings)
        vals = self._evaluate(st, S, obs)
        return (vals, pref) if inverse else vals

    def expectation_sample(self, obs, rng=None):
        """One sample (``monte_carlo_sim.py:30-35``)."""
        return float(self.expectation_samples(obs, 1, rng)[0])


def trotter_mc_sim(ham, step_size, max_steps, channel, op, num_samples=1000, rng=None, dtype=torch.complex64):
    """``trotter_mc_sim`` (``applications/trotter.py:61-78``): ``num_samples``
    states evolved one Trotter step at a time, a fresh noise sample per step and
    sample; returns the mean <op> after each step."""
    circ = ham.trotter_circ(step_size, 1)
    sim = MonteCarloSim(circ, nm=channel, dtype=dtype)
    rng = np.random.default_rng() if rng is None else rng
    S = int(num_samples)
    st = sim._init_states(S)
    out = []
    nlayers = len(sim._layers())
    for _ in range(int(max_steps)):
        strings, _ = sim.sample_noise(S, nlayers, rng)
        sim._apply_layers(st, S, strings)
        out.append(float(np.mean(sim._evaluate(st, S, op))))
    return out
