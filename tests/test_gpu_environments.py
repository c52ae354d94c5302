"""Environment tensors and environment-based state preparation on the device
against a NumPy restatement of tensorQ/environments.py (the oracle's op_action
and partial_overlap, numpy SVD): the environment of a gate, and two full
left/right sweeps of environment_state_prep (cost after every update and the
final gate matrices)."""
import numpy as np
import pytest

from oracle import ref

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built(cuda_ok):
    from qaravan_gb300 import build
    build.build()


def _skeleton(n):
    return [[i, i + 1] for i in range(0, n - 1, 2)] + [[i, i + 1] for i in range(1, n - 1, 2)] + \
           [[i, i + 1] for i in range(0, n - 1, 2)]


def _circ(n, seed):
    from qaravan_gb300.circuits import two_local_circ
    np.random.seed(seed)
    return two_local_circ(_skeleton(n))


def _target(n, seed):
    rng = np.random.default_rng(seed)
    v = rng.normal(size=2 ** n) + 1j * rng.normal(size=2 ** n)
    return v / np.linalg.norm(v)


def test_sv_environment_matches_oracle():
    from qaravan_gb300.environments import sv_environment
    n = 8
    circ = _circ(n, 1)
    left = _target(n, 2)
    for gi in (0, 3, len(circ) - 1):
        env, mat = sv_environment(circ, left, gi)
        sv1 = ref.run_sv(list(circ.gate_list[:gi]), n) if gi > 0 else ref.initial_sv(n).reshape(-1)
        sv2 = ref.run_sv(list(circ[gi + 1:].dag().gate_list), n, init_state=left) if gi + 1 < len(circ) else left
        want = ref.partial_overlap(sv1, sv2, skip=circ[gi].indices)
        assert np.max(np.abs(env - want)) < 1e-12
        assert mat is circ[gi].matrix


def _prep_numpy(target, circ, iters):
    """The reference's environment_state_prep (environments.py:48-80) with the oracle's kernels."""
    n = circ.num_sites
    ansatz = ref.run_sv(list(circ.gate_list), n)
    cost = [1 - abs(np.vdot(target, ansatz))]
    last = circ[-1]
    pre = ref.op_action(np.asarray(last.matrix).conj().T, last.indices, ansatz.reshape([2] * n)).reshape(-1)
    post = target.copy()
    init = ref.initial_sv(n).reshape(-1)

    def upd(i, pre, post, direction):
        idx = circ[i].indices
        env = ref.partial_overlap(pre, post, skip=idx)
        x, _, yh = np.linalg.svd(env)
        new = yh.conj().T @ x.conj().T
        circ.update_gate(i, new)
        sh = [2] * n
        if direction == "decreasing":
            pre = init.copy() if i == 1 else ref.op_action(np.asarray(circ[i - 1].matrix).conj().T,
                                                           circ[i - 1].indices, pre.reshape(sh)).reshape(-1)
            post = ref.op_action(new.conj().T, idx, post.reshape(sh)).reshape(-1)
        else:
            pre = ref.op_action(new, idx, pre.reshape(sh)).reshape(-1)
            post = target.copy() if i == len(circ) - 2 else ref.op_action(circ[i + 1].matrix, circ[i + 1].indices,
                                                                          post.reshape(sh)).reshape(-1)
        return 1 - np.abs(np.trace(new @ env)), pre, post

    for _ in range(iters):
        for i in reversed(range(1, len(circ))):
            c, pre, post = upd(i, pre, post, "decreasing")
            cost.append(c)
        for i in range(len(circ) - 1):
            c, pre, post = upd(i, pre, post, "increasing")
            cost.append(c)
    return circ, cost


def test_environment_state_prep_matches_numpy_restatement():
    from qaravan_gb300.environments import RunContext, environment_state_prep
    n = 6
    base = _circ(n, 7)
    target = _target(n, 8)
    c_gpu, cost_gpu = environment_state_prep(target, circ=base.copy(), context=RunContext(max_iter=2, quiet=True))
    c_np, cost_np = _prep_numpy(target, base.copy(), 2)
    assert len(cost_gpu) == len(cost_np)
    assert np.max(np.abs(np.array(cost_gpu) - np.array(cost_np))) < 1e-9
    for g1, g2 in zip(c_gpu.gate_list, c_np.gate_list):
        assert np.max(np.abs(np.asarray(g1.matrix) - np.asarray(g2.matrix))) < 1e-8
    assert cost_gpu[-1] < cost_gpu[0]  # the sweeps improve the fidelity
