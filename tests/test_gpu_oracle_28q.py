"""The benchmark's own configuration pinned to the oracle: the 28-qubit
depth-20 Haar brickwork (1100 gates) run through the reference's op_action on
the host in complex128 (torch CPU tensors, all cores; several minutes), against
the default complex64 path (6-qubit fused blocks on the tensor cores with the
norm chain, bar 1e-5) and the complex128 path (bar 1e-12).

Long: runs only with QGB_LONG=1 (the default GPU suite stays short)."""
import os

import numpy as np
import pytest
import torch

from oracle import ref

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(os.environ.get("QGB_LONG") != "1", reason="long: set QGB_LONG=1")]


def test_28_qubit_brickwork_against_the_oracle(cuda_ok):
    from qaravan_gb300 import StatevectorSim, build, workloads
    from qaravan_gb300.circuits import Circuit
    build.build()
    n = 28
    gates = workloads.brickwork_gates(n, 20, 2028)  # the benchmark's circuit (seed 2028)
    torch.set_num_threads(os.cpu_count() or 1)
    state = torch.zeros([2] * n, dtype=torch.complex128)
    state.view(-1)[0] = 1
    for g in gates:
        state = ref.op_action_torch(torch.tensor(np.asarray(g.matrix), dtype=torch.complex128), g.indices, state)
    exp = state.contiguous().reshape(-1)
    del state
    res = {}
    for name, dtype, tol in (("c64", torch.complex64, 1e-5), ("c128", torch.complex128, 1e-12)):
        sim = StatevectorSim(Circuit(gates, n=n), dtype=dtype)
        got = sim.get_statevector().reshape(-1).cpu().to(torch.complex128)
        d = (got - exp).abs()
        res[name] = {"max_abs": float(d.max()), "max_rel": float(d.max() / exp.abs().max()),
                     "l2": float(torch.linalg.vector_norm(got - exp))}
        del sim, got, d
        torch.cuda.empty_cache()
        assert res[name]["max_abs"] < tol, (name, res[name])
    print("28-qubit brickwork vs oracle:", res)
