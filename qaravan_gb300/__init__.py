"""qaravan_gb300 -- GB300 (sm_103a) engine for qaravan's tensorQ gate-application path.

Drop-in for the reference's torch backend: ``StatevectorSim``,
``DensityMatrixSim``, ``MonteCarloSim`` / ``trotter_mc_sim`` (sampled Pauli
noise), ``TrajectorySim`` (depolarising + amplitude-damping trajectories),
measurement and sampling, the adjoint gradient, and the reference's circuit /
gate / noise objects (which work
unchanged when the reference package itself is installed). All arithmetic
runs in the hand-written CUDA kernels of ``libqgb.so`` (C ABI in
``include/qgb.h``); there is no CPU path.
"""
from . import workloads
from .circuits import Circuit, brickwall_skeleton, two_local_circ
from .density_matrix import DensityMatrixSim
from .gates import (CNOT, CZ, H, ID, RX, RY, RZ, RXX, RYY, RZZ, SDG, SWAP, SX, U, X, Y, Z, CUGate, Gate, Reset,
                    SuperOp, embed_operator, iSWAP, kak_unitary)
from .hamiltonians import TFI
from .environments import RunContext, environment_state_prep, environment_update, sv_environment
from .montecarlo import MonteCarloSim, trotter_mc_sim
from .noise import AmplitudeDamping, PauliLindbladNoise, PauliNoise, QubitNoise, amplitude_damping, depolarizing
from .statevector import StatevectorSim

__version__ = "0.1.0"
