"""ctypes binding of ``libqgb.so`` (the C ABI declared in ``include/qgb.h``).

The library is built in-tree by ``qaravan_gb300.build.build()``. There is no
fallback: if the library is missing or a CUDA device is absent, calls raise.
"""
from __future__ import annotations

import ctypes as C
import os

import torch

from . import build as _build

QGB_C64, QGB_C128 = 0, 1
QGB_OK, QGB_EINVAL, QGB_ECUDA, QGB_ETIMEOUT, QGB_ESCRATCH = 0, -1, -2, -3, -4
QGB_MAX_K = 6
QGB_SWEEP_MAX_OPS = 64
QGB_SWEEP_MAX_HIGH = 10
QGB_SWEEP_MAX_TILE_BITS = 14

_ERRORS = {-1: "invalid argument", -2: "CUDA error", -3: "device wait timed out", -4: "scratch too small"}


class QgbError(RuntimeError):
    pass


class Sweep(C.Structure):
    """Mirror of ``qgb_sweep``."""
    _fields_ = [
        ("low_bits", C.c_int32),
        ("n_high", C.c_int32),
        ("high_bits", C.c_int32 * QGB_SWEEP_MAX_HIGH),
        ("n_ops", C.c_int32),
        ("op_k", C.c_int32 * QGB_SWEEP_MAX_OPS),
        ("op_pos", (C.c_int32 * QGB_MAX_K) * QGB_SWEEP_MAX_OPS),
        ("op_mat", C.c_int64 * QGB_SWEEP_MAX_OPS),
    ]


QGB_TCS_MAX_BLOCKS = 4


class TcSweep(C.Structure):
    """Mirror of ``qgb_tc_sweep``."""
    _fields_ = [
        ("low_bits", C.c_int32),
        ("high_bits", C.c_int32 * 9),
        ("n_blocks", C.c_int32),
        ("block_pos", (C.c_int32 * 5) * QGB_TCS_MAX_BLOCKS),
        ("block_mat", C.c_int64 * QGB_TCS_MAX_BLOCKS),
    ]


class AdjointSweep(C.Structure):
    """Mirror of ``qgb_adjoint_sweep``."""
    _fields_ = [
        ("low_bits", C.c_int32),
        ("n_high", C.c_int32),
        ("high_bits", C.c_int32 * QGB_SWEEP_MAX_HIGH),
        ("n_ops", C.c_int32),
        ("op_k", C.c_int32 * QGB_SWEEP_MAX_OPS),
        ("op_pos", (C.c_int32 * 2) * QGB_SWEEP_MAX_OPS),
        ("op_mat", C.c_int64 * QGB_SWEEP_MAX_OPS),
        ("op_out", C.c_int32 * QGB_SWEEP_MAX_OPS),
        ("op_gen_col", (C.c_int32 * 4) * QGB_SWEEP_MAX_OPS),
        ("op_gen_val", ((C.c_double * 2) * 4) * QGB_SWEEP_MAX_OPS),
    ]


_vp, _i, _i64, _u64, _sz, _dp, _cp, _ip = (C.c_void_p, C.c_int, C.c_int64, C.c_uint64, C.c_size_t,
                                           C.POINTER(C.c_double), C.c_char_p, C.POINTER(C.c_int))

# name -> (restype, argtypes)
SIGNATURES = {
    "qgb_abi_version": (C.c_int, []),
    "qgb_last_error": (C.c_char_p, []),
    "qgb_check_status": (C.c_int, [_vp]),
    "qgb_wait_probe": (C.c_int, [_i, C.c_ulonglong, _vp, _vp]),
    "qgb_fma_probe": (C.c_int, [_i, _i, _i, _vp, _vp]),
    "qgb_op_action": (C.c_int, [_vp, _i, _i, _ip, _i, _vp, _i64, _i64, _i64, _vp]),
    "qgb_op_action_unitary": (C.c_int, [_vp, _i, _i, _ip, _i, _vp, _i64, _i64, _i64, _vp]),
    "qgb_op_action_unitary_chain": (C.c_int, [_vp, _i, _i, _ip, _i, _vp, _i64, _i64, _i64, _vp, _i, _vp]),
    "qgb_op_action_scaled": (C.c_int, [_vp, _i, _i, _ip, _i, _vp, _vp, _vp]),
    "qgb_dm_trace_factor": (C.c_int, [_vp, _i, _i, _vp, _i, _vp]),
    "qgb_apply_sweep": (C.c_int, [_vp, _i, _i, C.POINTER(Sweep), _vp, _i64, _i64, _i64, _vp]),
    "qgb_set_sweep_impl": (C.c_int, [_i]),
    "qgb_set_c128_arith": (C.c_int, [_i]),
    "qgb_set_adjoint_runs": (C.c_int, [_i]),
    "qgb_apply_tc_sweep": (C.c_int, [_vp, _i, _i, C.POINTER(TcSweep), _vp, _vp, _i, _vp]),
    "qgb_dm_batch_circuit_bytes": (C.c_size_t, []),
    "qgb_dm_batch_pass_bytes": (C.c_size_t, []),
    "qgb_dm_batch_items": (C.c_int64, [_vp, _i, _i]),
    "qgb_dm_batch_table_bytes": (C.c_size_t, [_i, _i, _i64]),
    "qgb_dm_batch_build": (C.c_int, [_vp, _sz, _vp, _i, _vp, _i, _i]),
    "qgb_dm_batch_work_bytes": (C.c_size_t, [_i, _i64]),
    "qgb_dm_batch_run": (C.c_int, [_vp, _sz, _i, _i, _i64, _vp, _i, _i, _vp, _sz, _vp]),
    "qgb_tc_sweep_bytes": (C.c_size_t, []),
    "qgb_get_c128_arith": (C.c_int, []),
    "qgb_init_basis": (C.c_int, [_vp, _i, _i, _u64, _i64, _i64, _vp]),
    "qgb_scale": (C.c_int, [_vp, _i, _i, _vp, _i64, _i64, _vp]),
    "qgb_pauli_layer": (C.c_int, [_vp, _i, _i, _vp, _vp, _vp, _i64, _i64, _vp]),
    "qgb_adjoint_step_batched": (C.c_int, [_vp, _vp, _i, _i, _ip, _i, _vp, _i64, _i64, _i64, _vp, _vp, _sz, _vp]),
    "qgb_param_matrices": (C.c_int, [_vp, _vp, _i, _vp, _i, _i64, _vp, _i, _i64, _i64, _vp]),
    "qgb_param_grads": (C.c_int, [_vp, _vp, _i, _i64, _vp, C.c_double, _vp, _vp]),
    "qgb_adjoint_sweep_scratch_bytes": (C.c_size_t, [_i, _i, _i, _i64]),
    "qgb_partial_overlap_scratch_bytes": (C.c_size_t, [_i, _i, _i64]),
    "qgb_adjoint_sweep_step": (C.c_int, [_vp, _vp, _i, _i, C.POINTER(AdjointSweep), _vp, _i64, _i64, _i64, _vp, _vp,
                                         _sz, _vp]),
    "qgb_adjoint_step_rotation": (C.c_int, [_vp, _vp, _i, _i, _ip, _i, _vp, _i64, _dp, _i64, _i64, _vp, _vp, _sz, _vp]),
    "qgb_probs_scratch_bytes": (C.c_size_t, [_i, _i]),
    "qgb_outcome_probs": (C.c_int, [_vp, _i, _i, _ip, _i, _vp, _vp, _sz, _vp]),
    "qgb_sample_scratch_bytes": (C.c_size_t, [_i]),
    "qgb_sample_outcomes": (C.c_int, [_vp, _i, _i64, C.c_uint64, _vp, _vp, _sz, _vp]),
    "qgb_collapse": (C.c_int, [_vp, _i, _i, _ip, _i, C.c_uint64, _vp, _vp, _vp]),
    "qgb_fuse_block_bytes": (C.c_size_t, []),
    "qgb_fuse_entry_bytes": (C.c_size_t, []),
    "qgb_fuse_blocks": (C.c_int, [_vp, _i, _i64, _vp, _i, _vp, _i, _vp, _i64, _vp]),
    "qgb_set_dense_impl": (C.c_int, [_i]),
    "qgb_get_dense_impl": (C.c_int, []),
    "qgb_reduce_scratch_bytes": (C.c_size_t, [_i, _i, _i64]),
    "qgb_norm2": (C.c_int, [_vp, _i, _i, _i64, _i64, _vp, _vp, _sz, _vp]),
    "qgb_pauli_expectation": (C.c_int, [_vp, _i, _i, _cp, _dp, _i, _i64, _i64, _vp, _vp, _sz, _vp]),
    "qgb_pauli_expectation_noalloc": (C.c_int, [_vp, _i, _i, _cp, _dp, _i, _vp, _vp]),
    "qgb_inner_product": (C.c_int, [_vp, _vp, _i, _i, _i64, _i64, _vp, _vp, _sz, _vp]),
    "qgb_pauli_apply": (C.c_int, [_vp, _vp, _i, _i, _cp, _dp, _i, _i64, _i64, _vp]),
    "qgb_partial_overlap": (C.c_int, [_vp, _vp, _i, _i, _ip, _i, _i64, _i64, _vp, _vp, _sz, _vp]),
    "qgb_adjoint_step": (C.c_int, [_vp, _vp, _i, _i, _ip, _i, _vp, _vp, _vp, _sz, _vp]),
    "qgb_batch_circuit_bytes": (C.c_size_t, []),
    "qgb_batch_op_bytes": (C.c_size_t, []),
    "qgb_batch_small": (C.c_int, [_vp, _i, _vp, _i, _vp, _vp, _i, _i, _vp, _vp]),
    "qgb_traj_blocks": (C.c_int, [_i]),
    "qgb_traj_step": (C.c_int, [_vp, _i, _i, _i64, _i64, _ip, _i, _vp, _ip, _i, _vp, C.c_double, C.c_double,
                                _u64, C.c_uint32, _vp, _vp, _vp, _vp]),
    "qgb_philox_uniform": (None, [C.c_uint32, C.c_uint32, C.c_uint32, _u64, C.POINTER(C.c_double)]),
    "qgb_traj_run": (C.c_int, [_vp, _i, _i, _i64, _i64, _vp, _vp, _i, _vp, _vp, _i, _vp, _i64, C.c_double,
                               C.c_double, _u64, _vp, _vp, _i, _vp, _sz, _vp]),
    "qgb_traj_run_scratch_bytes": (C.c_size_t, [_i, _i, _i, _i64]),
    "qgb_traj_sweep_bytes": (C.c_size_t, []),
    "qgb_traj_op_bytes": (C.c_size_t, []),
    "qgb_dm_apply_superop": (C.c_int, [_vp, _i, _i, _ip, _i, _vp, _i64, _i64, _vp]),
    "qgb_dm_pauli_expectation": (C.c_int, [_vp, _i, _i, _cp, _dp, _i, _i64, _i64, _vp, _vp, _sz, _vp]),
    "qgb_dm_product_expectation": (C.c_int, [_vp, _i, _i, _dp, _i64, _i64, _vp, _vp, _sz, _vp]),
    "qgb_dm_trace": (C.c_int, [_vp, _i, _i, _i64, _i64, _vp, _vp, _sz, _vp]),
}

_lib = None


def lib():
    """Load (once) and return the ctypes library; raises if it is not built."""
    global _lib
    if _lib is None:
        path = _build.LIB
        if not os.path.exists(path):
            raise QgbError(f"CUDA extension not built ({path} missing): call qaravan_gb300.build.build()")
        L = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        if L.qgb_abi_version() != 1:
            raise QgbError("libqgb ABI version mismatch")
        _lib = L
    return _lib


def check(rc: int, what: str = ""):
    if rc != 0:
        msg = lib().qgb_last_error().decode(errors="replace")
        raise QgbError(f"{what}: {_ERRORS.get(rc, rc)}: {msg}")


def dtype_code(t: torch.dtype) -> int:
    if t == torch.complex64:
        return QGB_C64
    if t == torch.complex128:
        return QGB_C128
    raise QgbError(f"unsupported state dtype {t}")


def stream_ptr(device=None) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def require_cuda(t: torch.Tensor):
    if not t.is_cuda:
        raise QgbError("qaravan_gb300 runs on a CUDA device only (no CPU path)")
    if not t.is_contiguous():
        raise QgbError("state tensors must be contiguous")


def int_array(vals):
    arr = (C.c_int * max(1, len(vals)))(*[int(v) for v in vals])
    return arr


def double_array(vals):
    return (C.c_double * max(1, len(vals)))(*[float(v) for v in vals])
