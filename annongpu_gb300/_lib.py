"""ctypes binding of libannongpu.so (include/annongpu.h).

The library is the product: there is no CPU fallback. Importing this module
fails loudly when the shared library has not been built.
"""

from __future__ import annotations

import ctypes as ct
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libannongpu.so")

if not os.path.exists(LIB_PATH):
    raise ImportError(
        f"{LIB_PATH} is missing: build the CUDA library first "
        "(python -m annongpu_gb300.build, or __graft_entry__.build())")

lib = ct.CDLL(LIB_PATH)

P = ct.c_void_p
U = ct.c_uint
I = ct.c_int
D = ct.c_double
U64 = ct.c_uint64

ANN_OK = 0
ANN_ERR_INVALID = 1
ANN_ERR_CUDA = 2
ANN_ERR_NUMERIC = 3
ANN_ERR_UNSUPPORTED = 4

LAYOUT_RBM, LAYOUT_DEEP = 0, 1
ACT_POLY, ACT_LOGCOSH = 0, 1
PREC_FP32, PREC_FP64 = 0, 1
MOVE_FLIP, MOVE_EXCHANGE_BONDS, MOVE_EXCHANGE_PAIRS = 0, 1, 2
S_FP32, S_BF16, S_BF16_SPLIT = 0, 1, 2
BASIS_SPINS, BASIS_PAULIS = 0, 1
SOLVER_FP64, SOLVER_MIXED, SOLVER_FP32 = 0, 1, 2


class RbmDesc(ct.Structure):
    _fields_ = [("N", U), ("M", U), ("C", U), ("connections", P), ("params", P), ("final_weights", P),
                ("log_prefactor", D * 2), ("layout", I), ("a_in_log_psi", I), ("activation", I),
                ("precision", I)]


class CnnDesc(ct.Structure):
    _fields_ = [("extent", U * 3), ("num_layers", U), ("num_channels", P), ("connectivity", P),
                ("symmetry_classes", P), ("params", P), ("num_params", U), ("final_factor", D),
                ("log_prefactor", D * 2), ("activation", I), ("precision", I)]


class DeepDesc(ct.Structure):
    _fields_ = [("N", U), ("num_layers", U), ("sizes", P), ("connectivity", P), ("connections", P),
                ("params", P), ("num_params", U), ("final_weights", P), ("log_prefactor", D * 2),
                ("a_in_log_psi", I), ("activation", I), ("precision", I)]


class ClassicalDesc(ct.Structure):
    _fields_ = [("num_sites", U), ("n_features", U), ("feature_begin", P), ("num_words", U), ("a", P), ("b", P),
                ("coeff", P), ("params", P), ("log_prefactor", D * 2), ("order", U), ("ref", P), ("precision", I)]


class McDesc(ct.Structure):
    _fields_ = [("num_samples", U), ("num_sweeps", U), ("num_thermalization_sweeps", U),
                ("num_markov_chains", U), ("move", I), ("bonds", P), ("n_bonds", U), ("n_up", I),
                ("seed", U64), ("persistent", I)]


_SIGS = {
    "ann_last_error": ([], ct.c_char_p),
    "ann_version": ([], I),
    "ann_set_device": ([I], I),
    "ann_profiler_start": ([], I),
    "ann_profiler_stop": ([], I),
    "ann_kernel_launch_count": ([], ct.c_ulonglong),
    "ann_status": ([P], I),
    "ann_psi_create_rbm": ([P, P], I),
    "ann_psi_create_cnn": ([P, P], I),
    "ann_psi_create_deep": ([P, P], I),
    "ann_ens_set_basis": ([P, I], I),
    "ann_psi_create_classical": ([P, P], I),
    "ann_psi_ref_log_prefactor": ([P, P, P], I),
    "ann_kl_create": ([U, P], I),
    "ann_kl_destroy": ([P], I),
    "ann_kl_log_psi_scale": ([P, P, P], I),
    "ann_kl_value": ([P, P, P, P, D, P, P], I),
    "ann_kl_gradient": ([P, P, P, P, D, D, P, P, P, P], I),
    "ann_kl_stats": ([P, P, P], I),
    "ann_log_psi_paulis": ([P, P, U, P, P], I),
    "ann_psi_O_k_paulis": ([P, P, P], I),
    "ann_local_energies_paulis": ([P, P, P, U, P, P], I),
    "ann_psi_copy": ([P, P], I),
    "ann_psi_destroy": ([P], I),
    "ann_psi_num_params": ([P, P], I),
    "ann_psi_get_params": ([P, P], I),
    "ann_psi_set_params": ([P, P], I),
    "ann_psi_set_params_async": ([P, P, P], I),
    "ann_psi_get_log_prefactor": ([P, P], I),
    "ann_psi_set_log_prefactor": ([P, D, D], I),
    "ann_psi_params_device": ([P, P], I),
    "ann_psi_sync_device_params": ([P, P], I),
    "ann_op_create_pauli": ([U, U, P, P, P, P], I),
    "ann_op_destroy": ([P], I),
    "ann_op_num_strings": ([P, P], I),
    "ann_ens_create_exact": ([U, P], I),
    "ann_ens_create_mc": ([P, P], I),
    "ann_ens_copy": ([P, P], I),
    "ann_ens_destroy": ([P], I),
    "ann_ens_num_steps": ([P, P], I),
    "ann_ens_refresh_stats": ([P, P], I),
    "ann_ens_acceptance_rate": ([P, P], I),
    "ann_ens_get_chains": ([P, P, P], I),
    "ann_ens_set_chains": ([P, P, P], I),
    "ann_ens_set_tape": ([P, P, P, P, U], I),
    "ann_ens_get_samples": ([P, P, P, P], I),
    "ann_expectation": ([P, P, P, P, P], I),
    "ann_expectation_list": ([P, U, P, P, P, P], I),
    "ann_fluctuation": ([P, P, P, P, P], I),
    "ann_gradient": ([P, P, P, P, P, P], I),
    "ann_exp_sigma_z": ([P, P, P, P, P], I),
    "ann_log_psi_s": ([P, P, P], I),
    "ann_log_psi_batch": ([P, P, U, P, P], I),
    "ann_local_energies": ([P, P, P, U, P, P], I),
    "ann_psi_O_k": ([P, P, P], I),
    "ann_psi_O_k_vector": ([P, P, P, P], I),
    "ann_log_psi": ([P, P, P, P], I),
    "ann_psi_vector": ([P, P, P, P], I),
    "ann_log_psi_vector": ([P, P, P, P], I),
    "ann_psi_norm": ([P, P, P, P], I),
    "ann_apply_operator": ([P, P, P, P, P], I),
    "ann_activation_function": ([D, D, U, I, P], I),
    "ann_tdvp_create": ([U, P], I),
    "ann_tdvp_destroy": ([P], I),
    "ann_tdvp_set_s_mode": ([P, I], I),
    "ann_tdvp_eval": ([P, P, P, P, P], I),
    "ann_tdvp_eval_F": ([P, P, P, P, P], I),
    "ann_tdvp_get_S": ([P, P], I),
    "ann_tdvp_get_F": ([P, P], I),
    "ann_tdvp_get_O": ([P, P], I),
    "ann_tdvp_get_energy": ([P, P, P], I),
    "ann_tdvp_get_total_weight": ([P, P], I),
    "ann_tdvp_get_O_samples": ([P, P], I),
    "ann_force_vector_noalloc": ([P, ct.c_size_t, ct.c_size_t, U, P, D, P, P, P, P, P], I),
    "ann_tdvp_S_dot_vector": ([P, P, P, P], I),
    "ann_tdvp_set_solver": ([P, I, U, D], I),
    "ann_tdvp_solver_info": ([P, P], I),
    "ann_tdvp_solver_form": ([P, P], I),
    "ann_tdvp_set_chol_update": ([P, I], I),
    "ann_autotune": ([P, P, P, P, D, P, P, U, P], I),
    "ann_hsd_distance": ([P, P, P, I, P, P, P], I),
    "ann_hsd_gradient": ([P, P, P, I, P, D, P, P, P], I),
    "ann_tuning_set": ([ct.c_char_p, I], I),
    "ann_tuning_get": ([ct.c_char_p, P, P], I),
    "ann_tuning_dump": ([ct.c_char_p, ct.c_size_t, P], I),
    "ann_tuning_clear": ([], I),
    "ann_tdvp_solve": ([P, D, P, P, P], I),
    "ann_sr_update": ([P, P, D, P], I),
    "ann_sr_step": ([P, P, P, P, D, D, P], I),
    "ann_sr_graph_capture": ([P, P, P, P, D, D, P], I),
    "ann_sr_graph_launch": ([P, P], I),
    "ann_set_phase_timing": ([I], I),
    "ann_batch_create": ([U, P, P, P, P, P], I),
    "ann_batch_destroy": ([P], I),
    "ann_batch_sample": ([P, P], I),
    "ann_batch_energies": ([P, P], I),
    "ann_batch_sr_step": ([P, D, D, P], I),
    "ann_batch_graph_capture": ([P, D, D, P], I),
    "ann_batch_graph_launch": ([P, P], I),
    "ann_ens_set_proposal": ([P, P, U, D], I),
    "ann_ens_proposal_stats": ([P, P, P], I),
    "ann_ens_set_history": ([P, U], I),
    "ann_made_create": ([U, U, U64, P], I),
    "ann_made_destroy": ([P], I),
    "ann_made_get_params": ([P, P, P, P, P], I),
    "ann_made_set_params": ([P, P, P, P, P], I),
    "ann_made_log_prob": ([P, P, U, P], I),
    "ann_made_sample": ([P, U, U64, U64, P, P], I),
    "ann_made_gradient": ([P, P, U, P, P, P, P, P], I),
    "ann_made_train": ([P, P, U, U, U, D, P, P], I),
    "ann_made_train_on_samples": ([P, P, U, U, D, P, P], I),
    "ann_get_solve_times": ([P], I),
    "ann_set_factor_trace": ([I], I),
    "ann_get_factor_trace": ([P, U, P], I),
    "ann_get_phase_times": ([P], I),
}

MISSING = []
for _name, (_args, _res) in _SIGS.items():
    try:
        _f = getattr(lib, _name)
    except AttributeError:  # a stale library: calls to this entry point raise; rebuild to fix
        MISSING.append(_name)
        continue
    _f.argtypes = _args
    _f.restype = _res


class AnnError(RuntimeError):
    """A C-ABI call failed (the reference raises RuntimeError from CUDA_CHECK, include/types.h:139-147)."""

    def __init__(self, code, msg):
        super().__init__(f"annongpu error {code}: {msg}")
        self.code = code


def check(rc: int) -> None:
    if rc != ANN_OK:
        raise AnnError(rc, lib.ann_last_error().decode())


def call(name: str, *args) -> None:
    if name in MISSING:
        raise AnnError(ANN_ERR_UNSUPPORTED, f"{name} missing from {LIB_PATH}: rebuild the library")
    check(getattr(lib, name)(*args))


def ptr(a):
    return None if a is None else a.ctypes.data_as(ct.c_void_p)


def cbuf(n: int) -> np.ndarray:
    return np.zeros(n, np.complex128)


def c128(x) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(x, dtype=np.complex128))


def stream_ptr(stream) -> ct.c_void_p | None:
    """Accepts None, an int handle or a torch.cuda.Stream."""
    if stream is None:
        return None
    if hasattr(stream, "cuda_stream"):
        return ct.c_void_p(stream.cuda_stream)
    return ct.c_void_p(int(stream))


def launch_count() -> int:
    return int(lib.ann_kernel_launch_count())
