"""ctypes binding of the C ABI in include/rbmg.h (librbmg.so, built in-tree).

There is no fallback: if the CUDA library is missing or cannot be loaded the import
of any compute entry point raises.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "librbmg.so")

RBMG_OK, RBMG_EINVAL, RBMG_ENOMEM, RBMG_ECUDA, RBMG_ETIMEOUT, RBMG_ENAN, RBMG_EUNSUPPORTED = range(7)


class RbmgError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, code, msg):
        super().__init__(f"rbmg error {code}: {msg}")
        self.code = code


_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_u64p = C.POINTER(C.c_uint64)
_vp = C.c_void_p
_vpp = C.POINTER(C.c_void_p)
_fp = C.POINTER(C.c_float)

# name -> argtypes (all return int status unless listed in _RESTYPE)
SIGNATURES = {
    "rbmg_last_error": [],
    "rbmg_version": [],
    "rbmg_set_device": [C.c_int],
    "rbmg_profiler_start": [],
    "rbmg_profiler_stop": [],
    "rbmg_activation": [C.c_double, C.c_double, _dp],
    "rbmg_psi_create": [C.c_int, C.c_int, _dp, _dp, _dp, _dp, C.c_double, C.c_int, _vpp],
    "rbmg_psi_deep_create": [C.c_int, C.c_int, _ip, _ip, C.POINTER(C.POINTER(C.c_uint32)), C.POINTER(_dp),
                             C.POINTER(_dp), _dp, _dp, _dp, C.c_double, C.c_int, C.c_int, _vpp],
    "rbmg_psi_copy": [_vp, _vpp],
    "rbmg_psi_destroy": [_vp],
    "rbmg_psi_kind": [_vp, _ip],
    "rbmg_psi_free_quantum_axis": [_vp, _ip],
    "rbmg_psi_shape": [_vp, _ip, _ip, _ip],
    "rbmg_psi_get_params": [_vp, _dp],
    "rbmg_psi_set_params": [_vp, _dp],
    "rbmg_psi_get_prefactor": [_vp, _dp],
    "rbmg_psi_set_prefactor": [_vp, C.c_double],
    "rbmg_psi_set_translational_invariance": [_vp, C.c_int],
    "rbmg_psi_log_psi": [_vp, C.c_int, _u64p, _dp],
    "rbmg_psi_vector": [_vp, _dp],
    "rbmg_psi_norm": [_vp, _vp, _dp],
    "rbmg_psi_O_k_vector": [_vp, _u64p, _dp],
    "rbmg_operator_create": [C.c_int, C.c_int, _dp, _ip, _ip, _vpp],
    "rbmg_operator_destroy": [_vp],
    "rbmg_operator_shape": [_vp, _ip, _ip],
    "rbmg_operator_tables": [_vp, _dp, _ip, _ip],
    "rbmg_mc_create": [C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint64, _vpp],
    "rbmg_mc_copy": [_vp, _vpp],
    "rbmg_mc_set_total_z_symmetry": [_vp, C.c_int],
    "rbmg_mc_set_fast_sweep": [_vp, C.c_uint32],
    "rbmg_mc_acceptance": [_vp, _u64p, _u64p, _u64p],
    "rbmg_exact_create": [C.c_uint32, _vpp],
    "rbmg_samples_create": [C.c_uint32, C.c_uint32, _u64p, _vpp],
    "rbmg_exact_set_total_z_symmetry": [_vp, C.c_int],
    "rbmg_ensemble_num_steps": [_vp, _u64p],
    "rbmg_ensemble_destroy": [_vp],
    "rbmg_ensemble_samples": [_vp, _vp, _vp, _u64p, _dp, _dp],
    "rbmg_ev_value": [_vp, _vp, _vp, _dp],
    "rbmg_ev_values": [_vp, _vpp, C.c_int, _vp, _dp],
    "rbmg_ev_fluctuation_gradient": [_vp, _vp, _vp, _dp, _dp],
    "rbmg_ev_difference": [_vp, _vp, _vpp, C.c_int, _vp, _dp],
    "rbmg_ev_corrected": [_vp, _vp, _vp, _vp, _dp, _dp],
    "rbmg_ev_fluctuation": [_vp, _vp, _vp, _dp, _dp],
    "rbmg_ev_gradient": [_vp, _vp, _vp, _dp, _dp],
    "rbmg_local_energies": [_vp, _vp, C.c_int, _u64p, _dp],
    "rbmg_ev_eloc_gradient": [_vp, _vp, _vp, C.c_int, _dp, _dp],
    "rbmg_hsd_distance": [_vp, _vp, _vp, C.c_int, _vp, _dp],
    "rbmg_hsd_gradient": [_vp, _vp, _vp, C.c_int, _vp, C.c_float, _dp, _dp],
    "rbmg_chain_create": [_vp, C.c_uint32, C.c_uint64, _vpp],
    "rbmg_chain_destroy": [_vp],
    "rbmg_chain_sweep_async": [_vp, _vp, _vp, C.c_int, C.c_int, _vp, _vp],
    "rbmg_chain_state": [_vp, _u64p, _u64p, _u64p],
    "rbmg_stream": [_vpp],
    "rbmg_probe_fp32_tflops": [C.c_int, _dp],
    "rbmg_probe_fp32x2_tflops": [C.c_int, _dp],
    "rbmg_ev_value_exact_noalloc": [_vp, _vp, C.c_int, _dp],
    "rbmg_proposal_create": [C.c_int, C.c_uint64, C.c_float, _vpp],
    "rbmg_proposal_destroy": [_vp],
    "rbmg_proposal_num_params": [_vp, C.POINTER(C.c_int64)],
    "rbmg_proposal_get_params": [_vp, C.POINTER(C.c_float)],
    "rbmg_proposal_set_params": [_vp, C.POINTER(C.c_float)],
    "rbmg_proposal_eval": [_vp, C.c_int, _u64p, C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float)],
    "rbmg_proposal_adam": [_vp, C.POINTER(C.c_float)],
    "rbmg_proposal_set_objective": [_vp, C.c_int],
    "rbmg_proposal_status": [_vp],
    "rbmg_proposal_get_state": [_vp, C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float),
                                C.POINTER(C.c_int64)],
    "rbmg_proposal_set_state": [_vp, C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_int64],
    "rbmg_chain_get_checkpoint": [_vp, _u64p, _u64p, _u64p, _u64p],
    "rbmg_chain_set_checkpoint": [_vp, _u64p, _u64p, _u64p, _u64p],
    "rbmg_batch_create": [C.c_int, _vpp, _vpp, C.POINTER(C.c_uint32), _u64p, _vpp],
    "rbmg_batch_destroy": [_vp],
    "rbmg_batch_run": [_vp, C.c_int, C.c_int],
    "rbmg_batch_set_shape": [_vp, C.c_int, C.c_int],
    "rbmg_batch_get_shape": [_vp, _ip, _ip, _ip],
    "rbmg_batch_autotune": [_vp, C.c_int, C.c_int, _dp],
    "rbmg_batch_set_register_cap": [_vp, C.c_int],
    "rbmg_batch_set_wait": [_vp, C.c_double, C.c_uint32],
    "rbmg_batch_get_register_cap": [_vp, _ip],
    "rbmg_batch_result": [_vp, C.c_int, _dp, _dp, _dp],
    "rbmg_batch_spins": [_vp, C.c_int, _u64p],
    "rbmg_batch_info": [_vp, _ip, _u64p, _dp],
    "rbmg_chain_learned_async": [_vp, _vp, _vp, _vp, C.c_int, C.c_int, C.c_int, _vp, _vp],
    "rbmg_chain_learned_kernel_times": [_vp, _vp, _vp, C.c_int, _dp, _dp],
    "rbmg_proposal_lb_target": [_vp, _vp, C.c_int, _u64p, _fp, _fp],
    "rbmg_chain_learned_trace": [_vp, _vp, _vp, C.c_int, _u64p, _u64p, _fp, _fp, _fp, _fp, _ip, _ip, _fp, _u64p,
                                 _u64p, _u64p],
    "rbmg_chain_set_learned_streams": [_vp, C.c_int],
    "rbmg_optimizer_create": [C.c_int, C.c_int, _dp, C.c_int, C.c_int, _vpp],
    "rbmg_optimizer_destroy": [_vp],
    "rbmg_optimizer_reset": [_vp],
    "rbmg_optimizer_num_steps": [_vp, _u64p],
    "rbmg_optimizer_update": [_vp, _dp, _dp, C.c_double],
    "rbmg_optimizer_lookahead": [_vp, _dp, _dp],
    "rbmg_optimizer_step_energy": [_vp, _vp, _vp, _vp, C.c_double, _dp],
    "rbmg_s_matrix": [_vp, _vp, C.c_int, _dp],
    "rbmg_s_matrix_timing": [_dp, _ip],
    "rbmg_hsd_distance_2nd_order": [_vp, _vp, _vp, _vp, _vp, _dp],
    "rbmg_diag_density": [_vp, _vp, _vp, C.c_int, _dp],
    "rbmg_kl_gradient": [_vp, _vp, _vp, C.c_double, _dp, _dp],
    "rbmg_psi_angles": [_vp, C.c_int, _u64p, _dp],
}
_RESTYPE = {"rbmg_last_error": C.c_char_p, "rbmg_version": C.c_char_p}

_lib = None


def lib():
    """Loads librbmg.so (building it first when the sources are newer)."""
    global _lib
    if _lib is None:
        from . import build as _build
        if not os.path.exists(LIB_PATH):
            _build.build()
        L = C.CDLL(LIB_PATH)
        for name, args in SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = _RESTYPE.get(name, C.c_int)
        _lib = L
    return _lib


def check(code):
    if code != RBMG_OK:
        raise RbmgError(code, lib().rbmg_last_error().decode())
    return code


def call(name, *args):
    return check(getattr(lib(), name)(*args))
