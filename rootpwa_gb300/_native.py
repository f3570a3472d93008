"""ctypes binding of libpwa_gb300.so (the C ABI in include/pwa_gb300.h).

The library is the product: there is no Python or CPU implementation of any
evaluation behind these wrappers.  If the shared library is missing or fails
to load, every call raises.
"""
import ctypes as C
import os
import re

_HERE = os.path.dirname(os.path.abspath(__file__))
# PWA_GB300_DEBUG=1 selects the build with shared-memory bounds checks
# (rootpwa_gb300.build.build_debug())
LIB_PATH = os.path.join(_HERE, "libpwa_gb300_debug.so" if os.environ.get("PWA_GB300_DEBUG") == "1"
                        else "libpwa_gb300.so")
HEADER = os.path.join(os.path.dirname(_HERE), "include", "pwa_gb300.h")

SUCCESS = 0
ERROR_INVALID_ARGUMENT, ERROR_DEVICE_TIMEOUT = 1, 5
STATUS_NAMES = {
    0: "PWA_SUCCESS", 1: "PWA_ERROR_INVALID_ARGUMENT", 2: "PWA_ERROR_INVALID_STATE", 3: "PWA_ERROR_CUDA",
    4: "PWA_ERROR_OUT_OF_MEMORY", 5: "PWA_ERROR_DEVICE_TIMEOUT", 6: "PWA_ERROR_IO", 7: "PWA_ERROR_UNSUPPORTED",
    8: "PWA_ERROR_NUMERICAL",
}
COMPLEX64, COMPLEX128 = 0, 1
MEMORY_HOST, MEMORY_DEVICE = 0, 1
PRIOR_FLAT, PRIOR_HALF_CAUCHY = 0, 1
REDUCE_FP64, REDUCE_KAHAN_FP32, REDUCE_FP32 = 0, 1, 2
PRECISION = {"fp64": 0, "fp32": 1, "tf32": 2, "tf32x3": 3, "bf16x3": 4}
CALL_FDF, CALL_GRADIENT, CALL_DOEVAL, CALL_DODERIVATIVE, CALL_HESSIAN = range(5)


class PwaError(RuntimeError):
    """A C-ABI call returned a status other than PWA_SUCCESS."""

    def __init__(self, status, message):
        super().__init__("%s: %s" % (STATUS_NAMES.get(status, str(status)), message))
        self.status = status


_lib = None

vp = C.c_void_p
pd = C.POINTER(C.c_double)
u32, u64, i32, i64 = C.c_uint32, C.c_uint64, C.c_int32, C.c_int64
cc = C.c_char_p
i = C.c_int
pvp = C.POINTER(C.c_void_p)

class IsobarWave(C.Structure):
    """struct pwa_isobar_wave of include/pwa_gb300.h."""
    _fields_ = [(n, C.c_int32) for n in ("J", "P", "M", "refl", "L", "S", "isobarJ", "isobarL", "isobarS",
                                          "massDependence")] + \
        [("isobarMass", C.c_double), ("isobarWidth", C.c_double)] + \
        [(n, C.c_int32) for n in ("isobarDaughter1", "isobarDaughter2", "bachelor", "bachelorFirst", "isospin",
                                  "isobarIsospin")] + \
        [("binLower", C.c_double), ("binUpper", C.c_double), ("massDepParams", C.c_double * 10)]


SIGNATURES = {
    "pwa_abi_version": (i, []),
    "pwa_last_error": (cc, []),
    "pwa_kernel_launch_count": (u64, []),
    "pwa_integral_create": (i, [pvp]),
    "pwa_integral_destroy": (i, [vp]),
    "pwa_integral_copy": (i, [vp, vp]),
    "pwa_integral_set_wave_names": (i, [vp, u32, C.POINTER(cc)]),
    "pwa_integral_integrate": (i, [vp, u32, C.POINTER(cc), vp, u64, u32, i, i, pd, u64, vp, i64, i]),
    "pwa_integral_add_event": (i, [vp, pd]),
    "pwa_integral_element": (i, [vp, u32, u32, pd, pd]),
    "pwa_integral_matrix": (i, [vp, pd]),
    "pwa_integral_set_matrix": (i, [vp, pd]),
    "pwa_integral_nmb_waves": (i, [vp, C.POINTER(u32)]),
    "pwa_integral_nmb_events": (i, [vp, C.POINTER(u64)]),
    "pwa_integral_set_nmb_events": (i, [vp, u64]),
    "pwa_integral_wave_name": (i, [vp, u32, cc, u32]),
    "pwa_integral_wave_index": (i, [vp, cc, C.POINTER(u32)]),
    "pwa_integral_add": (i, [vp, vp]),
    "pwa_integral_subtract": (i, [vp, vp]),
    "pwa_integral_scale": (i, [vp, C.c_double]),
    "pwa_integral_divide": (i, [vp, C.c_double]),
    "pwa_integral_renormalize": (i, [vp, u64]),
    "pwa_integral_read_ascii": (i, [vp, cc]),
    "pwa_integral_write_ascii": (i, [vp, cc]),
    "pwa_gram_device_noalloc": (i, [vp, u64, u64, u32, vp, i, vp, vp]),
    "pwa_gram_device_batch": (i, [C.POINTER(vp), C.POINTER(u64), u32, u32, i, vp, vp, vp]),
    "pwa_multibin_create": (i, [pvp]),
    "pwa_multibin_destroy": (i, [vp]),
    "pwa_multibin_add_bin": (i, [vp, vp, u32]),
    "pwa_multibin_set_options": (i, [vp, u32, u32, C.c_double, C.c_double, u32]),
    "pwa_multibin_set_chunks": (i, [vp, C.POINTER(u32)]),
    "pwa_multibin_set_floor_window": (i, [vp, u32]),
    "pwa_multibin_trace": (i, [vp, u32, pd, pd, C.POINTER(u32)]),
    "pwa_multibin_chunks": (i, [vp, C.POINTER(u32)]),
    "pwa_multibin_autotune": (i, [vp, pd]),
    "pwa_multibin_nmb_problems": (i, [vp, C.POINTER(u32)]),
    "pwa_multibin_nmb_pars": (i, [vp, C.POINTER(u32)]),
    "pwa_multibin_fdf": (i, [vp, pd, pd, pd]),
    "pwa_multibin_sweep_ms": (i, [vp, pd, u32, pd]),
    "pwa_mlp_create": (i, [pvp, u32, u32, u32, u32, u64]),
    "pwa_mlp_destroy": (i, [vp]),
    "pwa_mlp_nmb_params": (i, [vp, C.POINTER(u64)]),
    "pwa_mlp_get_params": (i, [vp, C.POINTER(C.c_float)]),
    "pwa_mlp_set_params": (i, [vp, C.POINTER(C.c_float)]),
    "pwa_mlp_forward": (i, [vp, C.POINTER(C.c_float), u32, C.POINTER(C.c_float)]),
    "pwa_mlp_gradient": (i, [vp, C.POINTER(C.c_float), C.POINTER(C.c_float), u32, pd, C.POINTER(C.c_float)]),
    "pwa_mlp_train": (i, [vp, C.POINTER(C.c_float), C.POINTER(C.c_float), u64, u32, u32, C.c_float, u64, pd]),
    "pwa_multibin_fit": (i, [vp, pd, i, u32, u32, pd, pd, pd, C.POINTER(i32), C.POINTER(u32), C.POINTER(u32)]),
    "pwa_multibin_resume": (i, [vp, i, u32, u32, pd, pd, pd, C.POINTER(i32), C.POINTER(u32), C.POINTER(u32)]),
    "pwa_multibin_save_state": (i, [vp, C.c_char_p]),
    "pwa_multibin_load_state": (i, [vp, C.c_char_p]),
    "pwa_multibin_set_checkpoint": (i, [vp, C.c_char_p, u32]),
    "pwa_multibin_sweeps_done": (i, [vp, C.POINTER(u32)]),
    "pwa_likelihood_create": (i, [pvp]),
    "pwa_likelihood_destroy": (i, [vp]),
    "pwa_likelihood_use_normalized_amps": (i, [vp, i]),
    "pwa_likelihood_set_prior_type": (i, [vp, i]),
    "pwa_likelihood_set_cauchy_width": (i, [vp, C.c_double]),
    "pwa_likelihood_set_shard": (i, [vp, u64, i]),
    "pwa_likelihood_set_otf_binning": (i, [vp, u32, pd, pd, C.POINTER(vp), u64, i]),
    "pwa_likelihood_otf_selected": (i, [vp, C.POINTER(u64)]),
    "pwa_debug_fail_alloc_after": (i, [i64]),
    "pwa_debug_stalled_wait": (i, [u32]),
    "pwa_autotune_cache_save": (i, [C.c_char_p]),
    "pwa_autotune_cache_load": (i, [C.c_char_p]),
    "pwa_autotune_cache_clear": (i, []),
    "pwa_autotune_cache_size": (i, [C.POINTER(u32)]),
    "pwa_likelihood_load_amp_files": (i, [vp, u32, C.POINTER(C.c_char_p), u32, C.POINTER(C.c_char_p), pd, pd]),
    "pwa_ampfile_write": (i, [C.c_char_p, u32, C.POINTER(C.c_char_p), u64, vp, u32, C.POINTER(C.c_char_p), pd]),
    "pwa_ampfile_info": (i, [C.c_char_p, C.POINTER(u32), C.POINTER(u64), C.POINTER(u32)]),
    "pwa_ampfile_name": (i, [C.c_char_p, i, u32, C.c_char_p, u32]),
    "pwa_likelihood_set_stream": (i, [vp, vp]),
    "pwa_likelihood_set_reduction": (i, [vp, i]),
    "pwa_likelihood_set_autotune": (i, [vp, i]),
    "pwa_likelihood_plan": (i, [vp, C.POINTER(i), C.POINTER(i), C.POINTER(i)]),
    "pwa_likelihood_set_plan": (i, [vp, i]),
    "pwa_likelihood_set_plan_variant": (i, [vp, i, i]),
    "pwa_likelihood_set_store_block": (i, [vp, u32]),
    "pwa_likelihood_plan_variant": (i, [vp, C.POINTER(C.c_int)]),
    "pwa_likelihood_init": (i, [vp, u32, C.POINTER(cc), C.POINTER(i32), pd, u32, C.c_double]),
    "pwa_likelihood_add_norm_integral": (i, [vp, vp]),
    "pwa_likelihood_add_acc_integral": (i, [vp, vp, u64]),
    "pwa_likelihood_add_amplitude": (i, [vp, cc, vp, u64, i, i]),
    "pwa_likelihood_finish_init": (i, [vp]),
    "pwa_likelihood_nmb_pars": (i, [vp, C.POINTER(u32)]),
    "pwa_likelihood_nmb_pars_fixed": (i, [vp, C.POINTER(u32)]),
    "pwa_likelihood_nmb_events": (i, [vp, C.POINTER(u64)]),
    "pwa_likelihood_rank": (i, [vp, C.POINTER(u32)]),
    "pwa_likelihood_nmb_waves": (i, [vp, i, C.POINTER(u32)]),
    "pwa_likelihood_parameter": (i, [vp, u32, cc, u32, C.POINTER(i), C.POINTER(i), C.POINTER(i32), pd]),
    "pwa_likelihood_tot_acc": (i, [vp, pd]),
    "pwa_likelihood_fdf": (i, [vp, pd, pd, pd]),
    "pwa_likelihood_doeval": (i, [vp, pd, pd]),
    "pwa_likelihood_gradient": (i, [vp, pd, pd]),
    "pwa_likelihood_doderivative": (i, [vp, pd, u32, pd]),
    "pwa_likelihood_fdf_batch": (i, [vp, u32, pd, pd, pd]),
    "pwa_likelihood_fdf_device": (i, [vp, vp, vp, i, vp]),
    "pwa_likelihood_hessian": (i, [vp, pd, pd]),
    "pwa_likelihood_covariance_matrix": (i, [vp, pd, pd]),
    "pwa_likelihood_hessian_eigenvectors": (i, [vp, pd, pd, pd, C.POINTER(u32)]),
    "pwa_likelihood_options": (i, [vp, C.POINTER(i), C.POINTER(i), pd]),
    "pwa_likelihood_deriv_cache": (i, [vp, pd]),
    "pwa_likelihood_clear": (i, [vp]),
    "pwa_integral_contains_wave": (i, [vp, cc, C.POINTER(i)]),
    "pwa_integral_compare": (i, [vp, vp, C.POINTER(i), C.POINTER(i)]),
    "pwa_integral_clear": (i, [vp]),
    "pwa_isobar_create": (i, [pvp]),
    "pwa_isobar_destroy": (i, [vp]),
    "pwa_isobar_set_final_state": (i, [vp, u32, pd, C.POINTER(i32), C.c_double]),
    "pwa_isobar_set_options": (i, [vp, i, i, i, i]),
    "pwa_isobar_set_stream": (i, [vp, vp]),
    "pwa_isobar_set_formalism": (i, [vp, i]),
    "pwa_isobar_set_chunk_events": (i, [vp, u64]),
    "pwa_isobar_write_amp_file": (i, [vp, cc, C.POINTER(cc), vp, vp, u64, u32, C.POINTER(cc), vp]),
    "pwa_isobar_add_wave": (i, [vp, C.POINTER(IsobarWave)]),
    "pwa_isobar_nmb_waves": (i, [vp, C.POINTER(u32)]),
    "pwa_isobar_nmb_sym_terms": (i, [vp, u32, C.POINTER(u32)]),
    "pwa_isobar_set_isospins": (i, [vp, C.POINTER(i32), C.POINTER(i32), C.POINTER(i32)]),
    "pwa_isobar_enable_isospin_symmetrization": (i, [vp, i]),
    "pwa_isobar_amplitudes": (i, [vp, vp, vp, u64, vp, i, i]),
    "pwa_clebsch_gordan": (i, [i32, i32, i32, i32, i32, i32, pd]),
    "pwa_wigner_d": (i, [i32, i32, i32, C.c_double, pd]),
    "pwa_barrier_factor": (i, [i32, C.c_double, pd]),
    "pwa_likelihood_correct_param_signs": (i, [vp, pd, pd]),
    "pwa_likelihood_integral_matrices": (i, [vp, pd, pd, pd, i]),
    "pwa_likelihood_build_prod_amp_arrays": (i, [vp, pd, pd, C.POINTER(i32), C.POINTER(u32), i]),
    "pwa_likelihood_func_call_info": (i, [vp, i, C.POINTER(u64), pd, pd, pd]),
    "pwa_likelihood_reset_func_call_info": (i, [vp]),
    "pwa_likelihood_set_timing": (i, [vp, i]),
    "pwa_likelihood_kernel_times": (i, [vp, pd, pd, C.POINTER(u64)]),
}


def header_symbols():
    """Names of all functions declared in include/pwa_gb300.h."""
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pwa_[a-z0-9_]+)\s*\(", text)))


def lib():
    """Loads libpwa_gb300.so (raises if it is missing)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libpwa_gb300.so is not built (run __graft_entry__.build() or "
                               "python rootpwa_gb300/build.py); there is no fallback implementation")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(status):
    if status != SUCCESS:
        raise PwaError(status, lib().pwa_last_error().decode(errors="replace"))
    return status


def call(name, *args):
    return check(getattr(lib(), name)(*args))
