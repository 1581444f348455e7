"""ctypes binding of libmpsgb.so (C ABI declared in include/mpsgb.h).

The shared library is built in-tree by `mpsgb.build.build()`; importing this module
fails loudly when it is missing -- there is no CPU fallback for any operation.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libmpsgb.so")

GB_OK = 0
GB_ERR_ARG = 1
GB_ERR_OOM = 2
GB_ERR_CUDA = 3
GB_ERR_NOCONV = 4
GB_ERR_TIMEOUT = 5
GB_ERR_NAN = 6
GB_ERR_UNSUPPORTED = 7

GB_F64 = 1
GB_C128 = 2

GB_KIND_GENERIC = 0
GB_KIND_MPS = 1
GB_KIND_BOND = 2
GB_KIND_AC2 = 3
GB_KIND_GL = 4
GB_KIND_GR = 5
GB_KIND_MPO = 6

GB_HEFF_C = 0
GB_HEFF_AC = 1
GB_HEFF_AC2 = 2
GB_HEFF_AC_MPO = 3
GB_HEFF_AC2_MPO = 4

GB_PREC_FP64 = 0
GB_PREC_BF16X3 = 1
GB_PREC_TF32X3 = 2
PRECISIONS = {"fp64": GB_PREC_FP64, "bf16x3": GB_PREC_BF16X3, "tf32x3": GB_PREC_TF32X3}
GB_SCHED_PERSISTENT = 0
GB_SCHED_PERSISTENT_DENSE = 1
GB_SCHED_TILE = 2
GB_SCHED_GROUPED = 3


class KrylovInfo(ctypes.Structure):
    _fields_ = [("converged", ctypes.c_int), ("numops", ctypes.c_int),
                ("numiter", ctypes.c_int), ("normres", ctypes.c_double)]


class GBError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"libmpsgb error {code}: {msg}")
        self.code = code


_lib = None

P = ctypes.c_void_p
I64 = ctypes.c_int64
PI64 = ctypes.POINTER(ctypes.c_int64)
PI32 = ctypes.POINTER(ctypes.c_int32)
D = ctypes.c_double
PD = ctypes.POINTER(ctypes.c_double)
INT = ctypes.c_int
SZ = ctypes.c_size_t

_SIGS = {
    "gb_version": ([], INT),
    "gb_last_error": ([], ctypes.c_char_p),
    "gb_ctx_create": ([INT, ctypes.c_uint32, ctypes.POINTER(P)], INT),
    "gb_ctx_destroy": ([P], INT),
    "gb_ctx_synchronize": ([P], INT),
    "gb_ctx_kernel_launches": ([P, PI64], INT),
    "gb_ctx_device_status": ([P, ctypes.POINTER(ctypes.c_int32)], INT),
    "gb_ctx_set_wait_bound": ([P, D], INT),
    "gb_ctx_set_precision": ([P, INT], INT),
    "gb_ctx_profile_begin": ([P], INT),
    "gb_ctx_set_svd_method": ([P, INT], INT),
    "gb_ctx_set_gemm_schedule": ([P, INT, INT], INT),
    "gb_ctx_set_counting": ([P, INT], INT),
    "gb_ctx_read_work": ([P, PD, PD, INT], INT),
    "gb_ctx_profile_end": ([P, PD, PI64, PD, PD], INT),
    "gb_ctx_profile_kernel": ([P, INT, PD, PI64, PD], INT),
    "gb_ctx_trace_begin": ([P], INT),
    "gb_ctx_trace_end": ([P, PI64, PD], INT),
    "gb_ctx_trace_site": ([P, ctypes.c_int64, ctypes.c_char_p, SZ, PD, PI64], INT),
    "gb_tensor_create": ([P, INT, INT, INT, PI64, ctypes.POINTER(P)], INT),
    "gb_tensor_free": ([P], INT),
    "gb_tensor_shape": ([P, ctypes.POINTER(INT), ctypes.POINTER(INT), ctypes.POINTER(INT), PI64], INT),
    "gb_tensor_upload": ([P, P, SZ], INT),
    "gb_tensor_download": ([P, P, SZ], INT),
    "gb_tensor_copy": ([P, P], INT),
    "gb_tensor_scale": ([P, D, D], INT),
    "gb_tensor_axpy": ([P, D, D, P], INT),
    "gb_tensor_dot": ([P, P, PD, PD], INT),
    "gb_tensor_norm": ([P, PD], INT),
    "gb_heff_build": ([P, INT, P, P, P, P, INT, ctypes.POINTER(P)], INT),
    "gb_heff_free": ([P], INT),
    "gb_heff_terms": ([P, ctypes.c_char_p, SZ], INT),
    "gb_heff_flops": ([P, PD], INT),
    "gb_heff_set_precision": ([P, INT], INT),
    "gb_heff_set_sectors": ([P, PI32, PI32, PI32, PI32], INT),
    "gb_heff_apply": ([P, P, P], INT),
    "gb_heff_eigsolve": ([P, P, INT, INT, D, INT, PD, ctypes.POINTER(KrylovInfo)], INT),
    "gb_heff_exponentiate": ([P, P, D, D, INT, INT, D, ctypes.POINTER(KrylovInfo)], INT),
    "gb_mps_transfer_bond": ([P, INT, P, P, P, P], INT),
    "gb_env_linsolve": ([P, INT, P, P, INT, P, P, P, P, INT, INT, D, ctypes.POINTER(KrylovInfo)],
                        INT),
    "gb_env_transfer_left": ([P, P, P, P, P, INT, P], INT),
    "gb_env_transfer_right": ([P, P, P, P, P, INT, P], INT),
    "gb_env_regularize": ([P, P, I64, P, P], INT),
    "gb_env_channel_copy": ([P, P, I64, P, I64, I64], INT),
    "gb_tensor_adjoint": ([P, P, P], INT),
    "gb_mps_ac2": ([P, P, P, P], INT),
    "gb_mps_mul_front": ([P, P, P, P], INT),
    "gb_mps_mul_tail": ([P, P, P, P], INT),
    "gb_project_complement": ([P, P, P], INT),
    "gb_project_complement_right": ([P, P, P], INT),
    "gb_svd_batch": ([P, I64, ctypes.POINTER(P), ctypes.POINTER(P), ctypes.POINTER(P),
                      ctypes.POINTER(ctypes.c_double)], INT),
    "gb_mps_permute": ([P, P, INT, PI64, P], INT),
    "gb_basis_set": ([P, P, I64, P], INT),
    "gb_basis_orthogonalize": ([P, P, I64, P, ctypes.POINTER(ctypes.c_double)], INT),
    "gb_basis_combine": ([P, P, I64, ctypes.POINTER(ctypes.c_double), P], INT),
    "gb_heff_describe": ([P, ctypes.c_char_p, ctypes.c_size_t], INT),
    "gb_ctx_set_gauge": ([P, INT, INT], INT),
    "gb_ctx_set_option": ([P, INT, ctypes.c_int64], INT),
    "gb_tensor_pack": ([P, P, ctypes.POINTER(P)], INT),
    "gb_packed_unpack": ([P, P, P], INT),
    "gb_packed_info": ([P, PI64, PI64, ctypes.POINTER(ctypes.c_size_t)], INT),
    "gb_packed_free": ([P], INT),
    "gb_mps_perturb": ([P, INT, P, P, P, INT, P], INT),
    "gb_mpo_project": ([P, P, P, P, P, INT, P], INT),
    "gb_mps_cat": ([P, P, P, INT, P], INT),
    "gb_tensor_reshape": ([P, INT, INT, PI64], INT),
    "gb_svd_trunc": ([P, P, I64, D, INT, ctypes.POINTER(P), ctypes.POINTER(P), ctypes.POINTER(P), PD], INT),
    "gb_u1_left_orth": ([P, P, PI32, PI32, PI32, ctypes.POINTER(P), ctypes.POINTER(P), PI32, PI64], INT),
    "gb_u1_right_orth": ([P, P, PI32, PI32, PI32, ctypes.POINTER(P), ctypes.POINTER(P), PI32, PI64], INT),
    "gb_u1_svd_trunc": ([P, P, PI32, PI32, PI32, PI32, I64, D, INT, ctypes.POINTER(P), ctypes.POINTER(P),
                         ctypes.POINTER(P), PI32, PI64, PD], INT),
    "gb_left_orth": ([P, P, ctypes.POINTER(P), ctypes.POINTER(P)], INT),
    "gb_right_orth": ([P, P, ctypes.POINTER(P), ctypes.POINTER(P)], INT),
    "gb_c_apply_noalloc": ([P, P, P, P, I64, I64, I64, INT, P], INT),
}


def exported_names():
    return list(_SIGS)


def lib():
    """Load libmpsgb.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"libmpsgb.so not found at {LIB_PATH}: build it with "
                "`python -c 'import __graft_entry__ as g; g.build()'` (no CPU fallback exists)")
        L = ctypes.CDLL(LIB_PATH)
        for name, (args, res) in _SIGS.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _lib = L
    return _lib


def check(code):
    if code != GB_OK:
        msg = lib().gb_last_error()
        raise GBError(code, msg.decode() if msg else "")
    return code
