"""ctypes binding of libqgpu.so (include/qgpu.h).

Loading fails loudly: there is no CPU fallback.  Device buffers are torch CUDA tensors
(torch is used for device memory and the stream only); every call passes raw pointers.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libqgpu.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "qgpu.h")

QG_ERR_TIMEOUT = 3
STATUS = {0: "QG_OK", 1: "QG_ERR_OOM", 2: "QG_ERR_TABLE_FULL", 3: "QG_ERR_TIMEOUT", 4: "QG_ERR_ARG",
          5: "QG_ERR_CUDA", 6: "QG_ERR_NOT_HERMITIAN"}

_lib = None


class QGError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (STATUS.get(status, status), msg))
        self.status = status


def load(path=LIB_PATH):
    """Load libqgpu.so and declare its signatures.  Raises if the library is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError("libqgpu.so not built (%s); run quanty_gb300.build.build()" % path)
    L = C.CDLL(path)
    P, I32, I64, D = C.c_void_p, C.c_int32, C.c_int64, C.c_double
    PP = C.POINTER(C.c_void_p)
    sig = {
        "qg_init": (C.c_int, [C.c_int, PP]),
        "qg_finalize": (C.c_int, [P]),
        "qg_set_stream": (C.c_int, [P, P]),
        "qg_get_stream": (P, [P]),
        "qg_last_error": (C.c_char_p, [P]),
        "qg_launch_count": (I64, [P]),
        "qg_synchronize": (C.c_int, [P]),
        "qg_operator_create": (C.c_int, [P, I32, I32, P, P, P, P, PP]),
        "qg_operator_destroy": (C.c_int, [P]),
        "qg_operator_info": (C.c_int, [P, P, P, P]),
        "qg_operator_create_sum": (C.c_int, [P, I32, P, P, P, PP]),
        "qg_operator_set_coefficients": (C.c_int, [P, P, P]),
        "qg_basis_create": (C.c_int, [P, I32, I64, P, PP, P]),
        "qg_basis_destroy": (C.c_int, [P]),
        "qg_basis_size": (I64, [P]),
        "qg_basis_get_dets": (C.c_int, [P, P]),
        "qg_basis_find": (C.c_int, [P, I64, P, P]),
        "qg_operator_psi_basis": (C.c_int, [P, P, P, P, PP]),
        "qg_basis_closure": (C.c_int, [P, P, P, P, I32, PP, P]),
        "qg_basis_union": (C.c_int, [P, P, P, PP]),
        "qg_basis_map": (C.c_int, [P, P, P, P, P, I32]),
        "qg_apply": (C.c_int, [P, P, P, P, P, P, I32]),
        "qg_apply_host": (C.c_int, [P, P, P, P, P, P, I32]),
        "qg_count_nnz": (C.c_int, [P, P, P, P]),
        "qg_count_nnz_offdiag": (C.c_int, [P, P, P, P]),
        "qg_count_nnz_rows": (C.c_int, [P, P, P, I64, I64, I32, P]),
        "qg_set_autotune": (C.c_int, [P, I32]),
        "qg_hermitian_eigh": (C.c_int, [P, I32, P, P, P, I32]),
        "qg_operator_dense": (C.c_int, [P, P, P, P]),
        "qg_poles_spectra": (C.c_int, [P, I32, I32, P, P, P, D, D, I32, D, P]),
        "qg_apply_chunk": (C.c_int, [P, P, P, I32, P]),
        "qg_apply_set_chunk": (C.c_int, [P, P, P, I32, I32]),
        "qg_set_connection_lists": (C.c_int, [P, I32]),
        "qg_set_small_basis_lanczos": (C.c_int, [P, I32]),
        "qg_set_split_chains": (C.c_int, [P, I32]),
        "qg_apply_list_info": (C.c_int, [P, P, P, P, P]),
        "qg_apply_fp64_ops": (C.c_int, [P, P, P, P]),
        "qg_expectation": (C.c_int, [P, P, P, P, I32, P]),
        "qg_dot": (C.c_int, [P, I64, I32, P, P, P]),
        "qg_dot_noalloc": (C.c_int, [I64, I32, P, P, P, P]),
        "qg_norm": (C.c_int, [P, I64, I32, P, P]),
        "qg_axpy": (C.c_int, [P, I64, I32, P, P, P]),
        "qg_lanczos_tridiag": (C.c_int, [P, P, P, P, I32, I32, D, D, P, P, P]),
        "qg_cf_spectra": (C.c_int, [P, I32, I32, P, P, P, D, D, I32, D, P]),
        "qg_block_lanczos": (C.c_int, [P, P, P, P, I32, I32, D, D, P, P, P, P]),
        "qg_krylov_combine": (C.c_int, [P, P, I64, I32, P, I32, P]),
        "qg_block_adjoint_product": (C.c_int, [P, P, I32, I32, P, I32, I32, I64, P]),
        "qg_block_product": (C.c_int, [P, P, I32, I32, P, I32, I64, D, D, P, I32]),
        "qg_block_cf_spectra": (C.c_int, [P, I32, I32, P, P, D, D, D, I32, D, P]),
        "qg_block_groundstate": (C.c_int, [P, P, P, I32, P, P, D, I32, I32, P]),
        "qg_lanczos_krylov": (C.c_int, [P, P, P, P, I32, D, P, P, P]),
        "qg_resonant_spectra": (C.c_int, [P, P, P, P, P, I32, P, P, P, P]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def header_symbols(path=HEADER):
    """Names of the functions include/qgpu.h declares."""
    import re
    txt = open(path).read()
    return sorted(set(re.findall(r"^\s*(?:qg_status|int64_t|void \*|const char \*)\s*(qg_\w+)\s*\(", txt, re.M)))


class Restrictions(C.Structure):
    _fields_ = [("n", C.c_int32), ("masks", C.c_void_p), ("min", C.c_void_p), ("max", C.c_void_p)]


class RixsSettings(C.Structure):
    _fields_ = [("ntri1", C.c_int32), ("ntri2", C.c_int32), ("epsilon", C.c_double),
                ("emin1", C.c_double), ("emax1", C.c_double), ("ne1", C.c_int32), ("gamma1", C.c_double),
                ("emin2", C.c_double), ("emax2", C.c_double), ("ne2", C.c_int32), ("gamma2", C.c_double),
                ("energy1", C.c_double), ("energy2", C.c_double), ("res1", C.c_void_p), ("res2", C.c_void_p)]
