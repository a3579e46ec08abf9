"""ctypes binding of the C ABI in ``include/tbsla_gb300.h``.

The shared library is built in-tree by ``tbsla_gb300.build`` (nvcc for
sm_103a); importing this module without it raises, there is no fallback.
"""
from __future__ import annotations

import ctypes as C
import os

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libtbsla_gb300.so")

OK = 0
ERR_INVALID_ARG = -1
ERR_BAD_MATRIX = -2
ERR_ALLOC = -3
ERR_CUDA = -4
ERR_IO = -5
ERR_NOT_CONVERGED = -6
ERR_TIMEOUT = -7
ERR_UNSUPPORTED = -8
ERR_NO_DEVICE = -9

COO, SCOO, CSR, ELL, DENSE = 0, 1, 2, 3, 4
F64, F32, BF16 = 0, 1, 2
FORMAT_NAMES = {COO: "COO", SCOO: "SCOO", CSR: "CSR", ELL: "ELL", DENSE: "DENSE"}


class Info(C.Structure):
    _fields_ = [("n_row", C.c_int), ("n_col", C.c_int), ("ln_row", C.c_int), ("ln_col", C.c_int),
                ("f_row", C.c_int), ("f_col", C.c_int), ("nnz", C.c_long), ("pr", C.c_int),
                ("pc", C.c_int), ("NR", C.c_int), ("NC", C.c_int), ("max_col", C.c_int)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class Tuning(C.Structure):
    _fields_ = [("algorithm", C.c_int), ("items", C.c_int), ("short_thr", C.c_int), ("long_thr", C.c_int),
                ("sigma", C.c_int), ("col_block", C.c_int), ("tile", C.c_int), ("ms", C.c_double)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class TbslaError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        msg = _lib.tbsla_status_string(status).decode() if _lib else str(status)
        super().__init__(f"{what}: {msg} ({status})" if what else f"{msg} ({status})")


def _load() -> C.CDLL:
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"tbsla_gb300 native library missing ({LIB_PATH}); "
                          "build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    return C.CDLL(LIB_PATH)


_lib: C.CDLL | None = None
_lib = _load()

P = C.c_void_p
DP = C.POINTER(C.c_double)
IP = C.POINTER(C.c_int)
I = C.c_int
D = C.c_double
L = C.c_long
U = C.c_uint
ULL = C.c_ulonglong

_SIGS = {
    "tbsla_status_string": (C.c_char_p, [I]),
    "tbsla_version": (C.c_char_p, []),
    "tbsla_device_init": (I, [I]),
    "tbsla_host_alloc": (I, [C.POINTER(P), C.c_size_t]),
    "tbsla_host_free": (I, [P]),
    "tbsla_matrix_create": (I, [C.POINTER(P), I]),
    "tbsla_matrix_destroy": (I, [P]),
    "tbsla_matrix_format": (I, [P, IP]),
    "tbsla_matrix_info": (I, [P, C.POINTER(Info)]),
    "tbsla_matrix_set_coo": (I, [P, C.POINTER(Info), P, P, P]),
    "tbsla_matrix_set_csr": (I, [P, C.POINTER(Info), P, P, P]),
    "tbsla_matrix_push_back": (I, [P, I, I, D]),
    "tbsla_matrix_set_ell": (I, [P, C.POINTER(Info), P, P]),
    "tbsla_matrix_set_dense": (I, [P, C.POINTER(Info), P]),
    "tbsla_matrix_arrays": (I, [P, C.POINTER(P), C.POINTER(P), C.POINTER(P)]),
    "tbsla_matrix_fill_cdiag": (I, [P, I, I, I, I, I, I, I]),
    "tbsla_matrix_fill_cqmat": (I, [P, I, I, I, D, U, I, I, I, I]),
    "tbsla_matrix_fill_random": (I, [P, I, I, D, U, I, I, I, I]),
    "tbsla_matrix_fill_uniform_rows": (I, [P, I, I, ULL]),
    "tbsla_matrix_fill_powerlaw": (I, [P, I, D, D, I, D, I, ULL]),
    "tbsla_matrix_fill_dense_uniform": (I, [P, I, I, ULL]),
    "tbsla_matrix_fill_pa_graph": (I, [P, I, D, D, I, D, ULL]),
    "tbsla_matrix_fill_diffusion7": (I, [P, I, D, D, ULL]),
    "tbsla_fill_uniform": (I, [P, L, D, D, ULL]),
    "tbsla_matrix_convert": (I, [C.POINTER(P), P, I]),
    "tbsla_matrix_convert_device": (I, [C.POINTER(P), P, I]),
    "tbsla_matrix_write": (I, [P, C.c_char_p, I]),
    "tbsla_matrix_read": (I, [P, C.c_char_p, L]),
    "tbsla_matrix_set_precision": (I, [P, I]),
    "tbsla_matrix_upload": (I, [P]),
    "tbsla_matrix_device_bytes": (I, [P, C.POINTER(C.c_size_t)]),
    "tbsla_matrix_kernel_launches": (I, [P, IP]),
    "tbsla_matrix_set_csr_tile": (I, [P, I]),
    "tbsla_matrix_set_csr_algorithm": (I, [P, I, I]),
    "tbsla_matrix_set_sell_params": (I, [P, I, I, I, I]),
    "tbsla_matrix_set_pagerank_gather": (I, [P, I]),
    "tbsla_matrix_set_pagerank_fused": (I, [P, I]),
    "tbsla_matrix_set_pagerank_stream": (I, [P, I]),
    "tbsla_matrix_autotune": (I, [P, I, C.POINTER(Tuning), C.POINTER(Tuning), I, IP]),
    "tbsla_batch_create": (I, [C.POINTER(P), C.POINTER(P), I, I]),
    "tbsla_batch_destroy": (I, [P]),
    "tbsla_batch_rows": (I, [P, IP, C.POINTER(L)]),
    "tbsla_batch_cg": (I, [P, P, P, I, D, I, I, I, IP, DP]),
    "tbsla_batch_set_factors": (I, [P, C.POINTER(P), I, I]),
    "tbsla_batch_fallbacks": (I, [P, IP, IP]),
    "tbsla_batch_set_wait_limit": (I, [P, C.c_longlong]),
    "tbsla_batch_set_rows_per_thread": (I, [P, I]),
    "tbsla_batch_set_ctas_per_sm": (I, [P, I]),
    "tbsla_batch_tuning": (I, [P, IP, IP]),
    "tbsla_batch_engine": (I, [P, IP, IP, IP]),
    "tbsla_batch_set_seven_point": (I, [P, I]),
    "tbsla_batch_factor_mpnn": (I, [P, P, I]),
    "tbsla_batch_factor_dia": (I, [P, IP, IP, DP]),
    "tbsla_mpnn_create": (I, [C.POINTER(P), ULL]),
    "tbsla_mpnn_destroy": (I, [P]),
    "tbsla_mpnn_params": (I, [P, P, IP]),
    "tbsla_mpnn_set_params": (I, [P, P, I]),
    "tbsla_mpnn_loss_grad": (I, [P, P, I, P, DP, P]),
    "tbsla_mpnn_train_step": (I, [P, P, I, ULL, C.c_float, DP]),
    "tbsla_mpnn_factor": (I, [P, P, P]),
    "tbsla_Ax": (I, [P, P, P, I]),
    "tbsla_spmv": (I, [P, P, P, I]),
    "tbsla_Ax_device": (I, [P, P, P, I, P]),
    "tbsla_spmv_device": (I, [P, P, P, I, P]),
    "tbsla_csr_Ax_device_noalloc": (I, [I, L, I, P, P, P, P, P, P]),
    "tbsla_a_axpx_": (I, [P, P, P, I]),
    "tbsla_AAxpAx": (I, [P, P, P, P, I]),
    "tbsla_AAxpAxpx": (I, [P, P, P, P, I]),
    "tbsla_get_col_sums": (I, [P, P]),
    "tbsla_normalize_cols": (I, [P, P]),
    "tbsla_make_stochastic": (I, [P, P]),
    "tbsla_dense_multiply": (I, [P, P, P, I]),
    "tbsla_get_row_max_abs": (I, [P, P]),
    "tbsla_get_row_sums": (I, [P, P]),
    "tbsla_normalize_rows": (I, [P, P]),
    "tbsla_apply_exponential": (I, [P, P, I]),
    "tbsla_page_rank": (I, [P, D, D, I, P, IP, DP]),
    "tbsla_page_rank_batched": (I, [P, I, P, D, D, I, P, IP]),
    "tbsla_cg": (I, [P, P, P, I, D, I, I, IP, DP]),
}

for _name, (_res, _args) in _SIGS.items():
    _f = getattr(_lib, _name)
    _f.restype = _res
    _f.argtypes = _args

lib = _lib
EXPORTED = tuple(_SIGS)


def check(status: int, what: str = "") -> int:
    if status != OK:
        raise TbslaError(status, what)
    return status
