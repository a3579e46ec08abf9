"""ORACLE — test infrastructure only.

numpy front end of the C restatement (``tbsla_oracle.c``) and, where it was
built, of the unmodified reference core (``_ref/libtbsla_ref.so``).  Only the
test suite, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use
this package, and only as the checker; the product library never imports it.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

HERE = os.path.dirname(os.path.abspath(__file__))
_o: C.CDLL | None = None
_r: C.CDLL | None = None

P = C.c_void_p
I = C.c_int
L = C.c_long
D = C.c_double


def _p(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def lib() -> C.CDLL:
    global _o
    if _o is None:
        path = _build.build_oracle()
        _o = C.CDLL(path)
        _o.orc_pagerank.restype = I
        _o.orc_cg.restype = I
        _o.orc_ell_max_col.restype = I
        _o.orc_gen_powerlaw_rows.restype = L
        _o.orc_gen_powerlaw_rows.argtypes = [I, D, D, I, D, I, C.c_ulonglong, P]
        _o.orc_gen_powerlaw_entries.argtypes = [I, D, I, C.c_ulonglong, P, P, P]
        _o.orc_gen_uniform.argtypes = [P, L, D, D, C.c_ulonglong]
    return _o


def ref_available() -> bool:
    try:
        return ref() is not None
    except OSError:
        return False


def ref() -> C.CDLL | None:
    """The reference core compiled from its own sources (None if absent)."""
    global _r
    if _r is None:
        path = _build.build_reference()
        if path is None or not os.path.exists(path):
            return None
        _r = C.CDLL(path)
        _r.ref_new.restype = P
        _r.ref_convert.restype = P
        _r.ref_convert.argtypes = [P, I]
        for name in ("ref_delete", "ref_fill_cdiag", "ref_fill_cqmat", "ref_fill_random", "ref_info",
                     "ref_arrays", "ref_adopt", "ref_write", "ref_read", "ref_Ax", "ref_spmv",
                     "ref_a_axpx_", "ref_AAxpAx", "ref_AAxpAxpx", "ref_get_col_sums",
                     "ref_normalize_cols", "ref_dense_multiply", "ref_row_max_abs", "ref_apply_exponential",
                     "ref_row_sums", "ref_normalize_rows"):
            getattr(_r, name).restype = None if not name.endswith(("write", "read")) else I
        _r.ref_fill_cqmat.argtypes = [P, I, I, I, D, C.c_uint, I, I, I, I]
        _r.ref_fill_random.argtypes = [P, I, I, D, C.c_uint, I, I, I, I]
        _r.ref_adopt.argtypes = [P, P, L, P, P, P]
        _r.ref_dense_multiply.argtypes = [P, P, P, I]
        _r.ref_apply_exponential.argtypes = [P, P, I]
    return _r


# ---- restated kernels ---------------------------------------------------------

def csr_ax(rowptr, colidx, values, v, r=None, f_col=0, nnz=None, threads=False):
    n = len(rowptr) - 1
    r = np.zeros(n) if r is None else r
    nnz = int(rowptr[-1]) if nnz is None else nnz
    fn = lib().orc_csr_ax_omp if threads else lib().orc_csr_ax
    fn(I(n), I(f_col), L(nnz), _p(values), _p(rowptr), _p(colidx), _p(v), _p(r))
    return r


def gen_powerlaw(n, mean_len=16.0, zipf_s=2.0, max_len=4096, local_frac=0.3, band=1024, seed=1):
    """The large-SpMV workload matrix as CSR arrays (rowptr, colidx, values),
    restated from this library's generator so that the CPU baseline does not
    load the library it is compared with."""
    rowptr = np.zeros(n + 1, np.int32)
    nnz = lib().orc_gen_powerlaw_rows(I(n), D(mean_len), D(zipf_s), I(max_len), D(local_frac), I(band),
                                      C.c_ulonglong(seed), _p(rowptr))
    if nnz < 0:
        raise ValueError("bad power-law parameters")
    colidx = np.empty(nnz, np.int32)
    values = np.empty(nnz, np.float64)
    lib().orc_gen_powerlaw_entries(I(n), D(local_frac), I(band), C.c_ulonglong(seed), _p(rowptr), _p(colidx),
                                   _p(values))
    return rowptr, colidx, values


def gen_uniform(n, lo, hi, seed):
    out = np.empty(n)
    lib().orc_gen_uniform(_p(out), L(n), D(lo), D(hi), C.c_ulonglong(seed))
    return out


def csr_ax_f32(rowptr, colidx, values32, v, r=None, f_col=0):
    n = len(rowptr) - 1
    r = np.zeros(n) if r is None else r
    lib().orc_csr_ax_f32_omp(I(n), I(f_col), L(int(rowptr[-1])), _p(values32), _p(rowptr), _p(colidx),
                             _p(v), _p(r))
    return r


def csr_absrow(rowptr, colidx, values, v, f_col=0):
    n = len(rowptr) - 1
    out = np.zeros(n)
    lib().orc_csr_absrow(I(n), I(f_col), _p(values), _p(rowptr), _p(colidx), _p(v), _p(out))
    return out


def ell_ax(values, columns, ln_row, max_col, v, r=None, f_col=0, nnz=1):
    r = np.zeros(ln_row) if r is None else r
    lib().orc_ell_ax(I(ln_row), I(max_col), I(f_col), L(nnz), _p(values), _p(columns), _p(v), _p(r))
    return r


def coo_ax(n_row, row, col, values, v, r=None, vect_incr=0):
    r = np.zeros(n_row) if r is None else r
    lib().orc_coo_ax(I(n_row), L(len(values)), _p(values), _p(row), _p(col), _p(v), _p(r), I(vect_incr))
    return r


def scoo_ax(ln_row, f_row, f_col, row, col, values, v, r=None, vect_incr=0):
    r = np.zeros(ln_row) if r is None else r
    lib().orc_scoo_ax(I(ln_row), I(f_row), I(f_col), L(len(values)), _p(values), _p(row), _p(col), _p(v),
                      _p(r), I(vect_incr))
    return r


def dense_ax(values, ln_row, ln_col, v, r=None, nnz=1, threads=False):
    r = np.zeros(ln_row) if r is None else r
    fn = lib().orc_dense_ax_omp if threads else lib().orc_dense_ax
    fn(I(ln_row), I(ln_col), L(nnz), _p(values), _p(v), _p(r))
    return r


def coo_to_csr(n_row, row, col, values):
    nnz = len(values)
    rowptr = np.zeros(n_row + 1, np.int32)
    colidx = np.zeros(nnz, np.int32)
    vals = np.zeros(nnz)
    lib().orc_coo_to_csr(I(n_row), L(nnz), _p(row), _p(col), _p(values), _p(rowptr), _p(colidx), _p(vals))
    return rowptr, colidx, vals


def coo_to_ell(n_row, row, col, values):
    nnz = len(values)
    mc = lib().orc_ell_max_col(I(n_row), L(nnz), _p(row))
    columns = np.zeros(n_row * mc, np.int32)
    vals = np.zeros(n_row * mc)
    lib().orc_coo_to_ell(I(n_row), L(nnz), _p(row), _p(col), _p(values), I(mc), _p(columns), _p(vals))
    return mc, columns, vals


def coo_to_dense(ln_row, ln_col, row, col, values):
    d = np.zeros(ln_row * ln_col)
    lib().orc_coo_to_dense(I(ln_row), I(ln_col), L(len(values)), _p(row), _p(col), _p(values), _p(d))
    return d


def csr_col_sums(rowptr, colidx, values, n_col, f_col=0):
    s = np.zeros(n_col)
    lib().orc_csr_col_sums(I(len(rowptr) - 1), I(f_col), L(int(rowptr[-1])), _p(values), _p(rowptr),
                           _p(colidx), _p(s))
    return s


def csr_normalize_cols(rowptr, colidx, values, s, f_col=0):
    vals = values.copy()
    lib().orc_csr_normalize_cols(I(len(rowptr) - 1), I(f_col), L(int(rowptr[-1])), _p(vals), _p(rowptr),
                                 _p(colidx), _p(s))
    return vals


def dangling_of(rowptr, colidx, n):
    has = np.zeros(n, bool)
    has[colidx[: int(rowptr[-1])]] = True
    return (~has).astype(np.uint8)


def pagerank(rowptr, colidx, values, beta=0.85, epsilon=1e-10, max_iterations=1000, stop_early=True,
             teleport=None):
    n = len(rowptr) - 1
    x = np.zeros(n)
    err = C.c_double()
    it = lib().orc_pagerank(I(n), _p(rowptr), _p(colidx), _p(values), _p(teleport), D(beta),
                            D(epsilon), I(max_iterations), I(int(stop_early)), _p(x), C.byref(err))
    return x, it, err.value


def cg(rowptr, colidx, values, b, x0=None, max_iterations=10000, rel_tol=1e-8, diag_inv=None):
    n = len(rowptr) - 1
    x = np.zeros(n) if x0 is None else x0.copy()
    rr = C.c_double()
    it = lib().orc_cg(I(n), _p(rowptr), _p(colidx), _p(values), _p(diag_inv), _p(b), _p(x),
                      I(max_iterations), D(rel_tol), C.byref(rr))
    return x, it, rr.value


def csr_dense_multiply(rowptr, colidx, values, B):
    n = len(rowptr) - 1
    B = np.ascontiguousarray(B, np.float64)
    cols = B.shape[1]
    Cm = np.empty((n, cols))
    lib().orc_csr_dense_multiply(I(n), _p(values), _p(rowptr), _p(colidx), _p(B), _p(Cm), I(cols))
    return Cm


def csr_row_max_abs(rowptr, values):
    n = len(rowptr) - 1
    out = np.empty(n)
    lib().orc_csr_row_max_abs(I(n), _p(values), _p(rowptr), _p(out))
    return out


def csr_row_sums(rowptr, values):
    n = len(rowptr) - 1
    out = np.empty(n)
    lib().orc_csr_row_sums(I(n), _p(values), _p(rowptr), _p(out))
    return out


def csr_normalize_rows(rowptr, values, s):
    v = np.array(values, np.float64)
    lib().orc_csr_normalize_rows(I(len(rowptr) - 1), _p(v), _p(rowptr), _p(np.ascontiguousarray(s, np.float64)))
    return v


def csr_apply_exponential(rowptr, values, max_abs=None, base=-1):
    v = np.array(values, np.float64)
    lib().orc_csr_apply_exponential(I(len(rowptr) - 1), _p(v), _p(rowptr), _p(max_abs), I(base))
    return v


def bf16_round(a: np.ndarray) -> np.ndarray:
    """float64 -> bfloat16 (round to nearest even, from the double's bits)
    -> float64, the rounding the device narrowing applies."""
    b = np.ascontiguousarray(a, np.float64).view(np.uint64).copy()
    finite = (b & np.uint64(0x7FF0000000000000)) != np.uint64(0x7FF0000000000000)
    add = np.uint64((1 << 44) - 1) + ((b >> np.uint64(45)) & np.uint64(1))
    b = np.where(finite, (b + add) & ~np.uint64((1 << 45) - 1), b)
    return b.view(np.float64).astype(np.float32).astype(np.float64)


def rel_err_normalized(y, y_ref, scale):
    """max_i |y_i - y_ref_i| / scale_i with scale_i = sum_j |a_ij x_j| (0/0 -> 0)."""
    d = np.abs(np.asarray(y) - np.asarray(y_ref))
    s = np.asarray(scale)
    out = np.where(s > 0, d / np.where(s > 0, s, 1), np.where(d > 0, np.inf, 0))
    return float(out.max()) if out.size else 0.0
