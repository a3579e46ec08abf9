"""Python mirror of the reference's ``tbsla::cpp::Matrix`` classes
(src/cpp/include/tbsla/cpp/Matrix.hpp:11-57 and the five format classes) over
the C ABI.  Method names, argument meaning and defaults follow the reference
so that code written against the reference reads the same here:

    m = MatrixCSR(); m.fill_cqmat(nr, nc, c, q, s)
    r = m.spmv(v)                 # new array, zero-filled then Ax
    m.Ax(r, v)                    # CSR/ELL overwrite r, COO/SCOO/DENSE add to r

Vectors are float64 numpy arrays (host; copied to and from the GPU per
call) or CUDA tensors (``Ax_device``; no copies, no synchronisation).  Every
failure raises TbslaError carrying the C status code; there is no CPU
fallback for any compute call.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from ._lib import Info, TbslaError, check, lib


def _ptr(a: np.ndarray):
    return C.c_void_p(a.ctypes.data) if a is not None and a.size else None


def _f64(a, name="vector") -> np.ndarray:
    if not isinstance(a, np.ndarray) or a.dtype != np.float64 or not a.flags.c_contiguous:
        raise TypeError(f"{name} must be a C-contiguous float64 numpy array")
    return a


class Matrix:
    """Base of the five formats; owns one tbsla_matrix handle."""

    FORMAT = -1

    def __init__(self, coo: "MatrixCOO | None" = None, _handle=None, device: bool = False):
        """coo: converting constructor (MatrixCSR(const MatrixCOO&) ...);
        device=True does the conversion on the GPU: the (row, column) order
        of CSR / ELL by the radix sort, the DENSE scatter by a kernel."""
        h = C.c_void_p()
        if _handle is not None:
            h = _handle
        elif coo is not None:
            if not isinstance(coo, MatrixCOO):
                raise TypeError("conversion constructors take a MatrixCOO")
            fn = lib.tbsla_matrix_convert_device if device else lib.tbsla_matrix_convert
            check(fn(C.byref(h), coo._h, self.FORMAT), "convert")
        else:
            check(lib.tbsla_matrix_create(C.byref(h), self.FORMAT), "create")
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            lib.tbsla_matrix_destroy(h)
            self._h = C.c_void_p()

    # ---- metadata (Matrix.hpp:21-32) ----------------------------------------
    def info(self) -> dict:
        i = Info()
        check(lib.tbsla_matrix_info(self._h, C.byref(i)))
        return i.as_dict()

    def get_n_row(self): return self.info()["n_row"]
    def get_n_col(self): return self.info()["n_col"]
    def get_f_row(self): return self.info()["f_row"]
    def get_f_col(self): return self.info()["f_col"]
    def get_ln_row(self): return self.info()["ln_row"]
    def get_ln_col(self): return self.info()["ln_col"]
    def get_pr(self): return self.info()["pr"]
    def get_pc(self): return self.info()["pc"]
    def get_NR(self): return self.info()["NR"]
    def get_NC(self): return self.info()["NC"]
    def get_nnz(self): return self.info()["nnz"]
    def get_vectorization(self): return "CUDA sm_103a"

    def _out_len(self):
        i = self.info()
        return i["n_row"] if self.FORMAT == L.COO else i["ln_row"]

    def _in_len(self):
        i = self.info()
        return i["n_col"] if self.FORMAT == L.COO else i["ln_col"]

    # ---- generators (Matrix.hpp:40-42) ------------------------------------------
    def fill_cdiag(self, n_row, n_col, cdiag, pr=0, pc=0, NR=1, NC=1):
        check(lib.tbsla_matrix_fill_cdiag(self._h, n_row, n_col, cdiag, pr, pc, NR, NC), "fill_cdiag")

    def fill_cqmat(self, n_row, n_col, c, q, seed_mult=1, pr=0, pc=0, NR=1, NC=1):
        check(lib.tbsla_matrix_fill_cqmat(self._h, n_row, n_col, c, float(q), seed_mult, pr, pc, NR, NC),
              "fill_cqmat")

    def fill_random(self, n_row, n_col, nnz_ratio, seed_mult=1, pr=0, pc=0, NR=1, NC=1):
        check(lib.tbsla_matrix_fill_random(self._h, n_row, n_col, float(nnz_ratio), seed_mult, pr, pc,
                                           NR, NC), "fill_random")

    # ---- binary I/O (write / read) --------------------------------------------------
    def write(self, path: str, append: bool = False):
        check(lib.tbsla_matrix_write(self._h, str(path).encode(), int(append)), "write")

    def read(self, path: str, pos: int = 0):
        check(lib.tbsla_matrix_read(self._h, str(path).encode(), pos), "read")

    # ---- device copy ------------------------------------------------------------------
    def set_precision(self, prec: int):
        check(lib.tbsla_matrix_set_precision(self._h, prec), "set_precision")

    def upload(self):
        check(lib.tbsla_matrix_upload(self._h), "upload")

    def device_bytes(self) -> int:
        b = C.c_size_t()
        check(lib.tbsla_matrix_device_bytes(self._h, C.byref(b)), "device_bytes")
        return b.value

    def kernel_launches(self) -> int:
        """Kernel launches one Ax makes on the device copy."""
        k = C.c_int()
        check(lib.tbsla_matrix_kernel_launches(self._h, C.byref(k)), "kernel_launches")
        return k.value

    # ---- SpMV (Matrix.hpp:14-15) --------------------------------------------------------
    def Ax(self, r: np.ndarray, v: np.ndarray, vect_incr: int = 0):
        _f64(r, "r"), _f64(v, "v")
        if r.size < self._out_len() or v.size < self._in_len():
            raise ValueError("vector too short for the matrix")
        check(lib.tbsla_Ax(self._h, _ptr(r), _ptr(v), vect_incr), "Ax")

    def spmv(self, v: np.ndarray, vect_incr: int = 0) -> np.ndarray:
        _f64(v, "v")
        if v.size < self._in_len():
            raise ValueError("vector too short for the matrix")
        r = np.empty(max(self._out_len(), 1))
        check(lib.tbsla_spmv(self._h, _ptr(r), _ptr(v), vect_incr), "spmv")
        return r[: self._out_len()]

    def Ax_device(self, r, v, vect_incr: int = 0, stream=None):
        """r, v: float64 CUDA tensors (device pointers); stream: a torch
        stream or raw handle, None = the matrix's own stream."""
        s = None if stream is None else C.c_void_p(getattr(stream, "cuda_stream", stream))
        check(lib.tbsla_Ax_device(self._h, C.c_void_p(r.data_ptr()), C.c_void_p(v.data_ptr()),
                                  vect_incr, s), "Ax_device")

    def spmv_device(self, r, v, vect_incr: int = 0, stream=None):
        s = None if stream is None else C.c_void_p(getattr(stream, "cuda_stream", stream))
        check(lib.tbsla_spmv_device(self._h, C.c_void_p(r.data_ptr()), C.c_void_p(v.data_ptr()),
                                    vect_incr, s), "spmv_device")

    # ---- composite ops (Matrix.cpp:5-31) -------------------------------------------------
    def a_axpx_(self, v: np.ndarray, vect_incr: int = 0) -> np.ndarray:
        _f64(v, "v")
        r = np.empty(self._out_len())
        check(lib.tbsla_a_axpx_(self._h, _ptr(r), _ptr(v), vect_incr), "a_axpx_")
        return r

    def AAxpAx(self, r, v, buffer, vect_incr: int = 0):
        check(lib.tbsla_AAxpAx(self._h, _ptr(_f64(r)), _ptr(_f64(v)), _ptr(_f64(buffer)), vect_incr),
              "AAxpAx")

    def AAxpAxpx(self, r, v, buffer, vect_incr: int = 0):
        check(lib.tbsla_AAxpAxpx(self._h, _ptr(_f64(r)), _ptr(_f64(v)), _ptr(_f64(buffer)), vect_incr),
              "AAxpAxpx")

    # ---- column-stochastic preparation -----------------------------------------------------
    def get_col_sums(self, s: np.ndarray):
        check(lib.tbsla_get_col_sums(self._h, _ptr(_f64(s, "s"))), "get_col_sums")

    def normalize_cols(self, s: np.ndarray):
        check(lib.tbsla_normalize_cols(self._h, _ptr(_f64(s, "s"))), "normalize_cols")

    def make_stochastic(self, s: np.ndarray):
        check(lib.tbsla_make_stochastic(self._h, _ptr(_f64(s, "s"))), "make_stochastic")

    # ---- host arrays (numpy copies of the reference-layout arrays) --------------------------
    def arrays(self) -> dict:
        i = self.info()
        v, a, b = C.c_void_p(), C.c_void_p(), C.c_void_p()
        check(lib.tbsla_matrix_arrays(self._h, C.byref(v), C.byref(a), C.byref(b)))

        def grab(p, n, ct, dt):
            if n <= 0 or not p.value:
                return np.zeros(0, dtype=dt)
            return np.ctypeslib.as_array(C.cast(p, C.POINTER(ct)), shape=(n,)).copy()

        f = self.FORMAT
        nnz = i["nnz"]
        if f in (L.COO, L.SCOO):
            return {"values": grab(v, nnz, C.c_double, np.float64),
                    "row": grab(a, nnz, C.c_int, np.int32), "col": grab(b, nnz, C.c_int, np.int32)}
        if f == L.CSR:
            rp = grab(a, i["ln_row"] + 1 if a.value else 0, C.c_int, np.int32)
            return {"values": grab(v, nnz, C.c_double, np.float64), "rowptr": rp,
                    "colidx": grab(b, nnz, C.c_int, np.int32)}
        if f == L.ELL:
            n = i["ln_row"] * i["max_col"]
            return {"values": grab(v, n, C.c_double, np.float64), "columns": grab(a, n, C.c_int, np.int32)}
        n = i["ln_row"] * i["ln_col"]
        return {"values": grab(v, n, C.c_double, np.float64)}


def _info(**kw) -> Info:
    i = Info()
    i.NR = i.NC = 1
    for k, val in kw.items():
        setattr(i, k, val)
    return i


class MatrixCOO(Matrix):
    FORMAT = L.COO

    @classmethod
    def from_arrays(cls, n_row, n_col, row, col, values, fmt=None):
        m = cls()
        row = np.ascontiguousarray(row, np.int32)
        col = np.ascontiguousarray(col, np.int32)
        values = np.ascontiguousarray(values, np.float64)
        i = _info(n_row=n_row, n_col=n_col, ln_row=n_row, ln_col=n_col, nnz=len(values))
        check(lib.tbsla_matrix_set_coo(m._h, C.byref(i), _ptr(values), _ptr(row), _ptr(col)), "set_coo")
        return m


class MatrixSCOO(Matrix):
    FORMAT = L.SCOO

    def push_back(self, r: int, c: int, v: float):
        """Appends the entry (r, c, v) (MatrixSCOO.hpp:25)."""
        check(lib.tbsla_matrix_push_back(self._h, int(r), int(c), float(v)), "push_back")

    @classmethod
    def from_arrays(cls, info: dict, row, col, values):
        m = cls()
        row = np.ascontiguousarray(row, np.int32)
        col = np.ascontiguousarray(col, np.int32)
        values = np.ascontiguousarray(values, np.float64)
        i = _info(**info)
        check(lib.tbsla_matrix_set_coo(m._h, C.byref(i), _ptr(values), _ptr(row), _ptr(col)), "set_coo")
        return m


class MatrixCSR(Matrix):
    FORMAT = L.CSR

    @classmethod
    def from_arrays(cls, n_row, n_col, rowptr, colidx, values, **info):
        m = cls()
        rowptr = np.ascontiguousarray(rowptr, np.int32)
        colidx = np.ascontiguousarray(colidx, np.int32)
        values = np.ascontiguousarray(values, np.float64)
        kw = dict(n_row=n_row, n_col=n_col, ln_row=n_row, ln_col=n_col, nnz=len(values))
        kw.update(info)
        i = _info(**kw)
        check(lib.tbsla_matrix_set_csr(m._h, C.byref(i), _ptr(values), _ptr(rowptr), _ptr(colidx)),
              "set_csr")
        return m

    def set_tile(self, nnz_per_block: int):
        check(lib.tbsla_matrix_set_csr_tile(self._h, nnz_per_block), "set_csr_tile")

    AUTO, MERGE, ROWBLOCK, SELL = -1, 0, 1, 2

    def set_algorithm(self, algorithm: int, items: int = 0):
        check(lib.tbsla_matrix_set_csr_algorithm(self._h, algorithm, items), "set_csr_algorithm")

    def autotune(self, reps: int = 5, max_trials: int = 64):
        """Times the CSR kernel configurations on this matrix, keeps the
        fastest; returns (best, trials) as dicts."""
        best = L.Tuning()
        trials = (L.Tuning * max_trials)()
        nt = C.c_int()
        check(lib.tbsla_matrix_autotune(self._h, reps, C.byref(best), trials, max_trials, C.byref(nt)), "autotune")
        return best.as_dict(), [trials[i].as_dict() for i in range(nt.value)]

    def set_pagerank_gather(self, gather: int):
        """Batched PageRank (FP32 / BF16 values): X-row gathers in flight per
        warp, 8 or 16."""
        check(lib.tbsla_matrix_set_pagerank_gather(self._h, int(gather)), "set_pagerank_gather")

    def set_pagerank_stream(self, stream: bool):
        """Batched PageRank (FP32 / BF16 values): a warp walks a whole row
        block's entries as one stream (True, default) or takes one row at a
        time."""
        check(lib.tbsla_matrix_set_pagerank_stream(self._h, int(bool(stream))), "set_pagerank_stream")

    def set_pagerank_fused(self, fused: bool):
        """PageRank on the sliced-ELL kernel with one column block: the step's
        epilogue inside the SpMV launch (True, default) or a pass of its own."""
        check(lib.tbsla_matrix_set_pagerank_fused(self._h, int(bool(fused))), "set_pagerank_fused")

    def set_sell_params(self, short_thr: int = 0, long_thr: int = 0, sigma: int = 16384, col_block: int = 0):
        """Sliced-ELL layout thresholds (0: automatic), window and column
        block (0: 8,388,608 columns)."""
        check(lib.tbsla_matrix_set_sell_params(self._h, short_thr, long_thr, sigma, col_block), "set_sell_params")

    # ---- SpMM / sparse softmax (MatrixCSR.cpp:1269-1334) ---------------------
    def dense_multiply(self, B: np.ndarray) -> np.ndarray:
        B = np.ascontiguousarray(B, np.float64)
        Cm = np.empty((self.get_n_row(), B.shape[1]))
        check(lib.tbsla_dense_multiply(self._h, _ptr(B), _ptr(Cm), B.shape[1]), "dense_multiply")
        return Cm

    def get_row_max_abs(self) -> np.ndarray:
        out = np.empty(self.info()["ln_row"])
        check(lib.tbsla_get_row_max_abs(self._h, _ptr(out)), "get_row_max_abs")
        return out

    def get_row_sums(self, s: np.ndarray | None = None) -> np.ndarray:
        """Row sums in entry order (MatrixCSR::get_row_sums)."""
        out = np.empty(self.info()["ln_row"]) if s is None else s
        check(lib.tbsla_get_row_sums(self._h, _ptr(out)), "get_row_sums")
        return out

    def normalize_rows(self, s: np.ndarray):
        """a_ij /= s[i], 0 where s[i] = 0 (MatrixCSR::normalize_rows)."""
        check(lib.tbsla_normalize_rows(self._h, _ptr(_f64(s, "s"))), "normalize_rows")

    def apply_exponential(self, max_abs: np.ndarray | None = None, base: int = -1):
        mx = None if max_abs is None else _f64(max_abs, "max_abs")
        check(lib.tbsla_apply_exponential(self._h, _ptr(mx) if mx is not None else None, base),
              "apply_exponential")

    # project generators
    def fill_uniform_rows(self, n, k, seed):
        check(lib.tbsla_matrix_fill_uniform_rows(self._h, n, k, seed), "fill_uniform_rows")

    def fill_powerlaw(self, n, mean_len=16.0, zipf_s=2.0, max_len=4096, local_frac=0.3, band=1024,
                      seed=1):
        check(lib.tbsla_matrix_fill_powerlaw(self._h, n, mean_len, zipf_s, max_len, local_frac, band,
                                             seed), "fill_powerlaw")

    def fill_pa_graph(self, n, mean_deg=16.0, zipf_s=2.1, max_deg=4096, dangling_frac=0.05, seed=2):
        check(lib.tbsla_matrix_fill_pa_graph(self._h, n, mean_deg, zipf_s, max_deg, dangling_frac, seed),
              "fill_pa_graph")

    def fill_diffusion7(self, n, sigma=1.0, corr_len=8.0, seed=3):
        check(lib.tbsla_matrix_fill_diffusion7(self._h, n, sigma, corr_len, seed), "fill_diffusion7")

    # PageRank / CG
    def page_rank(self, beta=0.85, epsilon=1e-10, max_iterations=1000, out: np.ndarray | None = None):
        """PageRank vector of this column-stochastic matrix.  out: an
        optional float64 array of n entries that receives the result
        (repeated solves then reuse one host buffer instead of faulting in
        a fresh one each call)."""
        n = self.get_n_row()
        if out is None:
            x = np.empty(n)
        else:
            x = out
            if x.dtype != np.float64 or x.shape != (n,) or not x.flags.c_contiguous:
                raise ValueError("out must be a contiguous float64 array of n entries")
        it = C.c_int()
        err = C.c_double()
        st = lib.tbsla_page_rank(self._h, beta, epsilon, max_iterations, _ptr(x), C.byref(it), C.byref(err))
        if st not in (L.OK, L.ERR_NOT_CONVERGED):
            check(st, "page_rank")
        return x, it.value, err.value, st == L.OK

    def page_rank_batched(self, teleport: np.ndarray, beta=0.85, epsilon=1e-10, max_iterations=1000,
                          out: np.ndarray | None = None):
        """Personalised PageRank for the columns of `teleport` (n x nvec,
        nvec <= 32).  `out` (n x nvec float64, C-contiguous), when given,
        receives the result: a buffer reused across calls is written at the
        host link's rate, where a fresh one is first faulted in page by
        page."""
        n, nvec = teleport.shape
        t = np.ascontiguousarray(teleport, np.float64)
        if out is None:
            x = np.empty((n, nvec))
        else:
            if out.shape != (n, nvec) or out.dtype != np.float64 or not out.flags.c_contiguous:
                raise ValueError("out must be a C-contiguous float64 array of the teleport's shape")
            x = out
        it = C.c_int()
        st = lib.tbsla_page_rank_batched(self._h, nvec, _ptr(t), beta, epsilon, max_iterations, _ptr(x),
                                         C.byref(it))
        if st not in (L.OK, L.ERR_NOT_CONVERGED):
            check(st, "page_rank_batched")
        return x, it.value, st == L.OK

    def CG(self, b: np.ndarray, x: np.ndarray | None = None, max_iterations=10000, rel_tol=1e-8,
           precond=0, refresh=50):
        b = _f64(b, "b")
        x = np.zeros_like(b) if x is None else _f64(x, "x")
        it = C.c_int()
        rr = C.c_double()
        st = lib.tbsla_cg(self._h, _ptr(b), _ptr(x), max_iterations, rel_tol, precond, refresh,
                          C.byref(it), C.byref(rr))
        if st not in (L.OK, L.ERR_NOT_CONVERGED):
            check(st, "cg")
        return x, it.value, rr.value, st == L.OK


class MatrixELL(Matrix):
    FORMAT = L.ELL

    @classmethod
    def from_arrays(cls, info: dict, columns, values):
        m = cls()
        columns = np.ascontiguousarray(columns, np.int32)
        values = np.ascontiguousarray(values, np.float64)
        i = _info(**info)
        check(lib.tbsla_matrix_set_ell(m._h, C.byref(i), _ptr(values), _ptr(columns)), "set_ell")
        return m


class MatrixDENSE(Matrix):
    FORMAT = L.DENSE

    @classmethod
    def from_arrays(cls, n_row, n_col, values):
        m = cls()
        values = np.ascontiguousarray(values, np.float64).reshape(-1)
        i = _info(n_row=n_row, n_col=n_col, ln_row=n_row, ln_col=n_col, nnz=n_row * n_col)
        check(lib.tbsla_matrix_set_dense(m._h, C.byref(i), _ptr(values)), "set_dense")
        return m

    def fill_dense_uniform(self, n_row, n_col, seed):
        check(lib.tbsla_matrix_fill_dense_uniform(self._h, n_row, n_col, seed), "fill_dense_uniform")


FORMATS = {L.COO: MatrixCOO, L.SCOO: MatrixSCOO, L.CSR: MatrixCSR, L.ELL: MatrixELL,
           L.DENSE: MatrixDENSE}


class Batch:
    """Many SPD CSR systems solved together by batched CG (tbsla_batch_*)."""

    def __init__(self, systems, precision=L.F64):
        self._systems = list(systems)  # the device copy is built from their arrays
        arr = (C.c_void_p * len(systems))(*[s._h.value for s in systems])
        h = C.c_void_p()
        check(lib.tbsla_batch_create(C.byref(h), arr, len(systems), precision), "batch_create")
        self._h = h
        ns = C.c_int()
        off = (C.c_long * (len(systems) + 1))()
        check(lib.tbsla_batch_rows(self._h, C.byref(ns), off))
        self.offsets = np.array(off[:], np.int64)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            lib.tbsla_batch_destroy(h)
            self._h = C.c_void_p()

    def cg(self, rhs: np.ndarray, x: np.ndarray | None = None, max_iterations=10000, rel_tol=1e-8,
           precond=0, refresh=50, graph_iters=0):
        rhs = _f64(rhs, "rhs")
        x = np.zeros_like(rhs) if x is None else _f64(x, "x")
        ns = len(self.offsets) - 1
        its = np.zeros(ns, np.int32)
        rr = np.zeros(ns)
        st = lib.tbsla_batch_cg(self._h, _ptr(rhs), _ptr(x), max_iterations, rel_tol, precond, refresh,
                                graph_iters, its.ctypes.data_as(C.POINTER(C.c_int)),
                                rr.ctypes.data_as(C.POINTER(C.c_double)))
        if st not in (L.OK, L.ERR_NOT_CONVERGED):
            check(st, "batch_cg")
        return x, its, rr, st == L.OK

    def set_factors(self, factors, precision=L.F32):
        """Lower-triangular CSR factors L (one per system), stored in
        `precision`: cg(precond=2) then applies z = L (L^T r)."""
        self._factors = list(factors)
        arr = (C.c_void_p * len(factors))(*[f._h.value for f in factors])
        check(lib.tbsla_batch_set_factors(self._h, arr, len(factors), precision), "batch_set_factors")

    def factor_mpnn(self, net, precision=L.BF16):
        """The network's factor of every system, computed on the GPU from the
        batch's device copy of A straight into the batch's factor storage
        (no host round trip); then cg(precond=2)."""
        check(lib.tbsla_batch_factor_mpnn(self._h, net._h, precision), "batch_factor_mpnn")

    def factor_dia(self):
        """The factor in its diagonal-slot form: (deltas [nsys, 8], values
        [slots, n]) with slot 0 the diagonal."""
        k = C.c_int()
        check(lib.tbsla_batch_factor_dia(self._h, C.byref(k), None, None), "batch_factor_dia")
        ns = len(self.offsets) - 1
        n = int(self.offsets[-1])
        deltas = np.zeros(ns * 8, np.int32)
        vals = np.zeros(k.value * n)
        check(lib.tbsla_batch_factor_dia(self._h, None, deltas.ctypes.data_as(C.POINTER(C.c_int)),
                                         vals.ctypes.data_as(C.POINTER(C.c_double))), "batch_factor_dia")
        return deltas.reshape(ns, 8), vals.reshape(k.value, n)

    def fallbacks(self):
        """Per system after the last cg(): (fallback code, preconditioner
        used at exit).  Codes: 0 none, 1 the factor failed its check and
        Jacobi ran instead, 2 the factored iteration stalled (a refinement
        cycle that did not lower the FP64 true residual, or one of 25
        iterations or more that cut it by less than 10%) and Jacobi took
        over."""
        ns = len(self.offsets) - 1
        fb = np.zeros(ns, np.int32)
        used = np.zeros(ns, np.int32)
        check(lib.tbsla_batch_fallbacks(self._h, fb.ctypes.data_as(C.POINTER(C.c_int)),
                                        used.ctypes.data_as(C.POINTER(C.c_int))), "batch_fallbacks")
        return fb, used

    def set_rows_per_thread(self, rows: int):
        """Persistent engine: 4 rows per thread (16-byte loads, the default
        where the layout allows) or 1."""
        check(lib.tbsla_batch_set_rows_per_thread(self._h, int(rows)), "batch_set_rows_per_thread")

    def set_ctas_per_sm(self, ctas: int):
        """Persistent engine: CTAs per SM of the cooperative launch (0: as
        many as fit)."""
        check(lib.tbsla_batch_set_ctas_per_sm(self._h, int(ctas)), "batch_set_ctas_per_sm")

    def tuning(self) -> dict:
        """Current persistent-engine settings."""
        rpt, cps = C.c_int(), C.c_int()
        check(lib.tbsla_batch_tuning(self._h, C.byref(rpt), C.byref(cps)), "batch_tuning")
        return {"rows_per_thread": rpt.value, "ctas_per_sm": cps.value}

    def set_wait_limit(self, ns: int):
        """Bound on one grid-wide wait of the persistent solver (ns)."""
        check(lib.tbsla_batch_set_wait_limit(self._h, int(ns)), "batch_set_wait_limit")

    def engine(self) -> dict:
        """Engine of the last cg(): persistent (one cooperative launch) or
        multi-launch, and whether a CUDA graph replayed it."""
        p, g, s7 = C.c_int(), C.c_int(), C.c_int()
        check(lib.tbsla_batch_engine(self._h, C.byref(p), C.byref(g), C.byref(s7)), "batch_engine")
        return {"persistent": bool(p.value), "graph": bool(g.value), "seven_point": bool(s7.value)}

    def set_seven_point(self, on: bool):
        """Persistent engine: the seven-point form where it applies (True,
        default) or always the general form."""
        check(lib.tbsla_batch_set_seven_point(self._h, int(bool(on))), "batch_set_seven_point")


class MPNN:
    """The learned preconditioner: a message-passing network that maps an SPD
    CSR matrix A to a lower-triangular L on the pattern of tril(A), with
    M^-1 = L L^T (tbsla_mpnn_*).  Untrained, L = D^-1/2 (Jacobi)."""

    NPARAMS = 6467

    def __init__(self, seed: int = 0):
        h = C.c_void_p()
        check(lib.tbsla_mpnn_create(C.byref(h), seed), "mpnn_create")
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            lib.tbsla_mpnn_destroy(h)
            self._h = C.c_void_p()

    def params(self) -> np.ndarray:
        th = np.empty(self.NPARAMS, np.float32)
        check(lib.tbsla_mpnn_params(self._h, th.ctypes.data_as(C.c_void_p), None), "mpnn_params")
        return th

    def set_params(self, theta):
        th = np.ascontiguousarray(theta, np.float32)
        check(lib.tbsla_mpnn_set_params(self._h, th.ctypes.data_as(C.c_void_p), len(th)), "mpnn_set_params")

    def loss_grad(self, A, Z: np.ndarray):
        Z = np.ascontiguousarray(Z, np.float64)
        g = np.empty(self.NPARAMS, np.float32)
        loss = C.c_double()
        check(lib.tbsla_mpnn_loss_grad(self._h, A._h, Z.shape[1], Z.ctypes.data_as(C.c_void_p), C.byref(loss),
                                       g.ctypes.data_as(C.c_void_p)), "mpnn_loss_grad")
        return loss.value, g

    def train_step(self, A, probes: int = 8, seed: int = 0, lr: float = 1e-3) -> float:
        loss = C.c_double()
        check(lib.tbsla_mpnn_train_step(self._h, A._h, probes, seed, lr, C.byref(loss)), "mpnn_train_step")
        return loss.value

    def factor(self, A):
        Lm = MatrixCSR()
        check(lib.tbsla_mpnn_factor(self._h, A._h, Lm._h), "mpnn_factor")
        return Lm


def fill_uniform(n: int, lo: float, hi: float, seed: int, out: np.ndarray | None = None) -> np.ndarray:
    out = np.empty(n) if out is None else _f64(out, "out")
    check(lib.tbsla_fill_uniform(_ptr(out), n, lo, hi, seed), "fill_uniform")
    return out


def device_init(device: int = 0):
    check(lib.tbsla_device_init(device), "device_init")


__all__ = ["Matrix", "MatrixCOO", "MatrixSCOO", "MatrixCSR", "MatrixELL", "MatrixDENSE", "FORMATS", "MPNN",
           "fill_uniform", "device_init", "TbslaError"]
