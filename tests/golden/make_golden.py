"""Records the golden vectors of tests/golden/*.npz from the reference itself.

Runs where the reference tree is mounted: it builds the unmodified reference
core from its own sources (oracle/build.py -> oracle/_ref/libtbsla_ref.so)
and drives it through oracle/ref_shim.cpp with one OpenMP thread (the
reference's COO reduction and column sums are then deterministic).  What it
records:

* gen.npz    -- arrays + metadata of fill_cdiag / fill_cqmat / fill_random and
                of the converting constructors from COO, every format, the
                shapes and sweeps of src/cpp/tests/test_spmv_cdiag.cpp:77-106
                and test_spmv_cqmat.cpp, 1x1 and block grids; with the
                reference's Ax result for a fixed input (r0 = 0.5, v = iota)
* ops.npz    -- a_axpx_ / AAxpAx / AAxpAxpx (test_a_axpx__cdiag.cpp,
                test_AAxpAx_cdiag.cpp inputs), get_col_sums + normalize_cols
* files.npz  -- bytes of the reference's binary write() for each format
* cfg1.npz   -- the reference Ax of each format on the 10^4-row, 10-per-row
                uniform matrix and the 2000x2000 DENSE matrix produced by this
                library's generators (seed 0), x = U[0,1) seed 0, plus
                checksums of the generated arrays

Usage: TBSLA_REFERENCE_ROOT=<root of the TBSLA source tree> python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes as C
import os
import sys
import tempfile

os.environ["OMP_NUM_THREADS"] = "1"
ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

import oracle  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
META = "n_row n_col ln_row ln_col f_row f_col pr pc NR NC max_col".split()
GRIDS = [(0, 0, 1, 1), (1, 0, 2, 1), (0, 1, 1, 2), (1, 2, 2, 3)]


class Ref:
    def __init__(self):
        self.L = oracle.ref()
        if self.L is None:
            raise SystemExit("reference core not available: set TBSLA_REFERENCE_ROOT to the TBSLA source tree")

    def new(self, fmt):
        return C.c_void_p(self.L.ref_new(fmt))

    def info(self, h):
        meta = (C.c_int * 11)()
        nnz = C.c_long()
        self.L.ref_info(h, meta, C.byref(nnz))
        d = dict(zip(META, list(meta)))
        d["nnz"] = nnz.value
        return d

    def arrays(self, h, fmt):
        i = self.info(h)
        v, a, b = C.c_void_p(), C.c_void_p(), C.c_void_p()
        self.L.ref_arrays(h, C.byref(v), C.byref(a), C.byref(b))

        def grab(p, n, ct, dt):
            if n <= 0 or not p.value:
                return np.zeros(0, dt)
            return np.ctypeslib.as_array(C.cast(p, C.POINTER(ct)), shape=(n,)).copy()

        nnz = i["nnz"]
        if fmt in (0, 1):
            return {"values": grab(v, nnz, C.c_double, np.float64), "row": grab(a, nnz, C.c_int, np.int32),
                    "col": grab(b, nnz, C.c_int, np.int32)}
        if fmt == 2:
            rp = grab(a, i["ln_row"] + 1, C.c_int, np.int32)
            end = int(rp[-1]) if rp.size else 0
            return {"values": grab(v, end, C.c_double, np.float64), "rowptr": rp,
                    "colidx": grab(b, end, C.c_int, np.int32)}
        if fmt == 3:
            n = i["ln_row"] * i["max_col"]
            return {"values": grab(v, n, C.c_double, np.float64), "columns": grab(a, n, C.c_int, np.int32)}
        n = i["ln_row"] * i["ln_col"] if v.value else 0
        return {"values": grab(v, n, C.c_double, np.float64)}

    def ax(self, h, fmt, r0, v, vect_incr=0):
        r = r0.copy()
        self.L.ref_Ax(h, C.c_void_p(r.ctypes.data), C.c_void_p(v.ctypes.data), vect_incr)
        return r


def lens(fmt, info):
    if fmt == 0:
        return info["n_row"], info["n_col"]
    return info["ln_row"], info["ln_col"]


def record_matrix(out, key, R, h, fmt, with_ax=True):
    info = R.info(h)
    arr = R.arrays(h, fmt)
    out[key + "/info"] = np.array([info[k] for k in META] + [info["nnz"]], np.int64)
    for k, a in arr.items():
        out[key + "/" + k] = a
    if with_ax and (fmt != 4 or arr["values"].size):
        nr, nc = lens(fmt, info)
        r0 = np.full(max(nr, 1), 0.5)
        v = np.arange(max(nc, 1), dtype=np.float64)
        out[key + "/ax"] = R.ax(h, fmt, r0, v)


def gen(R):
    out = {}
    shapes_c = [((10, 10), range(0, 13)), ((5, 10), range(0, 13)), ((10, 5), range(0, 13)),
                ((30, 30), range(0, 25, 2)), ((20, 30), range(0, 25, 2)), ((30, 20), range(0, 25, 2))]
    for (nr, nc), cs in shapes_c:
        for c in cs:
            for grid in GRIDS if c in (0, 3, 6, 8) else GRIDS[:1]:
                g = "-".join(map(str, grid))
                for fmt in range(5):
                    h = R.new(fmt)
                    R.L.ref_fill_cdiag(h, nr, nc, c, *grid)
                    record_matrix(out, f"cdiag/{fmt}/{nr}/{nc}/{c}/{g}", R, h, fmt, with_ax=grid == (0, 0, 1, 1))
                    if fmt == 0 and grid == (0, 0, 1, 1):
                        for tf in range(1, 5):
                            h2 = C.c_void_p(R.L.ref_convert(h, tf))
                            record_matrix(out, f"cdiag_conv/{tf}/{nr}/{nc}/{c}", R, h2, tf)
                            R.L.ref_delete(h2)
                    R.L.ref_delete(h)
    for nr, nc in [(10, 10), (5, 10), (10, 5), (30, 30), (20, 30), (30, 20)]:
        for c in (1, 3, 7, 12):
            for q in (0.0, 0.5, 1.0):
                for s in (0, 3):
                    for grid in GRIDS if (c == 7 and s == 3) else GRIDS[:1]:
                        g = "-".join(map(str, grid))
                        for fmt in range(5):
                            h = R.new(fmt)
                            R.L.ref_fill_cqmat(h, nr, nc, c, q, s, *grid)
                            record_matrix(out, f"cqmat/{fmt}/{nr}/{nc}/{c}/{q}/{s}/{g}", R, h, fmt,
                                          with_ax=grid == (0, 0, 1, 1))
                            if fmt == 0 and grid == (0, 0, 1, 1):
                                for tf in range(1, 5):
                                    h2 = C.c_void_p(R.L.ref_convert(h, tf))
                                    record_matrix(out, f"cqmat_conv/{tf}/{nr}/{nc}/{c}/{q}/{s}", R, h2, tf)
                                    R.L.ref_delete(h2)
                            R.L.ref_delete(h)
    # fill_random only where the reference's column repair (fix_list,
    # values_generation.cpp:162-203) never runs out of room for a row: there it
    # leaves the slot uninitialised and the output depends on heap contents.
    libc = C.CDLL(None)
    libc.rand_r.argtypes = [C.POINTER(C.c_uint)]

    def runs_out(nr, nc, ratio, s):
        c = max(1, int(nc * ratio))
        cc = min(c, nc)
        for i in range(nr):
            seed = C.c_uint((s * i * cc) & 0xFFFFFFFF if s > 0 else (i * cc) & 0xFFFFFFFF)
            raw = [libc.rand_r(C.byref(seed)) % nc for _ in range(cc)]
            used = set()
            dup = []
            for v in raw:
                dup.append(v in used)
                used.add(v)
            for k, v in enumerate(raw):
                if not dup[k]:
                    continue
                step = -1 if v > nc // 2 else 1
                while v in used and 0 < v < nc - 1:
                    v += step
                if v in used:
                    return True
                used.add(v)
        return False

    for nr, nc in [(30, 30), (20, 30), (30, 20), (100, 100), (64, 200), (200, 500)]:
        for s in (1, 2, 3):
            if runs_out(nr, nc, 0.1, s):
                continue
            for grid in GRIDS[:2]:
                g = "-".join(map(str, grid))
                for fmt in (1, 2, 3):
                    h = R.new(fmt)
                    R.L.ref_fill_random(h, nr, nc, 0.1, s, *grid)
                    record_matrix(out, f"random/{fmt}/{nr}/{nc}/0.1/{s}/{g}", R, h, fmt,
                                  with_ax=grid == (0, 0, 1, 1))
                    R.L.ref_delete(h)
    np.savez_compressed(os.path.join(OUT, "gen.npz"), **out)
    return len(out)


def ops(R):
    out = {}
    for n in (10, 30):
        for c in (0, 1, 3, 5, 9):
            for fmt in range(5):
                h = R.new(fmt)
                R.L.ref_fill_cdiag(h, n, n, c, 0, 0, 1, 1)
                v = 2 * np.arange(n, dtype=np.float64) + 1  # test_a_axpx__cdiag.cpp:28
                r = np.zeros(n)
                R.L.ref_a_axpx_(h, C.c_void_p(v.ctypes.data), 0, C.c_void_p(r.ctypes.data), n)
                out[f"a_axpx/{fmt}/{n}/{c}"] = r
                r = np.full(n, 0.25)
                buf = np.full(n, 0.125)
                R.L.ref_AAxpAx(h, C.c_void_p(r.ctypes.data), C.c_void_p(v.ctypes.data),
                               C.c_void_p(buf.ctypes.data), 0)
                out[f"AAxpAx/{fmt}/{n}/{c}/r"] = r
                out[f"AAxpAx/{fmt}/{n}/{c}/buffer"] = buf
                r = np.full(n, 0.25)
                buf = np.full(n, 0.125)
                R.L.ref_AAxpAxpx(h, C.c_void_p(r.ctypes.data), C.c_void_p(v.ctypes.data),
                                 C.c_void_p(buf.ctypes.data), 0)
                out[f"AAxpAxpx/{fmt}/{n}/{c}/r"] = r
                out[f"AAxpAxpx/{fmt}/{n}/{c}/buffer"] = buf
                R.L.ref_delete(h)
    for key, fill in [("cqmat", lambda h: R.L.ref_fill_cqmat(h, 40, 40, 6, 0.4, 2, 0, 0, 1, 1)),
                      ("cdiag", lambda h: R.L.ref_fill_cdiag(h, 40, 40, 3, 0, 0, 1, 1))]:
        h = R.new(2)
        fill(h)
        s = np.zeros(40)
        R.L.ref_get_col_sums(h, C.c_void_p(s.ctypes.data))
        out[f"colsum/{key}/s"] = s.copy()
        R.L.ref_normalize_cols(h, C.c_void_p(s.ctypes.data))
        out[f"colsum/{key}/values"] = R.arrays(h, 2)["values"]
        R.L.ref_delete(h)
    np.savez_compressed(os.path.join(OUT, "ops.npz"), **out)


def files(R):
    out = {}
    with tempfile.TemporaryDirectory() as td:
        for fmt in range(5):
            for key, fill in [("cdiag", lambda h: R.L.ref_fill_cdiag(h, 10, 10, 2, 0, 0, 1, 1)),
                              ("cqmat", lambda h: R.L.ref_fill_cqmat(h, 30, 30, 7, 0.5, 1, 0, 0, 1, 1)),
                              ("cqmat_block", lambda h: R.L.ref_fill_cqmat(h, 30, 20, 7, 0.5, 1, 1, 0, 2, 1))]:
                h = R.new(fmt)
                fill(h)
                p = os.path.join(td, "m.bin")
                R.L.ref_write(h, p.encode())
                out[f"{key}/{fmt}"] = np.frombuffer(open(p, "rb").read(), np.uint8)
                R.L.ref_delete(h)
    np.savez_compressed(os.path.join(OUT, "files.npz"), **out)


def cfg1(R):
    import tbsla_gb300 as T
    out = {}
    n = 10_000
    csr = T.MatrixCSR()
    csr.fill_uniform_rows(n, 10, 0)
    a = csr.arrays()
    x = T.fill_uniform(n, 0.0, 1.0, 0)
    out["x_sum"] = np.array([x.sum()])
    out["csr_checksum"] = np.array([a["rowptr"].astype(np.int64).sum(), a["colidx"].astype(np.int64).sum(),
                                    0], np.int64)
    out["csr_values_sum"] = np.array([a["values"].sum(), np.abs(a["values"]).sum()])
    rows = np.repeat(np.arange(n, dtype=np.int32), np.diff(a["rowptr"]))
    meta = np.array([n, n, n, n, 0, 0, 0, 0, 1, 1, 0], np.int32)
    coo = R.new(0)
    R.L.ref_adopt(coo, C.c_void_p(meta.ctypes.data), C.c_long(len(rows)), C.c_void_p(a["values"].ctypes.data),
                  C.c_void_p(rows.ctypes.data), C.c_void_p(a["colidx"].ctypes.data))
    for fmt in range(5):
        h = coo if fmt == 0 else C.c_void_p(R.L.ref_convert(coo, fmt))
        r0 = np.zeros(n)
        out[f"y/{fmt}"] = R.ax(h, fmt, r0, x)
        if fmt:
            R.L.ref_delete(h)
    R.L.ref_delete(coo)
    d = T.MatrixDENSE()
    d.fill_dense_uniform(2000, 2000, 0)
    dv = d.arrays()["values"]
    out["dense_values_sum"] = np.array([dv.sum(), np.abs(dv).sum()])
    xd = T.fill_uniform(2000, 0.0, 1.0, 0)
    hd = R.new(4)
    meta = np.array([2000, 2000, 2000, 2000, 0, 0, 0, 0, 1, 1, 0], np.int32)
    R.L.ref_adopt(hd, C.c_void_p(meta.ctypes.data), C.c_long(2000 * 2000), C.c_void_p(dv.ctypes.data),
                  None, None)
    out["y_dense"] = R.ax(hd, 4, np.zeros(2000), xd)
    R.L.ref_delete(hd)
    np.savez_compressed(os.path.join(OUT, "cfg1.npz"), **out)


def spmm(R):
    """dense_multiply, get_row_max_abs, apply_exponential, get_row_sums and
    normalize_rows of the reference's MatrixCSR (MatrixCSR.cpp:1147-1190,
    1269-1334) on cqmat / cdiag / random matrices."""
    out = {}
    fills = {"cqmat": lambda h: R.L.ref_fill_cqmat(h, 40, 40, 6, 0.4, 2, 0, 0, 1, 1),
             "cdiag": lambda h: R.L.ref_fill_cdiag(h, 40, 40, 3, 0, 0, 1, 1),
             "random": lambda h: R.L.ref_fill_random(h, 60, 50, 0.1, 3, 0, 0, 1, 1)}
    rng = np.random.default_rng(11)
    for key, fill in fills.items():
        h = R.new(2)
        fill(h)
        i = R.info(h)
        for cols in (1, 5, 33):
            B = rng.uniform(-1, 1, (i["n_col"], cols))
            Cm = np.full((i["n_row"], cols), 7.0)
            R.L.ref_dense_multiply(h, C.c_void_p(B.ctypes.data), C.c_void_p(Cm.ctypes.data), cols)
            out[f"{key}/B{cols}"] = B
            out[f"{key}/C{cols}"] = Cm
        mx = np.zeros(i["ln_row"])
        R.L.ref_row_max_abs(h, C.c_void_p(mx.ctypes.data))
        out[f"{key}/max_abs"] = mx
        R.L.ref_delete(h)
        for tag, use_max, base in (("exp_max", True, -1), ("exp", False, -1), ("pow2_max", True, 2)):
            h = R.new(2)
            fill(h)
            R.L.ref_apply_exponential(h, C.c_void_p(mx.ctypes.data) if use_max else None, base)
            out[f"{key}/{tag}"] = R.arrays(h, 2)["values"]
            R.L.ref_delete(h)
        h = R.new(2)
        fill(h)
        rs = np.zeros(i["ln_row"])
        R.L.ref_row_sums(h, C.c_void_p(rs.ctypes.data))
        out[f"{key}/row_sums"] = rs
        R.L.ref_delete(h)
        # normalize_rows by the row sums, and by sums with every third one
        # zero (the reference's safeguard sets those rows to 0)
        rz = rs.copy()
        rz[::3] = 0
        for tag, sv in (("norm_rows", rs), ("norm_rows_zero", rz)):
            h = R.new(2)
            fill(h)
            sv = np.ascontiguousarray(sv)
            R.L.ref_normalize_rows(h, C.c_void_p(sv.ctypes.data))
            out[f"{key}/{tag}"] = R.arrays(h, 2)["values"]
            R.L.ref_delete(h)
    np.savez_compressed(os.path.join(OUT, "spmm.npz"), **out)


if __name__ == "__main__":
    R = Ref()
    if len(sys.argv) > 1:  # only the named fixtures
        for name in sys.argv[1:]:
            globals()[name](R)
        raise SystemExit(0)
    print("gen", gen(R))
    ops(R)
    files(R)
    cfg1(R)
    spmm(R)
    print("done")
