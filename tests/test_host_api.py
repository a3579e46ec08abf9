"""Host-side behaviour of the C ABI, no GPU needed: the library loads and
exports every entry point the header declares; generators, converting
constructors and binary I/O reproduce the reference's arrays and bytes
(golden vectors recorded from the reference); bad input is rejected on the
host with a status code."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import tbsla_gb300 as T
from conftest import ROOT, golden_cases, has_gpu
from tbsla_gb300 import _lib as L


def header_functions():
    text = open(os.path.join(ROOT, "include", "tbsla_gb300.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(tbsla_\w+)\(", text, re.M)))


def test_library_exports_every_declared_symbol():
    names = header_functions()
    assert len(names) >= 40
    so = C.CDLL(L.LIB_PATH)
    for n in names:
        assert hasattr(so, n), n
    assert set(names) == set(L.EXPORTED)
    assert T.lib.tbsla_version().startswith(b"tbsla_gb300")


def test_status_strings():
    for s in range(0, -10, -1):
        assert T.lib.tbsla_status_string(s) != b"unknown status"


def compare(m, case, key):
    info = m.info()
    gi = case["info"]
    for k, v in gi.items():
        if k == "max_col" and m.FORMAT != T.ELL:
            continue
        if k == "nnz" and m.FORMAT == T.DENSE and case["values"].size == 0:
            continue  # the reference leaves nnz uninitialised there
        assert info[k] == v, (key, k, info[k], v)
    arr = m.arrays()
    for k, g in case.items():
        if k in ("info", "ax"):
            continue
        mine = arr[k]
        if k in ("values", "colidx") and m.FORMAT == T.CSR:
            mine = mine[: int(arr["rowptr"][-1])] if arr["rowptr"].size else mine[:0]
        if g.size == 0 and (mine.size == 0 or not mine.any()):
            continue
        assert np.array_equal(mine, g), (key, k)


@pytest.mark.parametrize("kind", ["cdiag", "cqmat", "random"])
def test_generators_match_reference(golden, kind):
    n = 0
    for key, case in golden_cases(golden["gen"], kind).items():
        p = key.split("/")
        fmt = int(p[1])
        grid = tuple(int(t) for t in p[-1].split("-"))
        m = T.FORMATS[fmt]()
        if kind == "cdiag":
            m.fill_cdiag(int(p[2]), int(p[3]), int(p[4]), *grid)
        elif kind == "cqmat":
            m.fill_cqmat(int(p[2]), int(p[3]), int(p[4]), float(p[5]), int(p[6]), *grid)
        else:
            m.fill_random(int(p[2]), int(p[3]), float(p[4]), int(p[5]), *grid)
        compare(m, case, key)
        n += 1
    assert n >= 30


@pytest.mark.parametrize("kind", ["cdiag", "cqmat"])
def test_conversions_match_reference(golden, kind):
    for key, case in golden_cases(golden["gen"], kind + "_conv").items():
        p = key.split("/")
        coo = T.MatrixCOO()
        if kind == "cdiag":
            coo.fill_cdiag(int(p[2]), int(p[3]), int(p[4]))
        else:
            coo.fill_cqmat(int(p[2]), int(p[3]), int(p[4]), float(p[5]), int(p[6]))
        m = T.FORMATS[int(p[1])](coo)
        compare(m, case, key)


def test_write_matches_reference_bytes(golden, tmp_path):
    files = golden["files"]
    for key in files.files:
        kind, fmt = key.split("/")
        fmt = int(fmt)
        m = T.FORMATS[fmt]()
        if kind == "cdiag":
            m.fill_cdiag(10, 10, 2)
        elif kind == "cqmat":
            m.fill_cqmat(30, 30, 7, 0.5, 1)
        else:
            m.fill_cqmat(30, 20, 7, 0.5, 1, 1, 0, 2, 1)
        p = tmp_path / f"{kind}.{fmt}"
        m.write(p)
        mine = np.frombuffer(p.read_bytes(), np.uint8)
        ref = files[key]
        if fmt == T.CSR and kind != "cdiag":
            # the reference sizes CSR arrays by its over-counting first pass and
            # leaves the unused tail uninitialised: compare header + used part
            assert mine.size == ref.size
            hdr = 48
            nnz = int(np.frombuffer(ref[24:32].tobytes(), np.int64)[0])
            used = int(m.arrays()["rowptr"][-1])
            ln_row = int(np.frombuffer(ref[8:12].tobytes(), np.int32)[0])
            assert np.array_equal(mine[:hdr + 8 + used * 8], ref[:hdr + 8 + used * 8]), key
            off = hdr + 8 + nnz * 8
            assert np.array_equal(mine[off:off + 8 + (ln_row + 1) * 4 + 8 + used * 4],
                                  ref[off:off + 8 + (ln_row + 1) * 4 + 8 + used * 4]), key
        else:
            assert np.array_equal(mine, ref), key
        # read the reference's bytes back
        q = tmp_path / f"ref.{kind}.{fmt}"
        q.write_bytes(ref.tobytes())
        m2 = T.FORMATS[fmt]()
        m2.read(q)
        assert m2.info() == m.info()


def test_read_rejects_truncated_file(tmp_path):
    m = T.MatrixCSR()
    m.fill_cqmat(50, 50, 5, 0.3, 1)
    p = tmp_path / "m.csr"
    m.write(p)
    data = p.read_bytes()
    (tmp_path / "short.csr").write_bytes(data[: len(data) - 7])
    with pytest.raises(T.TbslaError) as e:
        T.MatrixCSR().read(tmp_path / "short.csr")
    assert e.value.status == L.ERR_IO
    with pytest.raises(T.TbslaError) as e:
        T.MatrixCSR().read(tmp_path / "missing.csr")
    assert e.value.status == L.ERR_IO
    # a file of another format is rejected on its array counts
    with pytest.raises(T.TbslaError):
        T.MatrixELL().read(p)


def test_read_offset_and_append(tmp_path):
    a, b = T.MatrixCOO(), T.MatrixCOO()
    a.fill_cdiag(12, 12, 1)
    b.fill_cqmat(9, 9, 3, 0.5, 2)
    p = tmp_path / "two.coo"
    a.write(p)
    size_a = p.stat().st_size
    b.write(p, append=True)
    m = T.MatrixCOO()
    m.read(p, size_a)
    assert m.info() == b.info()
    assert all(np.array_equal(m.arrays()[k], b.arrays()[k]) for k in ("values", "row", "col"))


def test_validation_rejects_bad_arrays():
    # out-of-range column
    m = T.MatrixCSR.from_arrays(3, 3, [0, 1, 2, 3], [0, 1, 3], [1.0, 1.0, 1.0])
    with pytest.raises(T.TbslaError) as e:
        m.upload()
    assert e.value.status == L.ERR_BAD_MATRIX
    # non-monotone row pointer
    m = T.MatrixCSR.from_arrays(3, 3, [0, 2, 1, 3], [0, 1, 2], [1.0, 1.0, 1.0])
    with pytest.raises(T.TbslaError) as e:
        m.upload()
    assert e.value.status == L.ERR_BAD_MATRIX
    # ELL column out of range
    m = T.MatrixELL.from_arrays(dict(n_row=2, n_col=2, ln_row=2, ln_col=2, nnz=2, max_col=1), [0, 5],
                                [1.0, 1.0])
    with pytest.raises(T.TbslaError) as e:
        m.upload()
    assert e.value.status == L.ERR_BAD_MATRIX
    # COO conversion with an out-of-range row
    coo = T.MatrixCOO.from_arrays(2, 2, [0, 2], [0, 1], [1.0, 1.0])
    with pytest.raises(T.TbslaError) as e:
        T.MatrixCSR(coo)
    assert e.value.status == L.ERR_BAD_MATRIX


def test_bad_arguments():
    with pytest.raises(T.TbslaError):
        T.MatrixCSR().fill_cdiag(10, 10, 1, 2, 0, 2, 1)  # pr >= NR
    with pytest.raises(T.TbslaError):
        T.MatrixCSR().set_tile(100)
    with pytest.raises(T.TbslaError):
        T.MatrixCOO().fill_powerlaw if False else T.MatrixDENSE().fill_dense_uniform(0, 4, 1)
    h = C.c_void_p()
    assert T.lib.tbsla_matrix_create(C.byref(h), 7) == L.ERR_INVALID_ARG
    # CSR kernel: -1 (automatic) .. 2
    m = T.MatrixCSR()
    for algo in (m.AUTO, m.MERGE, m.ROWBLOCK, m.SELL):
        m.set_algorithm(algo)
    for bad in (-2, 3):
        with pytest.raises(T.TbslaError):
            m.set_algorithm(bad)
    # sliced-ELL thresholds: 0 (automatic) .. 255; negative rejected
    m = T.MatrixCSR()
    m.set_sell_params(0, 0, 16384, 0)
    m.set_sell_params(255, 1000, 32, 1)
    for bad in ((-1, 0, 16384, 0), (256, 0, 16384, 0), (0, -1, 16384, 0), (0, 0, 16, 0), (0, 0, 16384, -1)):
        with pytest.raises(T.TbslaError):
            m.set_sell_params(*bad)


@pytest.mark.skipif(has_gpu(), reason="checks the no-device status on a host without a GPU")
def test_compute_without_gpu_fails_loudly():
    m = T.MatrixCSR()
    m.fill_cdiag(10, 10, 1)
    with pytest.raises(T.TbslaError) as e:
        m.spmv(np.arange(10.0))
    assert e.value.status == L.ERR_NO_DEVICE


def test_project_generators_are_deterministic():
    a, b = T.MatrixCSR(), T.MatrixCSR()
    a.fill_powerlaw(1 << 14, seed=11)
    b.fill_powerlaw(1 << 14, seed=11)
    x, y = a.arrays(), b.arrays()
    for k in x:
        assert np.array_equal(x[k], y[k])
    rp, ci = x["rowptr"], x["colidx"]
    lens = np.diff(rp)
    assert lens.min() >= 1 and lens.max() <= 4096
    # distinct, sorted columns per row
    d = np.diff(ci)
    starts = rp[1:-1]
    mask = np.ones(d.size, bool)
    mask[starts - 1] = False
    assert (d[mask] > 0).all()
    assert abs(lens.mean() - 16) < 2.5
    assert (np.abs(x["values"]) <= 1).all()
    g = T.MatrixCSR()
    g.fill_pa_graph(5000, 16.0, 2.1, 400, 0.05, 2)
    ga = g.arrays()
    outdeg = np.bincount(ga["colidx"], minlength=5000)
    assert 0.03 < (outdeg == 0).mean() < 0.08
    assert abs(outdeg.mean() - 16) < 3
    d7 = T.MatrixCSR()
    d7.fill_diffusion7(10, 1.0, 8.0, 3)
    a7 = d7.arrays()
    dense = np.zeros((1000, 1000))
    rows = np.repeat(np.arange(1000), np.diff(a7["rowptr"]))
    dense[rows, a7["colidx"]] = a7["values"]
    assert np.allclose(dense, dense.T)
    assert np.linalg.eigvalsh(dense).min() > 0


@pytest.mark.parametrize("n,max_len,local,band,seed", [(1 << 18, 4096, 0.3, 1024, 1), (5000, 300, 0.6, 16, 7),
                                                       (20000, 4096, 1.0, 64, 3)])
def test_oracle_powerlaw_generator_matches_library(n, max_len, local, band, seed):
    """The CPU baseline builds the large-SpMV matrix with the oracle's
    restatement of the library's power-law generator (so that it loads no
    library code); both must give the same arrays."""
    import oracle

    rp, ci, va = oracle.gen_powerlaw(n, 16.0, 2.0, max_len, local, band, seed)
    m = T.MatrixCSR()
    m.fill_powerlaw(n, 16.0, 2.0, max_len, local, band, seed)
    a = m.arrays()
    assert np.array_equal(rp, a["rowptr"]) and np.array_equal(ci, a["colidx"])
    assert np.array_equal(va, a["values"])
    assert np.array_equal(oracle.gen_uniform(n, 0.0, 1.0, seed), T.fill_uniform(n, 0.0, 1.0, seed))


def test_failed_host_allocation_returns_status_and_empties_matrix():
    """No C++ exception crosses the C ABI: a host allocation that cannot be
    made (here 2^60 entries) returns TBSLA_ERR_ALLOC, and a matrix whose
    arrays were being replaced is left empty, then takes new arrays as
    usual.  The source pointers are not read: the allocation fails first."""
    import ctypes as C

    from tbsla_gb300 import _lib as L

    m = C.c_void_p()
    L.check(L.lib.tbsla_matrix_create(C.byref(m), L.COO))
    try:
        vals = np.ones(3)
        rows = np.array([0, 1, 2], np.int32)
        cols = np.array([2, 1, 0], np.int32)
        ptr = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
        big = L.Info(n_row=3, n_col=3, ln_row=3, ln_col=3, nnz=1 << 60, NR=1, NC=1)
        st = L.lib.tbsla_matrix_set_coo(m, C.byref(big), ptr(vals), ptr(rows), ptr(cols))
        assert st == L.ERR_ALLOC
        info = L.Info()
        L.check(L.lib.tbsla_matrix_info(m, C.byref(info)))
        assert info.nnz == 0 and info.n_row == 0 and info.NR == 1
        ok = L.Info(n_row=3, n_col=3, ln_row=3, ln_col=3, nnz=3, NR=1, NC=1)
        L.check(L.lib.tbsla_matrix_set_coo(m, C.byref(ok), ptr(vals), ptr(rows), ptr(cols)))
        L.check(L.lib.tbsla_matrix_info(m, C.byref(info)))
        assert info.nnz == 3
    finally:
        L.lib.tbsla_matrix_destroy(m)
