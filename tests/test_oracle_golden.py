"""Pins the oracle (the C restatement in oracle/tbsla_oracle.c) against the
golden vectors recorded from the reference itself (tests/golden/make_golden.py):
every restated Ax, conversion, composite op and column-sum must reproduce
the reference's output bit for bit (the restatement keeps the reference's
evaluation order and rounding)."""
import numpy as np
import pytest

import oracle
from conftest import golden_cases, info_of


def oracle_ax(fmt, case, r0, v):
    i = case["info"]
    r = r0.copy()
    if fmt == 0:
        oracle.coo_ax(i["n_row"], case["row"], case["col"], case["values"], v, r)
    elif fmt == 1:
        if i["nnz"]:
            oracle.scoo_ax(i["ln_row"], i["f_row"], i["f_col"], case["row"], case["col"], case["values"], v, r)
    elif fmt == 2:
        if i["nnz"]:
            oracle.csr_ax(case["rowptr"], case["colidx"], case["values"], v, r, f_col=i["f_col"], nnz=i["nnz"])
    elif fmt == 3:
        oracle.ell_ax(case["values"], case["columns"], i["ln_row"], i["max_col"], v, r, f_col=i["f_col"],
                      nnz=i["nnz"])
    else:
        oracle.dense_ax(case["values"], i["ln_row"], i["ln_col"], v, r, nnz=i["nnz"])
    return r


def lens(fmt, i):
    return (i["n_row"], i["n_col"]) if fmt == 0 else (i["ln_row"], i["ln_col"])


@pytest.mark.parametrize("prefix", ["cdiag", "cqmat", "random", "cdiag_conv", "cqmat_conv"])
def test_oracle_ax_matches_reference(golden, prefix):
    cases = golden_cases(golden["gen"], prefix)
    n = 0
    for key, case in cases.items():
        if "ax" not in case:
            continue
        fmt = int(key.split("/")[1])
        nr, nc = lens(fmt, case["info"])
        r0 = np.full(max(nr, 1), 0.5)
        v = np.arange(max(nc, 1), dtype=np.float64)
        got = oracle_ax(fmt, case, r0, v)
        assert np.array_equal(got, case["ax"]), key
        n += 1
    assert n >= 20


def test_cdiag_closed_form(golden):
    """compute_spmv_res_cdiag (src/cpp/utils/array.cpp:17-30) restated: the
    golden Ax results equal the closed form (plus r0 for accumulating formats)."""
    for key, case in golden_cases(golden["gen"], "cdiag").items():
        if "ax" not in case or not key.endswith("0-0-1-1"):
            continue
        fmt, nr, nc, c = (int(t) for t in key.split("/")[1:5])
        v = np.arange(nc, dtype=np.float64)
        exp = np.zeros(nr)
        for i in range(nr):
            for j in (i - c, i + c) if c else (i,):
                if 0 <= j < nc:
                    exp[i] += v[j]
        # accumulating formats add to r0 = 0.5; CSR / ELL overwrite r but leave
        # it untouched when the matrix is empty
        if fmt in (0, 1, 4) or case["info"]["nnz"] == 0:
            exp += 0.5
        assert np.array_equal(case["ax"][:nr], exp), key


@pytest.mark.parametrize("prefix", ["cdiag", "cqmat"])
def test_oracle_conversions_match_reference(golden, prefix):
    g = golden["gen"]
    coo_cases = golden_cases(g, prefix)
    conv = golden_cases(g, prefix + "_conv")
    n = 0
    for key, case in conv.items():
        parts = key.split("/")
        tf = int(parts[1])
        src = coo_cases["/".join([prefix, "0"] + parts[2:] + ["0-0-1-1"])]
        si = src["info"]
        if tf == 2:
            rp, ci, va = oracle.coo_to_csr(si["n_row"], src["row"], src["col"], src["values"])
            assert np.array_equal(rp, case["rowptr"]) and np.array_equal(ci, case["colidx"]), key
            assert np.array_equal(va, case["values"]), key
        elif tf == 3:
            if si["nnz"] == 0:
                continue
            mc, cols, vals = oracle.coo_to_ell(si["n_row"], src["row"], src["col"], src["values"])
            assert mc == case["info"]["max_col"], key
            assert np.array_equal(cols, case["columns"]) and np.array_equal(vals, case["values"]), key
        elif tf == 4:
            d = oracle.coo_to_dense(si["n_row"], si["n_col"], src["row"], src["col"], src["values"])
            assert np.array_equal(d, case["values"]), key
        n += 1
    assert n > 20


def test_oracle_composite_ops(golden):
    """a_axpx_ / AAxpAx / AAxpAxpx (src/cpp/matrix/Matrix.cpp:5-31) over the
    restated Ax, on the reference's own test inputs."""
    import tbsla_gb300 as T

    ops = golden["ops"]
    for n in (10, 30):
        for c in (0, 1, 3, 5, 9):
            for fmt in range(5):
                m = T.FORMATS[fmt]()
                m.fill_cdiag(n, n, c)  # pinned to the reference by test_host_api
                case = m.arrays()
                case["info"] = m.info()
                v = 2 * np.arange(n, dtype=np.float64) + 1
                r = oracle_ax(fmt, case, np.zeros(n), v)
                r[:n] += v
                r2 = oracle_ax(fmt, case, np.zeros(n), r)
                assert np.array_equal(r2, ops[f"a_axpx/{fmt}/{n}/{c}"]), (fmt, n, c)
                buf = oracle_ax(fmt, case, np.full(n, 0.125), v)
                buf += v
                r = oracle_ax(fmt, case, np.full(n, 0.25), buf)
                assert np.array_equal(buf, ops[f"AAxpAx/{fmt}/{n}/{c}/buffer"])
                assert np.array_equal(r, ops[f"AAxpAx/{fmt}/{n}/{c}/r"])
                assert np.array_equal(r + v, ops[f"AAxpAxpx/{fmt}/{n}/{c}/r"])


def test_oracle_col_sums_normalize(golden):
    ops = golden["ops"]
    import tbsla_gb300 as T

    for key in ("cqmat", "cdiag"):
        m = T.MatrixCSR()
        if key == "cqmat":
            m.fill_cqmat(40, 40, 6, 0.4, 2)
        else:
            m.fill_cdiag(40, 40, 3)
        a = m.arrays()
        s = oracle.csr_col_sums(a["rowptr"], a["colidx"], a["values"], 40)
        assert np.array_equal(s, ops[f"colsum/{key}/s"])
        vals = oracle.csr_normalize_cols(a["rowptr"], a["colidx"], a["values"], s)
        end = int(a["rowptr"][-1])
        assert np.array_equal(vals[:end], ops[f"colsum/{key}/values"][:end])


def test_oracle_cfg1_matches_reference(golden):
    """The 10^4-row uniform matrix (this library's generator, seed 0): the
    restated Ax of every format equals the reference's."""
    import tbsla_gb300 as T

    c1 = golden["cfg1"]
    n = 10_000
    csr = T.MatrixCSR()
    csr.fill_uniform_rows(n, 10, 0)
    a = csr.arrays()
    assert a["rowptr"].astype(np.int64).sum() == c1["csr_checksum"][0]
    assert a["colidx"].astype(np.int64).sum() == c1["csr_checksum"][1]
    x = T.fill_uniform(n, 0.0, 1.0, 0)
    assert x.sum() == c1["x_sum"][0]
    rows = np.repeat(np.arange(n, dtype=np.int32), np.diff(a["rowptr"]))
    assert np.array_equal(oracle.csr_ax(a["rowptr"], a["colidx"], a["values"], x), c1["y/2"])
    assert np.array_equal(oracle.coo_ax(n, rows, a["colidx"], a["values"], x), c1["y/0"])
    assert np.array_equal(oracle.scoo_ax(n, 0, 0, rows, a["colidx"], a["values"], x), c1["y/1"])
    mc, cols, vals = oracle.coo_to_ell(n, rows, a["colidx"], a["values"])
    assert np.array_equal(oracle.ell_ax(vals, cols, n, mc, x), c1["y/3"])
    d = T.MatrixDENSE()
    d.fill_dense_uniform(2000, 2000, 0)
    xd = T.fill_uniform(2000, 0.0, 1.0, 0)
    assert np.array_equal(oracle.dense_ax(d.arrays()["values"], 2000, 2000, xd), c1["y_dense"])


def test_oracle_pagerank_and_cg_fixed_points():
    """The restated PageRank keeps sum(x) = 1 and satisfies its fixed-point
    equation; the restated CG reaches the relative tolerance on an SPD matrix."""
    import tbsla_gb300 as T

    g = T.MatrixCSR()
    g.fill_pa_graph(2000, 8.0, 2.1, 200, 0.05, 7)
    a = g.arrays()
    s = oracle.csr_col_sums(a["rowptr"], a["colidx"], a["values"], 2000)
    vals = oracle.csr_normalize_cols(a["rowptr"], a["colidx"], a["values"], s)
    x, it, err = oracle.pagerank(a["rowptr"], a["colidx"], vals, 0.85, 1e-13, 500)
    assert err < 1e-13 and abs(x.sum() - 1) < 1e-12
    d = oracle.dangling_of(a["rowptr"], a["colidx"], 2000).astype(bool)
    ax = oracle.csr_ax(a["rowptr"], a["colidx"], vals, x)
    fp = 0.85 * ax + (0.85 * x[d].sum() + 0.15) / 2000
    assert np.abs(fp - x).sum() < 1e-11
    # FP32-rounded values: column sums are 1 +- 6e-8, yet the iteration
    # still converges (the teleport weight returns the rounding's mass loss)
    v32 = vals.astype(np.float32).astype(np.float64)
    x32, it32, err32 = oracle.pagerank(a["rowptr"], a["colidx"], v32, 0.85, 1e-13, 500)
    assert err32 < 1e-13 and abs(x32.sum() - 1) < 1e-12
    w = oracle.csr_col_sums(a["rowptr"], a["colidx"], v32, 2000)
    ax32 = oracle.csr_ax(a["rowptr"], a["colidx"], v32, x32)
    fp32 = 0.85 * ax32 + (1 - 0.85 * (w * x32).sum()) / 2000
    assert np.abs(fp32 - x32).sum() < 1e-11
    assert np.abs(x32 - x).sum() < 1e-5
    m = T.MatrixCSR()
    m.fill_diffusion7(12, 1.0, 4.0, 5)
    a = m.arrays()
    b = T.fill_uniform(12 ** 3, -1.0, 1.0, 9)
    x, it, rr = oracle.cg(a["rowptr"], a["colidx"], a["values"], b, rel_tol=1e-8)
    assert rr <= 1e-8 and it > 5


def test_mpnn_oracle_gradient_is_the_derivative_of_its_loss():
    """The learned preconditioner's restated loss gradient (oracle/mpnn.py)
    against central finite differences, bfloat16 rounding switched off."""
    import tbsla_gb300 as T
    import oracle.mpnn as M

    m = T.MatrixCSR()
    m.fill_diffusion7(5, 1.0, 3.0, 11)
    a = m.arrays()
    rng = np.random.default_rng(0)
    th = M.unpack(M.init_params(1))
    th["we"] = rng.normal(0, 0.3, M.H)
    th["wd"] = rng.normal(0, 0.3, M.H)
    th["ce"], th["be"] = -0.4, 0.05
    theta = M.pack(th)
    Z = rng.normal(size=(len(a["rowptr"]) - 1, 3))
    keep = M.bf16
    M.bf16 = lambda x: np.asarray(x, np.float64)
    try:
        _, g = M.loss_and_grad(theta, a["rowptr"], a["colidx"], a["values"], Z)
        for k in rng.choice(M.NPARAMS, 30, replace=False):
            tp, tm = theta.copy(), theta.copy()
            tp[k] += 1e-6
            tm[k] -= 1e-6
            fd = (M.loss_and_grad(tp, a["rowptr"], a["colidx"], a["values"], Z)[0]
                  - M.loss_and_grad(tm, a["rowptr"], a["colidx"], a["values"], Z)[0]) / 2e-6
            assert abs(fd - g[k]) <= 1e-5 * max(1.0, abs(fd)), k
    finally:
        M.bf16 = keep


SPMM_FILLS = {"cqmat": lambda m: m.fill_cqmat(40, 40, 6, 0.4, 2), "cdiag": lambda m: m.fill_cdiag(40, 40, 3),
              "random": lambda m: m.fill_random(60, 50, 0.1, 3)}


def test_oracle_spmm_and_softmax_helpers(golden):
    """dense_multiply, get_row_max_abs, apply_exponential, get_row_sums and
    normalize_rows restated, bit for bit against the reference's MatrixCSR
    (tests/golden/spmm.npz)."""
    import tbsla_gb300 as T

    g = golden["spmm"]
    for key, fill in SPMM_FILLS.items():
        m = T.MatrixCSR()
        fill(m)
        a = m.arrays()
        for cols in (1, 5, 33):
            Cm = oracle.csr_dense_multiply(a["rowptr"], a["colidx"], a["values"], g[f"{key}/B{cols}"])
            assert np.array_equal(Cm, g[f"{key}/C{cols}"]), (key, cols)
        mx = oracle.csr_row_max_abs(a["rowptr"], a["values"])
        assert np.array_equal(mx, g[f"{key}/max_abs"]), key
        for tag, use_max, base in (("exp_max", True, -1), ("exp", False, -1), ("pow2_max", True, 2)):
            v = oracle.csr_apply_exponential(a["rowptr"], a["values"], mx if use_max else None, base)
            end = int(a["rowptr"][-1])  # CSR fill_cqmat over-counts nnz; the arrays end at rowptr[n]
            assert np.array_equal(v[:end], g[f"{key}/{tag}"]), (key, tag)
        rs = oracle.csr_row_sums(a["rowptr"], a["values"])
        assert np.array_equal(rs, g[f"{key}/row_sums"]), key
        end = int(a["rowptr"][-1])
        rz = rs.copy()
        rz[::3] = 0
        for tag, sv in (("norm_rows", rs), ("norm_rows_zero", rz)):
            v = oracle.csr_normalize_rows(a["rowptr"], a["values"], sv)
            assert np.array_equal(v[:end], g[f"{key}/{tag}"][:end]), (key, tag)
