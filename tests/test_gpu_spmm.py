"""CSR dense_multiply (SpMM) and the sparse-softmax helpers on the GPU
against the reference's recordings (tests/golden/spmm.npz) and the oracle:
SpMM within the FP64 bar (one fused multiply-add per product, the reference
rounds the product first), row maxima, row sums and row normalisation
exact, exponentials within 2 ulp of the host libm."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

FILLS = {"cqmat": lambda m: m.fill_cqmat(40, 40, 6, 0.4, 2), "cdiag": lambda m: m.fill_cdiag(40, 40, 3),
         "random": lambda m: m.fill_random(60, 50, 0.1, 3)}


def spmm_scale(a, B):
    """|A| |B|: the per-entry scale of the SpMM rounding bound."""
    return oracle.csr_dense_multiply(a["rowptr"], a["colidx"], np.abs(a["values"]), np.abs(B))


def test_against_reference_recordings(gpu, golden):
    T = gpu
    g = golden["spmm"]
    for key, fill in FILLS.items():
        m = T.MatrixCSR()
        fill(m)
        a = m.arrays()
        for cols in (1, 5, 33):
            B = g[f"{key}/B{cols}"]
            Cm = m.dense_multiply(B)
            ref = g[f"{key}/C{cols}"]
            scale = spmm_scale(a, B)
            assert np.all(np.abs(Cm - ref) <= 1e-13 * scale + 1e-300), (key, cols)
        mx = m.get_row_max_abs()
        assert np.array_equal(mx, g[f"{key}/max_abs"]), key
        end = int(a["rowptr"][-1])
        for tag, use_max, base in (("exp_max", True, -1), ("exp", False, -1), ("pow2_max", True, 2)):
            e = T.MatrixCSR()
            fill(e)
            e.apply_exponential(mx if use_max else None, base)
            v = e.arrays()["values"][:end]
            ref = g[f"{key}/{tag}"]
            assert np.allclose(v, ref, rtol=5e-16, atol=0), (key, tag)
        # row sums in entry order and the division: bit for bit, including
        # the rows whose sum is given as 0 (set to 0)
        rs = m.get_row_sums()
        assert np.array_equal(rs, g[f"{key}/row_sums"]), key
        rz = rs.copy()
        rz[::3] = 0
        for tag, sv in (("norm_rows", rs), ("norm_rows_zero", rz)):
            e = T.MatrixCSR()
            fill(e)
            e.normalize_rows(sv)
            assert np.array_equal(e.arrays()["values"][:end], g[f"{key}/{tag}"][:end]), (key, tag)
            x = np.linspace(0.5, 1.5, e.info()["n_col"])
            ea = e.arrays()
            assert np.allclose(e.spmv(x), oracle.csr_ax(ea["rowptr"], ea["colidx"], ea["values"], x),
                               rtol=1e-13, atol=1e-300), (key, tag)  # device copy refreshed


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_spmm_power_law(gpu, prec):
    T = gpu
    n = 1 << 15
    m = T.MatrixCSR()
    m.fill_powerlaw(n, seed=12, max_len=1024)
    a = m.arrays()
    vals = a["values"]
    if prec == "f32":
        m.set_precision(T.F32)
        vals = vals.astype(np.float32).astype(np.float64)
    rng = np.random.default_rng(3)
    for cols in (1, 7, 40):
        B = rng.uniform(-1, 1, (n, cols))
        Cm = m.dense_multiply(B)
        ref = oracle.csr_dense_multiply(a["rowptr"], a["colidx"], vals, B)
        scale = oracle.csr_dense_multiply(a["rowptr"], a["colidx"], np.abs(vals), np.abs(B))
        assert np.all(np.abs(Cm - ref) <= 1e-13 * scale + 1e-300), cols
    # softmax numerator: exp(a - rowmax) keeps the device copy in step
    mx = m.get_row_max_abs()
    m.apply_exponential(mx)
    x = T.fill_uniform(n, 0.0, 1.0, 4)
    v = oracle.csr_apply_exponential(a["rowptr"], a["values"], oracle.csr_row_max_abs(a["rowptr"], a["values"]))
    assert np.allclose(m.arrays()["values"], v, rtol=5e-16, atol=0)
    if prec == "f64":
        y = m.spmv(x)
        ref = oracle.csr_ax(a["rowptr"], a["colidx"], v, x)
        scale = oracle.csr_absrow(a["rowptr"], a["colidx"], v, x)
        assert oracle.rel_err_normalized(y, ref, scale) <= 1e-13
