"""Parity at the full workload sizes, through the same C-ABI calls as the
smaller tests:

* SpMV on the n = 2^24 power-law matrix (Zipf(2) rows, mean 16, at most
  4096 entries, 30% within +-1024 of the diagonal, seed 1; 268.7 M
  entries): every row of y within 1e-13 of the oracle (normalised by
  sum_j |a_ij x_j|) with FP64, FP32 and BF16 value storage, in CSR with the
  automatic kernel choice (sliced ELL, two column blocks, the last in two
  row parts) and in COO; repeated calls and the device-pointer entry point
  give the same vector bit for bit.
* PageRank on the 2^22-node preferential-attachment graph (67.2 M edges,
  5% dangling, FP32 values, seed 2): within 1e-10 in L1 of the oracle after
  the same number of iterations; the 32 personalised vectors, two against
  the oracle's solve and all 32 through the fixed-point residual
  |F(x) - x|_1 of one oracle iteration F.
* The 32768 x 16384 DENSE GEMV with FP64, FP32 and BF16 values.
* Batched CG on the 64 diffusion systems of sizes 16, 24, ..., 96 (17.1 M
  unknowns, FP32 values, FP64 refresh every 50 iterations): every system's
  true residual, recomputed by the oracle in FP64, is at most 1e-8.
"""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu
TOL = 1e-13


@pytest.fixture(scope="module")
def big(gpu):
    T = gpu
    n = 1 << 24
    m = T.MatrixCSR()
    m.fill_powerlaw(n, 16.0, 2.0, 4096, 0.3, 1024, 1)
    a = m.arrays()
    x = T.fill_uniform(n, 0.0, 1.0, 11)
    ref = oracle.csr_ax(a["rowptr"], a["colidx"], a["values"], x, threads=True)
    scale = oracle.csr_absrow(a["rowptr"], a["colidx"], a["values"], x)
    return {"m": m, "a": a, "x": x, "ref": ref, "scale": scale, "n": n}


@pytest.mark.parametrize("prec", ["f64", "f32", "bf16"])
def test_spmv_powerlaw_full_size(gpu, big, prec):
    T = gpu
    m, a, x, n = big["m"], big["a"], big["x"], big["n"]
    assert int(a["rowptr"][-1]) > 268_000_000
    m.set_precision({"f64": T.F64, "f32": T.F32, "bf16": T.BF16}[prec])
    y = m.spmv(x)
    if prec == "f64":
        ref, scale = big["ref"], big["scale"]
    else:
        if prec == "f32":
            v32 = a["values"].astype(np.float32)
            ref = oracle.csr_ax_f32(a["rowptr"], a["colidx"], v32, x)
            rv = v32.astype(np.float64)
            del v32
        else:
            rv = oracle.bf16_round(a["values"])
            ref = oracle.csr_ax(a["rowptr"], a["colidx"], rv, x, threads=True)
        scale = oracle.csr_absrow(a["rowptr"], a["colidx"], rv, x)
        del rv
        # against the FP64 matrix: the error of the value rounding alone
        err64 = oracle.rel_err_normalized(y, big["ref"], big["scale"])
        assert err64 <= (2.0 ** -24 if prec == "f32" else 2.0 ** -8) * 1.01, err64
    assert oracle.rel_err_normalized(y, ref, scale) <= TOL
    # the host entry point again (x copied under the first column block's
    # launch, y back by row parts): the same vector
    y2 = np.full(n, 3.0)
    m.Ax(y2, x)
    assert np.array_equal(y2, y)
    if prec == "f64":
        import torch

        xt = torch.from_numpy(x).cuda()
        yt = torch.full((n,), 9.0, dtype=torch.float64, device="cuda")
        m.Ax_device(yt, xt)
        torch.cuda.synchronize()
        assert np.array_equal(yt.cpu().numpy(), y)
        del xt, yt


def test_coo_full_size(gpu, big):
    """The same 268.7 M entries in COO (segmented reduction in warp chunks
    of 256 triplets; rows of up to 4096 entries span several chunks)."""
    T = gpu
    a, x, n = big["a"], big["x"], big["n"]
    rows = np.repeat(np.arange(n, dtype=np.int32), np.diff(a["rowptr"]))
    coo = T.MatrixCOO.from_arrays(n, n, rows, a["colidx"], a["values"])
    del rows
    y = coo.spmv(x)
    assert oracle.rel_err_normalized(y, big["ref"], big["scale"]) <= TOL


@pytest.mark.parametrize("prec", ["f64", "f32", "bf16"])
def test_dense_gemv_full_size(gpu, prec):
    """The 32768 x 16384 GEMV of the formats workload (4.3 GB of FP64
    values): double-float arithmetic on the FP32 pipes for every precision
    (an FP64 value split on load into two floats, about 2^-48), two launches
    (the split of x, the GEMV), every row within 1e-13 of the oracle on the
    same rounded values."""
    T = gpu
    nr, nc = 32768, 16384
    d = T.MatrixDENSE()
    d.fill_dense_uniform(nr, nc, 0)
    d.set_precision({"f64": T.F64, "f32": T.F32, "bf16": T.BF16}[prec])
    vals = d.arrays()["values"]
    if prec == "f32":
        vals = vals.astype(np.float32).astype(np.float64)
    elif prec == "bf16":
        vals = oracle.bf16_round(vals)
    x = T.fill_uniform(nc, 0.0, 1.0, 0)
    y = d.spmv(x)
    assert d.kernel_launches() == 2
    ref = oracle.dense_ax(vals, nr, nc, x, threads=True)
    scale = oracle.dense_ax(np.abs(vals), nr, nc, x, threads=True)  # x >= 0: sum_j |a_ij x_j|
    assert oracle.rel_err_normalized(y, ref, scale) <= TOL


def pa_graph(T):
    n = 1 << 22
    g = T.MatrixCSR()
    g.fill_pa_graph(n, 16.0, 2.1, 4096, 0.05, 2)
    g.make_stochastic(np.zeros(n))
    g.set_precision(T.F32)
    a = g.arrays()
    vals = a["values"].astype(np.float32).astype(np.float64)
    return g, a, vals, n


def test_pagerank_pa_graph_full_size(gpu):
    T = gpu
    g, a, vals, n = pa_graph(T)
    assert int(a["rowptr"][-1]) > 67_000_000
    x, it, err, ok = g.page_rank(0.85, 1e-10, 1000)
    assert ok and err < 1e-10 and it > 5
    xr, itr, _ = oracle.pagerank(a["rowptr"], a["colidx"], vals, 0.85, 1e-10, it, stop_early=False)
    assert itr == it
    assert np.abs(x - xr).sum() <= 1e-10
    assert abs(x.sum() - 1) < 1e-12

    nvec = 32
    rng = np.random.default_rng(2)
    tele = np.zeros((n, nvec))
    for k in range(nvec):
        tele[rng.choice(n, 100, replace=False), k] = 1.0 / 100
    X, itb, okb = g.page_rank_batched(tele, 0.85, 1e-10, 1000)
    assert okb and itb > 5
    for k in (0, 17):
        xr, _, _ = oracle.pagerank(a["rowptr"], a["colidx"], vals, 0.85, 1e-10, itb, stop_early=False,
                                   teleport=np.ascontiguousarray(tele[:, k]))
        assert np.abs(X[:, k] - xr).sum() <= 1e-10, k
    # every vector: one power step F(x) = b A x / S + (1 - b w.x / S) t, with
    # S = sum x and w the column sums of the stored values, moves it by at
    # most the stop tolerance
    w = oracle.csr_col_sums(a["rowptr"], a["colidx"], vals, n)
    for k in range(nvec):
        xk = np.ascontiguousarray(X[:, k])
        S = xk.sum()
        assert abs(S - 1) < 1e-12, k
        ax = oracle.csr_ax(a["rowptr"], a["colidx"], vals, xk, threads=True)
        fx = 0.85 * ax / S + (1.0 - 0.85 * float(w @ xk) / S) * tele[:, k]
        assert np.abs(fx - xk).sum() <= 1e-10, k


def test_batched_cg_diffusion_full_size(gpu):
    T = gpu
    sizes = [16 + 8 * (i % 11) for i in range(64)]
    systems = []
    for i, sz in enumerate(sizes):
        m = T.MatrixCSR()
        m.fill_diffusion7(sz, 1.0, 8.0, 3000 + i)
        systems.append(m)
    rhs = np.concatenate([T.fill_uniform(sz ** 3, -1.0, 1.0, 4000 + i) for i, sz in enumerate(sizes)])
    assert rhs.size > 17_000_000
    bt = T.Batch(systems, T.F32)
    off = bt.offsets
    for precond in (0, 1):
        x, its, rr, ok = bt.cg(rhs, max_iterations=20000, rel_tol=1e-8, precond=precond, refresh=50,
                               graph_iters=10)
        assert ok and (rr <= 1e-8).all(), (precond, rr.max())
        for k, m in enumerate(systems):
            ak = m.arrays()
            xs, bs = x[off[k]:off[k + 1]], rhs[off[k]:off[k + 1]]
            ax = oracle.csr_ax(ak["rowptr"], ak["colidx"], ak["values"], xs)
            assert np.linalg.norm(bs - ax) / np.linalg.norm(bs) <= 1e-8, (precond, k)
        assert its[sizes.index(96)] > its[sizes.index(16)]
