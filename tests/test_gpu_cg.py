"""CG parity (src/mpi/matrix/CG.cpp:32-73, restated in the oracle with the
argument order fixed and a relative stop test): GPU CG / Jacobi-PCG, single
and batched over systems of uneven size, in FP64 and in FP32 / BF16 value
storage with FP64 residual replacement, must reach the same 1e-8 relative
residual as the oracle, verified in FP64 on the host."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu
TOL = 1e-8


def diffusion(T, n, seed):
    m = T.MatrixCSR()
    m.fill_diffusion7(n, 1.0, 8.0, seed)
    return m


def true_rel_residual(m, x, b):
    a = m.arrays()
    ax = oracle.csr_ax(a["rowptr"], a["colidx"], a["values"], x)
    return np.linalg.norm(b - ax) / np.linalg.norm(b)


@pytest.mark.parametrize("precond", [0, 1])
def test_cg_single_matches_oracle(gpu, precond):
    T = gpu
    m = diffusion(T, 16, 3)
    n = 16 ** 3
    b = T.fill_uniform(n, -1.0, 1.0, 3)
    x, it, rr, ok = m.CG(b, max_iterations=5000, rel_tol=TOL, precond=precond)
    assert ok and rr <= TOL
    assert true_rel_residual(m, x, b) <= TOL
    a = m.arrays()
    dinv = None
    if precond:
        d = np.zeros(n)
        rows = np.repeat(np.arange(n), np.diff(a["rowptr"]))
        diag = rows == a["colidx"]
        d[rows[diag]] = a["values"][diag]
        dinv = 1.0 / d
    xo, ito, rro = oracle.cg(a["rowptr"], a["colidx"], a["values"], b, rel_tol=TOL, diag_inv=dinv)
    assert rro <= TOL
    # same algorithm in FP64: the iteration counts agree closely
    assert abs(it - ito) <= max(3, 0.05 * ito), (it, ito)
    assert np.linalg.norm(x - xo) / np.linalg.norm(xo) < 1e-6


@pytest.mark.parametrize("prec", ["f32"])
def test_cg_narrow_storage_reaches_fp64_residual(gpu, prec):
    """FP32 SpMV inside the iteration, FP64 true residual every 50
    iterations and at convergence: the FP64-verified 1e-8 is still met."""
    T = gpu
    m = diffusion(T, 20, 5)
    m.set_precision(T.F32)
    n = 20 ** 3
    b = T.fill_uniform(n, -1.0, 1.0, 5)
    x, it, rr, ok = m.CG(b, max_iterations=20000, rel_tol=TOL, precond=1, refresh=50)
    assert ok and rr <= TOL
    m.set_precision(T.F64)
    assert true_rel_residual(m, x, b) <= TOL


def test_batched_uneven_sizes(gpu):
    T = gpu
    sizes = [8, 12, 16, 6, 20, 10, 14]
    systems = [diffusion(T, s, 100 + i) for i, s in enumerate(sizes)]
    for precision in (T.F64, T.F32):
        batch = T.Batch(systems, precision)
        off = batch.offsets
        rhs = np.concatenate([T.fill_uniform(s ** 3, -1.0, 1.0, 200 + i) for i, s in enumerate(sizes)])
        for precond in (0, 1):
            x, its, rr, ok = batch.cg(rhs, max_iterations=5000, rel_tol=TOL, precond=precond, graph_iters=7)
            assert ok and (rr <= TOL).all(), (precision, precond, its, rr)
            for k, m in enumerate(systems):
                xs, bs = x[off[k]:off[k + 1]], rhs[off[k]:off[k + 1]]
                assert true_rel_residual(m, xs, bs) <= TOL, (k, precision, precond)
            # bigger systems need more iterations
            assert its[sizes.index(20)] > its[sizes.index(6)]


def test_iteration_limit_is_reported(gpu):
    T = gpu
    m = diffusion(T, 16, 7)
    b = T.fill_uniform(16 ** 3, -1.0, 1.0, 7)
    x, it, rr, ok = m.CG(b, max_iterations=5, rel_tol=TOL)
    assert not ok and it == 5 and rr > TOL


def test_start_vector_is_used(gpu):
    """x0 = the solution: converged before the first iteration."""
    T = gpu
    m = diffusion(T, 10, 9)
    b = T.fill_uniform(1000, -1.0, 1.0, 9)
    x, it, rr, ok = m.CG(b, rel_tol=1e-12)
    x2, it2, rr2, ok2 = m.CG(b, x=x.copy(), rel_tol=1e-6)
    assert ok2 and it2 == 0


def test_persistent_engine_runs_the_whole_solve(gpu):
    """Stencil systems take the persistent engine: one cooperative launch per
    solve, replayed from a CUDA graph; results verified in FP64 on the host
    for FP64 storage (FP64 iteration) and FP32 storage (FP32 iteration with
    FP64 refinement), plain and Jacobi."""
    T = gpu
    sizes = [9, 13, 6, 17]
    systems = [diffusion(T, s, 300 + i) for i, s in enumerate(sizes)]
    rhs = np.concatenate([T.fill_uniform(s ** 3, -1.0, 1.0, 400 + i) for i, s in enumerate(sizes)])
    for precision in (T.F64, T.F32):
        batch = T.Batch(systems, precision)
        off = batch.offsets
        for precond in (0, 1):
            for rep in range(2):  # the second solve replays the captured graph
                x, its, rr, ok = batch.cg(rhs, max_iterations=4000, rel_tol=TOL, precond=precond, refresh=50)
                assert ok and (rr <= TOL).all(), (precision, precond, its, rr)
                eng = batch.engine()
                assert eng["persistent"], eng
                for k, m in enumerate(systems):
                    xs, bs = x[off[k]:off[k + 1]], rhs[off[k]:off[k + 1]]
                    assert true_rel_residual(m, xs, bs) <= TOL, (k, precision, precond)
                fb, used = batch.fallbacks()
                assert (fb == 0).all() and (used == precond).all()


def test_general_pattern_takes_multi_launch_engine(gpu):
    """A matrix whose entries lie on more than 8 diagonals (here a random
    symmetric pattern made diagonally dominant) keeps the multi-launch
    engine and still reaches the FP64-verified tolerance."""
    T = gpu
    n = 3000
    rng = np.random.default_rng(3)
    rows = rng.integers(0, n, 12000)
    cols = rng.integers(0, n, 12000)
    vals = rng.uniform(-1, 0, 12000)
    import scipy.sparse as sp

    A = sp.coo_matrix((vals, (rows, cols)), shape=(n, n)).tocsr()
    A = A + A.T
    A = A + sp.diags(np.asarray(abs(A).sum(axis=1)).ravel() + 1.0)
    A = A.tocsr()
    A.sort_indices()
    m = T.MatrixCSR.from_arrays(n, n, A.indptr.astype(np.int32), A.indices.astype(np.int32), A.data)
    b = T.fill_uniform(n, -1.0, 1.0, 11)
    batch = T.Batch([m], T.F64)
    x, its, rr, ok = batch.cg(b, max_iterations=2000, rel_tol=TOL, precond=1)
    assert ok and rr[0] <= TOL
    assert not batch.engine()["persistent"]
    assert true_rel_residual(m, x, b) <= TOL


def test_bounded_wait_returns_timeout_status(gpu):
    """Every grid-wide wait of the persistent kernel is bounded.  With a
    limit of 0 ns the first wait runs out at once: the kernel returns, the
    call reports TBSLA_ERR_TIMEOUT (nothing hangs), and the next solve with
    the default limit on the same batch succeeds."""
    T = gpu
    systems = [diffusion(T, 10, 500 + i) for i in range(3)]
    rhs = np.concatenate([T.fill_uniform(1000, -1.0, 1.0, 600 + i) for i in range(3)])
    batch = T.Batch(systems, T.F32)
    batch.set_wait_limit(0)
    with pytest.raises(T.TbslaError) as e:
        batch.cg(rhs, max_iterations=2000, rel_tol=TOL, precond=1)
    assert e.value.status == T._lib.ERR_TIMEOUT
    batch.set_wait_limit(2_000_000_000)
    x, its, rr, ok = batch.cg(rhs, max_iterations=2000, rel_tol=TOL, precond=1)
    assert ok and (rr <= TOL).all()
    assert batch.engine()["persistent"]


def test_vector_rows_match_scalar_rows(gpu):
    """With every system size a multiple of 4 the FP32 iteration takes 4 rows
    per thread (16-byte loads); each row's arithmetic is that of the
    one-row-per-thread loops, so both forms give the same iterate up to the
    order of the FP64 atomic dot products: iteration counts within one,
    solutions within the tolerance, every system FP64-verified."""
    T = gpu
    sizes = [8, 12, 16, 10]
    systems = [diffusion(T, s, 700 + i) for i, s in enumerate(sizes)]
    rhs = np.concatenate([T.fill_uniform(s ** 3, -1.0, 1.0, 710 + i) for i, s in enumerate(sizes)])
    batch = T.Batch(systems, T.F32)
    off = batch.offsets
    for precond in (0, 1):
        out = []
        for rows in (4, 1):
            batch.set_rows_per_thread(rows)
            x, its, rr, ok = batch.cg(rhs, max_iterations=4000, rel_tol=TOL, precond=precond, refresh=50)
            assert ok and (rr <= TOL).all()
            for k, m in enumerate(systems):
                assert true_rel_residual(m, x[off[k]:off[k + 1]], rhs[off[k]:off[k + 1]]) <= TOL
            out.append(its)
        assert np.abs(out[0] - out[1]).max() <= 1, out


def test_grid_size_does_not_change_the_solve(gpu):
    """The persistent engine hands out warp units grid-stride, so a launch
    of 2 CTAs per SM does the same row arithmetic as the default 3; only the
    order of the FP64 atomic dot products differs, which over a thousand
    FP32 iterations of plain CG moves the stop by a few: iteration counts
    within 1% (at least one), every system FP64-verified, for plain and
    Jacobi."""
    T = gpu
    sizes = [16, 20, 12, 24, 8]
    systems = [diffusion(T, s, 720 + i) for i, s in enumerate(sizes)]
    rhs = np.concatenate([T.fill_uniform(s ** 3, -1.0, 1.0, 730 + i) for i, s in enumerate(sizes)])
    batch = T.Batch(systems, T.F32)
    off = batch.offsets
    for precond in (0, 1):
        out = []
        for ctas in (0, 2):
            batch.set_ctas_per_sm(ctas)
            assert batch.tuning()["ctas_per_sm"] == ctas
            x, its, rr, ok = batch.cg(rhs, max_iterations=4000, rel_tol=TOL, precond=precond, refresh=50)
            assert ok and (rr <= TOL).all()
            for k, m in enumerate(systems):
                assert true_rel_residual(m, x[off[k]:off[k + 1]], rhs[off[k]:off[k + 1]]) <= TOL
            out.append(its)
        assert (np.abs(out[0] - out[1]) <= np.maximum(1, out[0] // 100)).all(), out


def test_autotune_batch_cg_and_cache(gpu, tmp_path):
    """The autotuner times the persistent engine's settings on the batch's
    own solve, keeps the fastest, caches it, and a second call applies the
    cached settings without timing; the tuned batch still solves to the
    FP64-verified tolerance."""
    from tbsla_gb300 import autotune as A

    T = gpu
    sizes = [12, 16, 8]
    systems = [diffusion(T, s, 900 + i) for i, s in enumerate(sizes)]
    rhs = np.concatenate([T.fill_uniform(s ** 3, -1.0, 1.0, 910 + i) for i, s in enumerate(sizes)])
    batch = T.Batch(systems, T.F32)
    path = str(tmp_path / "tune.json")
    r = A.tune_batch_cg(batch, rhs, T.F32, precond=1, reps=1, path=path)
    assert not r["cached"] and len(r["trials"]) == 4
    assert batch.tuning() == r["settings"]
    r2 = A.tune_batch_cg(T.Batch(systems, T.F32), rhs, T.F32, precond=1, path=path)
    assert r2["cached"] and r2["settings"] == r["settings"]
    x, its, rr, ok = batch.cg(rhs, max_iterations=4000, rel_tol=TOL, precond=1)
    assert ok and (rr <= TOL).all()
    off = batch.offsets
    for k, m in enumerate(systems):
        assert true_rel_residual(m, x[off[k]:off[k + 1]], rhs[off[k]:off[k + 1]]) <= TOL


def test_seven_point_form_matches_general_form(gpu):
    """Batches of 7-point stencils whose line and plane sizes are multiples
    of 4 run the persistent kernel's seven-point form (neighbour alignments
    fixed when compiled); it does the general form's arithmetic in the same
    order, so the two agree up to the FP64 atomic dot products' order:
    iterations within 1% (at least one), every system FP64-verified, for
    plain, Jacobi and the factored preconditioner (an untrained network's
    factor on tril(A), from a network whose head makes every off-diagonal
    slot of the factor non-zero).  A batch with a system of
    line size 10 keeps the general form."""
    T = gpu
    sizes = [8, 12, 16, 20]
    systems = [diffusion(T, s, 740 + i) for i, s in enumerate(sizes)]
    rhs = np.concatenate([T.fill_uniform(s ** 3, -1.0, 1.0, 750 + i) for i, s in enumerate(sizes)])
    batch = T.Batch(systems, T.F32)
    net = _neumann_net(T, 3)
    batch.factor_mpnn(net, T.BF16)
    _, lv = batch.factor_dia()
    assert np.count_nonzero(lv[1]) > lv.shape[1] // 2  # the -1 slot of L is populated
    off = batch.offsets
    for precond in (0, 1, 2):
        out = []
        for on in (True, False):
            batch.set_seven_point(on)
            x, its, rr, ok = batch.cg(rhs, max_iterations=4000, rel_tol=TOL, precond=precond, refresh=50)
            assert ok and (rr <= TOL).all()
            assert batch.engine()["seven_point"] == on, (precond, on)
            for k, m in enumerate(systems):
                assert true_rel_residual(m, x[off[k]:off[k + 1]], rhs[off[k]:off[k + 1]]) <= TOL
            out.append(its)
        assert (np.abs(out[0] - out[1]) <= np.maximum(1, out[0] // 100)).all(), (precond, out)
    mixed = T.Batch([diffusion(T, 10, 760), diffusion(T, 8, 761)], T.F32)
    rhs2 = np.concatenate([T.fill_uniform(1000, -1.0, 1.0, 762), T.fill_uniform(512, -1.0, 1.0, 763)])
    x, its, rr, ok = mixed.cg(rhs2, max_iterations=4000, rel_tol=TOL, precond=1)
    assert ok and not mixed.engine()["seven_point"] and mixed.engine()["persistent"]


def _neumann_net(T, seed):
    """A network whose head gives L = D^-1/2 (I - E_lower / 2) on the
    pattern of tril(A) (E the scaled off-diagonal entries a_ij s_i s_j):
    a first-order approximate inverse factor, SPD as M^-1 = L L^T, with
    every off-diagonal slot of L populated."""
    import oracle.mpnn as M

    net = T.MPNN(seed)
    p = M.unpack(net.params().astype(np.float64))
    p["ce"] = -0.5
    net.set_params(M.pack(p).astype(np.float32))
    return net


def test_seven_point_form_needs_unit_neighbours(gpu):
    """With a factor, the seven-point form takes L's delta-0 and delta--1
    windows from the rows' own vectors, so it needs those exact deltas, not
    only their alignment classes: a system on the diagonals -64, -8, -5, 0,
    +5, +8, +64 (the classes of a 7-point stencil of line size 8; L on
    deltas 0, -5, -8, -64) runs the general form with a factor whose
    off-diagonal slots are populated; Jacobi, which reads every shift at
    run time, may take either form.  Both reach the FP64-verified
    tolerance."""
    T = gpu
    n = 512
    offs = (-64, -8, -5, 0, 5, 8, 64)
    rows, cols, vals = [], [], []
    for i in range(n):
        for d in offs:
            j = i + d
            if 0 <= j < n:
                rows.append(i)
                cols.append(j)
                vals.append(6.5 if d == 0 else -1.0)
    rowptr = np.zeros(n + 1, np.int64)
    np.add.at(rowptr, np.asarray(rows) + 1, 1)
    rowptr = np.cumsum(rowptr)
    a5 = T.MatrixCSR.from_arrays(n, n, rowptr, np.asarray(cols), np.asarray(vals))
    systems = [a5, diffusion(T, 8, 770)]
    rhs = np.concatenate([T.fill_uniform(n, -1.0, 1.0, 771), T.fill_uniform(512, -1.0, 1.0, 772)])
    batch = T.Batch(systems, T.F32)
    batch.factor_mpnn(_neumann_net(T, 4), T.BF16)
    off = batch.offsets
    for precond in (1, 2):
        x, its, rr, ok = batch.cg(rhs, max_iterations=4000, rel_tol=TOL, precond=precond, refresh=50)
        assert ok and (rr <= TOL).all()
        eng = batch.engine()
        assert eng["persistent"] and (precond == 1 or not eng["seven_point"]), (precond, eng)
        for k, m in enumerate(systems):
            assert true_rel_residual(m, x[off[k]:off[k + 1]], rhs[off[k]:off[k + 1]]) <= TOL
