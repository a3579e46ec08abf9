"""Learned preconditioner (tbsla_mpnn_*): the GPU forward / backward match
the oracle's float64 restatement (oracle/mpnn.py), the untrained factor is
Jacobi, PCG with M^-1 = L L^T reaches the FP64-verified 1e-8 residual, and
a short training run lowers the iteration count below Jacobi-PCG on
held-out systems."""
import numpy as np
import pytest

import oracle
import oracle.mpnn as M

pytestmark = pytest.mark.gpu


def diffusion(T, n, seed):
    m = T.MatrixCSR()
    m.fill_diffusion7(n, 1.0, 4.0, seed)
    return m


def test_loss_and_gradient_match_the_oracle(gpu):
    T = gpu
    A = diffusion(T, 9, 21)
    a = A.arrays()
    n = len(a["rowptr"]) - 1
    rng = np.random.default_rng(5)
    th = M.unpack(M.init_params(3))
    th["we"] = rng.normal(0, 0.2, M.H)
    th["wd"] = rng.normal(0, 0.2, M.H)
    th["ce"], th["be"] = -0.3, 0.02
    theta = M.bf16(M.pack(th)).astype(np.float32)  # exactly representable: no rounding on either side
    Z = rng.normal(size=(n, 4))
    net = T.MPNN(0)
    net.set_params(theta)
    loss, g = net.loss_grad(A, Z)
    loss_ref, g_ref = M.loss_and_grad(theta.astype(np.float64), a["rowptr"], a["colidx"], a["values"], Z)
    assert abs(loss - loss_ref) <= 1e-4 * loss_ref
    # FP32 kernels against float64: relative error of the whole gradient
    # and of each parameter block
    assert np.linalg.norm(g - g_ref) <= 1e-3 * np.linalg.norm(g_ref)
    o = 0
    for name, shape in M.PARAM_LAYOUT:
        k = int(np.prod(shape)) if shape else 1
        ref = g_ref[o:o + k]
        assert np.linalg.norm(g[o:o + k] - ref) <= 2e-3 * max(np.linalg.norm(ref), 1e-6), name
        o += k
    # the L values of the forward pass
    Lm = net.factor(A)
    la = Lm.arrays()
    r, c, v = M.factor(theta.astype(np.float64), a["rowptr"], a["colidx"], a["values"])
    dense = np.zeros((n, n))
    dense[r, c] = v
    got = np.zeros((n, n))
    rows = np.repeat(np.arange(n), np.diff(la["rowptr"]))
    got[rows, la["colidx"]] = la["values"]
    assert np.abs(got - dense).max() <= 1e-5 * np.abs(dense).max()


def test_untrained_factor_is_jacobi(gpu):
    T = gpu
    A = diffusion(T, 8, 2)
    a = A.arrays()
    n = len(a["rowptr"]) - 1
    L = T.MPNN(1).factor(A).arrays()
    rows = np.repeat(np.arange(n), np.diff(L["rowptr"]))
    diag = rows == L["colidx"]
    assert diag.sum() == n and np.all(L["colidx"] <= rows)
    assert np.all(L["values"][~diag] == 0)
    d = np.zeros(n)
    ar = np.repeat(np.arange(n), np.diff(a["rowptr"]))
    m = ar == a["colidx"]
    d[ar[m]] = a["values"][m]
    ratio = L["values"][diag] / (1 / np.sqrt(d[rows[diag]]))
    assert np.allclose(ratio, ratio[0], rtol=1e-6) and abs(ratio[0] - 1) < 1e-2


def _solve(T, systems, factors, precond, factor_prec=None):
    bt = T.Batch(systems, T.F32)
    if factors is not None:
        bt.set_factors(factors, T.F32 if factor_prec is None else factor_prec)
    rhs = np.concatenate([T.fill_uniform(len(s.arrays()["rowptr"]) - 1, -1.0, 1.0, 70 + i)
                          for i, s in enumerate(systems)])
    x, its, rr, ok = bt.cg(rhs, max_iterations=5000, rel_tol=1e-8, precond=precond, refresh=50, graph_iters=10)
    # FP64-verified on the host
    o = 0
    for s in systems:
        a = s.arrays()
        k = len(a["rowptr"]) - 1
        res = rhs[o:o + k] - oracle.csr_ax(a["rowptr"], a["colidx"], a["values"], x[o:o + k])
        assert np.linalg.norm(res) <= 1.0001e-8 * np.linalg.norm(rhs[o:o + k])
        o += k
    assert ok
    return its


def test_factored_pcg_converges_and_training_beats_jacobi(gpu):
    T = gpu
    net = T.MPNN(7)
    train = [diffusion(T, 10 + (i % 7), 1000 + i) for i in range(24)]
    losses = []
    for step in range(240):
        losses.append(net.train_step(train[step % len(train)], probes=8, seed=step, lr=3e-3))
    assert np.mean(losses[-24:]) < 0.8 * np.mean(losses[:24])
    held = [diffusion(T, 14, 9000 + i) for i in range(4)]
    its_j = _solve(T, held, None, 1)
    factors = [net.factor(A) for A in held]
    its_l = _solve(T, held, factors, 2)
    assert its_l.mean() < its_j.mean(), (its_l, its_j)
    # bfloat16 factor storage: still SPD, still converges to the FP64 bar
    its_b = _solve(T, held, factors, 2, T.BF16)
    assert its_b.mean() < its_j.mean(), (its_b, its_j)


def test_factor_layouts_agree(gpu):
    """Factors on at most 8 diagonals per system run in the persistent engine
    (DIA form, slot 0 the diagonal), any other factor in the multi-launch
    engine (ELL or CSR copies).  The same factor padded with explicit zeros
    at the columns i - z, 0 < z <= pad, stays a DIA factor for pad 2 (five
    diagonals: the extra zero slot leaves every FP32 sum unchanged, so the
    iteration counts agree up to the one that the order of the FP64 atomic
    dot products can move) and becomes a CSR factor of the
    multi-launch engine for pad 7 (eleven diagonals).  Every solve reaches
    the FP64-verified 1e-8 residual; the two engines' counts stay close."""
    T = gpu
    systems = [diffusion(T, 11 + i, 60 + i) for i in range(3)]
    layouts = {0: [], 2: [], 7: []}
    for A in systems:
        a = A.arrays()
        n = len(a["rowptr"]) - 1
        for pad, out in layouts.items():
            rp, ci, va = [0], [], []
            for i in range(n):
                cols = a["colidx"][a["rowptr"][i]:a["rowptr"][i + 1]]
                vals = a["values"][a["rowptr"][i]:a["rowptr"][i + 1]]
                d = vals[cols == i][0]
                row = {int(c): (-0.1 * v / d if c != i else 1 / np.sqrt(d)) for c, v in zip(cols, vals) if c <= i}
                for c in range(max(0, i - pad), i):
                    row.setdefault(c, 0.0)
                for c in sorted(row):
                    ci.append(c)
                    va.append(row[c])
                rp.append(len(ci))
            out.append(T.MatrixCSR.from_arrays(n, n, np.array(rp, np.int32), np.array(ci, np.int32), np.array(va)))
    its, engines = [], []
    for f in layouts.values():
        bt_its = _solve(T, systems, f, 2, T.F32)
        its.append(np.asarray(bt_its))
    # identical FP32 sums; the FP64 atomic dot products may move one count
    assert np.abs(its[0] - its[1]).max() <= 1, its
    assert np.abs(its[2] - its[0]).max() <= max(3, int(0.1 * its[0].max())), its


def _jacobi_factor(T, A, scale=1.0):
    """L = D^-1/2 plus -0.1 a_ij / a_ii on the strictly lower pattern."""
    a = A.arrays()
    n = len(a["rowptr"]) - 1
    rp, ci, va = [0], [], []
    for i in range(n):
        cols = a["colidx"][a["rowptr"][i]:a["rowptr"][i + 1]]
        vals = a["values"][a["rowptr"][i]:a["rowptr"][i + 1]]
        d = vals[cols == i][0]
        for c, v in sorted(zip(cols, vals)):
            if c < i:
                ci.append(int(c))
                va.append(scale * -0.1 * v / d)
        ci.append(i)
        va.append(scale / np.sqrt(d))
        rp.append(len(ci))
    return T.MatrixCSR.from_arrays(n, n, np.array(rp, np.int32), np.array(ci, np.int32), np.array(va))


def test_jacobi_fallback_on_bad_factors(gpu):
    """Jacobi-PCG is the fallback of the factored preconditioner.  Factors are
    spoiled on the host: system 0 gets a NaN, system 1 a zero diagonal entry
    (both fail the check made before the first iteration: fallback 1),
    system 2 a factor scaled by 1e-30 whose application underflows in FP32 so
    that r.z = 0 (fallback 2); system 3 keeps a good factor.  Every system
    must still end DONE at the FP64-verified 1e-8, the spoiled ones through
    Jacobi, and the per-system status must say so.  No device fault is
    involved: the bad values are ordinary data."""
    T = gpu
    systems = [diffusion(T, 9 + i, 800 + i) for i in range(4)]
    factors = [_jacobi_factor(T, A) for A in systems]
    f0 = factors[0].arrays()
    f0["values"][len(f0["values"]) // 2] = np.nan
    n0 = len(f0["rowptr"]) - 1
    factors[0] = T.MatrixCSR.from_arrays(n0, n0, f0["rowptr"], f0["colidx"], f0["values"])
    f1 = factors[1].arrays()
    n1 = len(f1["rowptr"]) - 1
    f1["values"][f1["rowptr"][n1 // 2 + 1] - 1] = 0.0  # a diagonal entry (last of its row)
    factors[1] = T.MatrixCSR.from_arrays(n1, n1, f1["rowptr"], f1["colidx"], f1["values"])
    factors[2] = _jacobi_factor(T, systems[2], scale=1e-30)
    for prec in (T.F32, T.BF16):
        bt = T.Batch(systems, T.F32)
        bt.set_factors(factors, prec)
        rhs = np.concatenate([T.fill_uniform(len(s.arrays()["rowptr"]) - 1, -1.0, 1.0, 90 + i)
                              for i, s in enumerate(systems)])
        x, its, rr, ok = bt.cg(rhs, max_iterations=5000, rel_tol=1e-8, precond=2, refresh=50)
        assert ok and (rr <= 1e-8).all(), (its, rr)
        fb, used = bt.fallbacks()
        assert list(fb) == [1, 1, 2, 0], fb
        assert list(used) == [1, 1, 1, 2], used
        assert bt.engine()["persistent"]
        o = 0
        for s in systems:
            a = s.arrays()
            k = len(a["rowptr"]) - 1
            res = rhs[o:o + k] - oracle.csr_ax(a["rowptr"], a["colidx"], a["values"], x[o:o + k])
            assert np.linalg.norm(res) <= 1.0001e-8 * np.linalg.norm(rhs[o:o + k])
            o += k


def test_slow_factor_falls_back(gpu):
    """A factor that keeps lowering the residual, but too slowly, is given up
    too: with the network head set to L = D^-1/2 (I + 4 E_lower) (E the
    scaled off-diagonal entries) the factored iteration keeps 0.90-0.99 of
    the residual norm per 50 iterations on these systems and does not
    converge in 4,000 iterations (float64 restatement on the host).  The
    first refinement cycle that cuts the FP64 true residual by less than
    10% hands each system to Jacobi: all reach the FP64-verified 1e-8, with
    fallback code 2."""
    T = gpu
    systems = [diffusion(T, 12 + 4 * i, 741 + i) for i in range(2)]
    net = T.MPNN(3)
    p = M.unpack(net.params().astype(np.float64))
    p["ce"] = 4.0
    net.set_params(M.pack(p).astype(np.float32))
    bt = T.Batch(systems, T.F32)
    bt.factor_mpnn(net, T.F32)
    rhs = np.concatenate([T.fill_uniform(len(s.arrays()["rowptr"]) - 1, -1.0, 1.0, 40 + i)
                          for i, s in enumerate(systems)])
    x, its, rr, ok = bt.cg(rhs, max_iterations=4000, rel_tol=1e-8, precond=2, refresh=50)
    assert ok and (rr <= 1e-8).all(), (its, rr)
    fb, used = bt.fallbacks()
    assert list(fb) == [2, 2] and list(used) == [1, 1], (fb, used)
    assert (its < 1000).all(), its
    o = 0
    for s in systems:
        a = s.arrays()
        k = len(a["rowptr"]) - 1
        res = rhs[o:o + k] - oracle.csr_ax(a["rowptr"], a["colidx"], a["values"], x[o:o + k])
        assert np.linalg.norm(res) <= 1.0001e-8 * np.linalg.norm(rhs[o:o + k])
        o += k


def test_device_factor_pipeline_matches_host_factor(gpu):
    """tbsla_batch_factor_mpnn runs the network on the batch's device copy of
    A and writes L into the batch's factor storage with no host round trip.
    It must produce the factor of tbsla_mpnn_factor (the network on the
    host-built graph) loaded through tbsla_batch_set_factors: the same FP32
    operations in the same order, so equal to a few units in the last place
    of FP32 (1e-6 of max |L|; the oracle bar for the factor is 1e-5).  Both
    solves then reach the FP64-verified 1e-8 in the same iterations, up to
    the one that the order of the FP64 atomic dot products can move."""
    T = gpu
    net = T.MPNN(11)
    train = [diffusion(T, 9 + (i % 5), 2000 + i) for i in range(10)]
    for step in range(60):
        net.train_step(train[step % len(train)], probes=8, seed=step, lr=3e-3)
    systems = [diffusion(T, 8 + 3 * i, 3000 + i) for i in range(4)]
    rhs = np.concatenate([T.fill_uniform(len(s.arrays()["rowptr"]) - 1, -1.0, 1.0, 70 + i)
                          for i, s in enumerate(systems)])
    for prec in (T.F32, T.BF16):
        host = T.Batch(systems, T.F32)
        host.set_factors([net.factor(A) for A in systems], prec)
        dev = T.Batch(systems, T.F32)
        dev.factor_mpnn(net, prec)
        dh, vh = host.factor_dia()
        dd, vd = dev.factor_dia()
        assert np.array_equal(dh, dd)
        assert np.abs(vh - vd).max() <= 1e-6 * np.abs(vh).max(), np.abs(vh - vd).max()
        its = []
        for bt in (host, dev):
            x, it, rr, ok = bt.cg(rhs, max_iterations=5000, rel_tol=1e-8, precond=2, refresh=50)
            assert ok and (rr <= 1e-8).all()
            assert bt.engine()["persistent"]
            fb, used = bt.fallbacks()
            assert (fb == 0).all() and (used == 2).all()
            its.append(it)
        assert np.abs(its[0] - its[1]).max() <= 1, its
