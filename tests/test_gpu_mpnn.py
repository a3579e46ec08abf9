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
    """Factors of at most 8 entries per row are applied from an ELL copy
    (2-byte column offsets, no row pointer; kernels unrolled for 4 or 8
    slots), longer ones from CSR.  The same factor padded with explicit
    zeros to 6 and to 11 entries per row takes the 8-slot ELL and the CSR
    paths: the same preconditioner (a zero product leaves an FP32 sum
    unchanged), so both solves reach the FP64-verified 1e-8 residual in the
    same number of iterations, to within the one that the order of the FP64
    atomic dot products can move."""
    T = gpu
    systems = [diffusion(T, 11 + i, 60 + i) for i in range(3)]
    # zeros added at the columns i - z, 0 < z <= pad: none (ELL, 4 slots),
    # 2 (ELL, up to 6 slots), 7 (CSR, up to 11 entries per row)
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
    its = [np.asarray(_solve(T, systems, f, 2, T.F32)) for f in layouts.values()]
    assert max(np.abs(its[0] - i).max() for i in its[1:]) <= 1
