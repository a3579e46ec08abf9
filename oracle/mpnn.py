"""Oracle (test infrastructure only): a float64 numpy restatement of the
learned preconditioner's network, its loss and the loss's gradient, used to
check the GPU forward / backward kernels.  The reference has no
preconditioner (src/mpi/matrix/CG.cpp:32-73 is plain CG), so this restates
the project's own model, defined here and in tbsla_gb300/csrc/kernels/mpnn.cu:

  A: SPD CSR matrix, s_i = a_ii^-1/2, e_ij = a_ij s_i s_j (stored entries).
  node input x_i = [1, sum_{j!=i} e_ij, sum_{j!=i} e_ij^2, deg_i / 8]
  h0_i = relu(W0 x_i + b0)                                  (H = 32)
  layer l = 1..3: m_i = sum_{j!=i} e_ij h_j;  z = W_l [h_i; m_i] + b_l;
                  h_i <- h_i + relu(z)
  factor L on the pattern of tril(A):
    L_ij = s_i (w_e . (h_i * h_j) + c_e e_ij + b_e)   (j < i)
    L_ii = s_i softplus(w_d . h_i + b_d)
  M^-1 = L L^T (SPD whenever every L_ii > 0).
  loss over probes Z (N x P): R = L L^T A Z - Z, loss = sum R^2 / (N P).

The parameters live in one flat vector (layout `PARAM_LAYOUT`); the forward
pass uses them rounded to bfloat16, as the GPU does.
"""
from __future__ import annotations

import numpy as np

H = 32
F0 = 4
NLAYERS = 3
PARAM_LAYOUT = ([("W0", (H, F0)), ("b0", (H,))]
                + [(f"{n}{l}", s) for l in range(1, NLAYERS + 1) for n, s in (("W", (H, 2 * H)), ("b", (H,)))]
                + [("we", (H,)), ("ce", ()), ("be", ()), ("wd", (H,)), ("bd", ())])
NPARAMS = sum(int(np.prod(s)) if s else 1 for _, s in PARAM_LAYOUT)


def unpack(theta):
    out, o = {}, 0
    for name, shape in PARAM_LAYOUT:
        k = int(np.prod(shape)) if shape else 1
        out[name] = theta[o:o + k].reshape(shape) if shape else theta[o]
        o += k
    return out


def pack(parts):
    return np.concatenate([np.atleast_1d(np.asarray(parts[n], np.float64)).ravel() for n, _ in PARAM_LAYOUT])


def bf16(a):
    """float -> bfloat16 (round to nearest even) -> float64."""
    f = np.ascontiguousarray(a, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def init_params(seed=0):
    """He-scaled random message layers; the head starts at L = D^-1/2
    (Jacobi): w_e = c_e = b_e = w_d = 0, softplus(b_d) = 1."""
    rng = np.random.default_rng(seed)
    p = {"W0": rng.normal(0, np.sqrt(2.0 / F0), (H, F0)), "b0": np.zeros(H)}
    for l in range(1, NLAYERS + 1):
        p[f"W{l}"] = rng.normal(0, 0.5 * np.sqrt(2.0 / (2 * H)), (H, 2 * H))
        p[f"b{l}"] = np.zeros(H)
    p.update(we=np.zeros(H), ce=0.0, be=0.0, wd=np.zeros(H), bd=np.log(np.e - 1.0))
    return pack(p)


def graph(rowptr, colidx, values):
    n = len(rowptr) - 1
    rows = np.repeat(np.arange(n), np.diff(rowptr))
    diag = np.zeros(n)
    m = colidx == rows
    np.add.at(diag, rows[m], values[m])
    s = 1.0 / np.sqrt(diag)
    e = values * s[rows] * s[colidx]
    off = ~m
    x = np.zeros((n, F0))
    x[:, 0] = 1.0
    np.add.at(x[:, 1], rows[off], e[off])
    np.add.at(x[:, 2], rows[off], e[off] ** 2)
    np.add.at(x[:, 3], rows[off], 1.0 / 8)
    low = colidx < rows
    return {"n": n, "rows": rows, "cols": colidx, "e": e, "s": s, "x": x, "off": off, "low": low}


def forward(theta, g):
    """Returns (Lrows, Lcols, Lvals, cache)."""
    p = unpack(bf16(theta))
    n, rows, cols, e, off = g["n"], g["rows"], g["cols"], g["e"], g["off"]
    cache = {}
    z0 = g["x"] @ p["W0"].T + p["b0"]
    h = np.maximum(z0, 0)
    cache["z0"], hs, ms, zs = z0, [h], [], []
    for l in range(1, NLAYERS + 1):
        m = np.zeros((n, H))
        np.add.at(m, rows[off], e[off, None] * h[cols[off]])
        z = np.concatenate([h, m], 1) @ p[f"W{l}"].T + p[f"b{l}"]
        h = h + np.maximum(z, 0)
        ms.append(m)
        zs.append(z)
        hs.append(h)
    cache.update(hs=hs, ms=ms, zs=zs, p=p)
    lo = g["low"]
    i, j = rows[lo], cols[lo]
    o = (h[i] * h[j]) @ p["we"] + p["ce"] * e[lo] + p["be"]
    xi = h @ p["wd"] + p["bd"]
    sp = np.logaddexp(0, xi)
    Lr = np.concatenate([i, np.arange(n)])
    Lc = np.concatenate([j, np.arange(n)])
    Lv = np.concatenate([g["s"][i] * o, g["s"] * sp])
    cache.update(i=i, j=j, o=o, xi=xi)
    return Lr, Lc, Lv, cache


def _spmm(r, c, v, X, n, transpose=False):
    out = np.zeros((n, X.shape[1]))
    if transpose:
        np.add.at(out, c, v[:, None] * X[r])
    else:
        np.add.at(out, r, v[:, None] * X[c])
    return out


def loss_and_grad(theta, rowptr, colidx, values, Z):
    """loss and d loss / d theta (float64), theta in PARAM_LAYOUT order."""
    g = graph(rowptr, colidx, values)
    n, P = g["n"], Z.shape[1]
    Lr, Lc, Lv, c = forward(theta, g)
    U = _spmm(g["rows"], g["cols"], values, Z, n)
    V = _spmm(Lr, Lc, Lv, U, n, transpose=True)
    W = _spmm(Lr, Lc, Lv, V, n)
    R = W - Z
    loss = float((R ** 2).sum() / (n * P))
    gW = 2 * R / (n * P)
    gV = _spmm(Lr, Lc, Lv, gW, n, transpose=True)
    dL = (gW[Lr] * V[Lc]).sum(1) + (U[Lr] * gV[Lc]).sum(1)
    p, hs, ms, zs = c["p"], c["hs"], c["ms"], c["zs"]
    h = hs[-1]
    nl = len(c["i"])
    i, j, s = c["i"], c["j"], g["s"]
    do = s[i] * dL[:nl]
    dsp = s * dL[nl:]
    dxi = dsp / (1 + np.exp(-c["xi"]))
    grads = {"we": (do[:, None] * h[i] * h[j]).sum(0), "ce": float((do * g["e"][g["low"]]).sum()),
             "be": float(do.sum()), "wd": dxi @ h, "bd": float(dxi.sum())}
    dh = np.outer(dxi, p["wd"])
    np.add.at(dh, i, do[:, None] * p["we"] * h[j])
    np.add.at(dh, j, do[:, None] * p["we"] * h[i])
    rows, cols, e, off = g["rows"], g["cols"], g["e"], g["off"]
    for l in range(NLAYERS, 0, -1):
        hp = hs[l - 1]
        dz = dh * (zs[l - 1] > 0)
        inp = np.concatenate([hp, ms[l - 1]], 1)
        grads[f"W{l}"] = dz.T @ inp
        grads[f"b{l}"] = dz.sum(0)
        din = dz @ p[f"W{l}"]
        dm = din[:, H:]
        dh = dh + din[:, :H]
        np.add.at(dh, cols[off], e[off, None] * dm[rows[off]])
    dz0 = dh * (c["z0"] > 0)
    grads["W0"] = dz0.T @ g["x"]
    grads["b0"] = dz0.sum(0)
    return loss, pack(grads)


def factor(theta, rowptr, colidx, values):
    """L as (rows, cols, vals) triplets: strictly lower entries, then the diagonal."""
    Lr, Lc, Lv, _ = forward(theta, graph(rowptr, colidx, values))
    return Lr, Lc, Lv
