"""The allocation-free CSR SpMV (tbsla_csr_Ax_device_noalloc), for callers
that may not call the CUDA allocator on the call path: against the handle
entry point tbsla_Ax_device with the same merge-path kernel (equal results
on two calls in a row, no device memory taken by the second call), against
the oracle's restatement of MatrixCSR::Ax (1e-13 of sum_j |a_ij x_j| per
row), and inputs past the scratch limit rejected.  The file sorts last so
that it also runs after every other GPU test."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def test_noalloc_matches_handle_entry_point(gpu):
    import torch

    T = gpu
    L = T.lib
    n = 300_000
    m = T.MatrixCSR()
    m.fill_powerlaw(n, seed=41)
    m.set_algorithm(m.MERGE, 8)
    a = m.arrays()
    nnz = int(a["rowptr"][-1] - a["rowptr"][0])
    rowptr = torch.from_numpy(a["rowptr"]).cuda()
    colidx = torch.from_numpy(a["colidx"]).cuda()
    values = torch.from_numpy(a["values"]).cuda()
    xs = [torch.from_numpy(T.fill_uniform(n, -1.0, 1.0, 50 + k)).cuda() for k in range(2)]
    ys = [torch.full((n,), 7.0, dtype=torch.float64, device="cuda") for _ in range(2)]
    refs = [torch.full((n,), 7.0, dtype=torch.float64, device="cuda") for _ in range(2)]
    stream = torch.cuda.current_stream()
    free = []
    for k in range(2):
        m.Ax_device(refs[k], xs[k], stream=stream)
        torch.cuda.synchronize()
        free.append(torch.cuda.mem_get_info()[0])
        st = L.tbsla_csr_Ax_device_noalloc(n, nnz, 0, _ptr(rowptr), _ptr(colidx), _ptr(values),
                                           _ptr(xs[k]), _ptr(ys[k]), C.c_void_p(stream.cuda_stream))
        torch.cuda.synchronize()
        assert st == 0, T.lib.tbsla_status_string(st)
        assert torch.equal(ys[k], refs[k]), k
        if k == 1:
            assert torch.cuda.mem_get_info()[0] == free[1]
    assert not torch.equal(ys[0], ys[1])
    # pinned directly to the oracle as well, not only to the other entry point
    import oracle

    for k in range(2):
        xk = xs[k].cpu().numpy()
        ref = oracle.csr_ax(a["rowptr"], a["colidx"], a["values"], xk)
        scale = oracle.csr_absrow(a["rowptr"], a["colidx"], a["values"], xk)
        assert oracle.rel_err_normalized(ys[k].cpu().numpy(), ref, scale) <= 1e-13, k


def test_noalloc_rejects_inputs_past_the_limit(gpu):
    import torch

    T = gpu
    L = T.lib
    limit = 134217728
    null = C.c_void_p(0)
    # one row of `limit` entries: one merge item too many.  The arrays are
    # real (1.5 GB), so nothing would read out of bounds even without the
    # check; the call must refuse and leave y alone.
    rowptr = torch.tensor([0, limit], dtype=torch.int32, device="cuda")
    colidx = torch.zeros(limit, dtype=torch.int32, device="cuda")
    values = torch.zeros(limit, dtype=torch.float64, device="cuda")
    x = torch.ones(1, dtype=torch.float64, device="cuda")
    y = torch.full((1,), 5.0, dtype=torch.float64, device="cuda")
    st = L.tbsla_csr_Ax_device_noalloc(1, limit, 0, _ptr(rowptr), _ptr(colidx), _ptr(values), _ptr(x),
                                       _ptr(y), null)
    torch.cuda.synchronize()
    assert st == T._lib.ERR_INVALID_ARG and y.item() == 5.0
    del colidx, values
    st = L.tbsla_csr_Ax_device_noalloc(-1, 0, 0, null, null, null, null, null, null)
    assert st == T._lib.ERR_INVALID_ARG
    y = torch.full((4,), 5.0, dtype=torch.float64, device="cuda")
    # nnz == 0: r untouched, as MatrixCSR::Ax
    rp = torch.zeros(5, dtype=torch.int32, device="cuda")
    st = L.tbsla_csr_Ax_device_noalloc(4, 0, 0, _ptr(rp), null, null, null, _ptr(y), null)
    torch.cuda.synchronize()
    assert st == 0 and torch.equal(y, torch.full((4,), 5.0, dtype=torch.float64, device="cuda"))
