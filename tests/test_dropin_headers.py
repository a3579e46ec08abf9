"""The C++ drop-in headers against the reference's own programs: every
src/cpp/tests/*.cpp and src/cpp/apps/tbsla_perf.cpp of the TBSLA tree must
compile unchanged (g++ -fsyntax-only) with tbsla_gb300/cpp/include ahead of
the reference's include directory, so the Matrix classes come from this
library and only the reference's utility headers (tbsla/cpp/utils/*) from
the tree.  Runs where TBSLA_REFERENCE_ROOT names the TBSLA source tree;
skipped elsewhere.  The push_back / empty-constructor additions are checked
on the host arrays."""
import glob
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT


def _ref_root():
    root = os.environ.get("TBSLA_REFERENCE_ROOT")
    if not root or not os.path.isdir(os.path.join(root, "src", "cpp", "include")):
        pytest.skip("TBSLA_REFERENCE_ROOT does not name the TBSLA source tree")
    return root


def _programs():
    root = os.environ.get("TBSLA_REFERENCE_ROOT")
    if not root:
        return []
    return sorted(glob.glob(os.path.join(root, "src", "cpp", "tests", "*.cpp"))) + \
        [os.path.join(root, "src", "cpp", "apps", "tbsla_perf.cpp")]


@pytest.mark.parametrize("program", _programs() or ["(reference tree absent)"],
                         ids=lambda p: os.path.basename(p))
def test_reference_program_compiles_against_dropin(program):
    root = _ref_root()
    cmd = ["g++", "-std=c++17", "-fsyntax-only",
           "-I", os.path.join(ROOT, "tbsla_gb300", "cpp", "include"),
           "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(root, "src", "cpp", "include"), program]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr[-3000:]


def test_scoo_push_back_builds_entries():
    import tbsla_gb300 as T

    import ctypes as C

    from tbsla_gb300.matrix import _info

    m = T.MatrixSCOO()
    T.check(T.lib.tbsla_matrix_set_coo(m._h, C.byref(_info(n_row=4, n_col=5, ln_row=4, ln_col=5, nnz=0)),
                                       None, None, None), "set_coo")
    entries = [(0, 1, 2.0), (3, 4, -1.5), (2, 0, 0.25)] * 7
    for r, c, v in entries:
        m.push_back(r, c, v)
    a = m.arrays()
    assert m.get_nnz() == len(entries)
    assert np.array_equal(a["row"], [e[0] for e in entries])
    assert np.array_equal(a["col"], [e[1] for e in entries])
    assert np.array_equal(a["values"], [e[2] for e in entries])
    csr = T.MatrixCSR()
    assert T.lib.tbsla_matrix_push_back(csr._h, 0, 0, 1.0) == T._lib.ERR_INVALID_ARG
