"""tbsla_gb300: GB300-native SpMV (COO / SCOO / CSR / ELL / DENSE), PageRank and
CG behind the TBSLA Matrix API.

The compute path is the native library ``libtbsla_gb300.so`` (hand-written
sm_103a kernels behind the C ABI of ``include/tbsla_gb300.h``); this package
is its Python mirror.  Import fails if the library has not been built.
"""
from . import _lib
from ._lib import BF16, COO, CSR, DENSE, ELL, F32, F64, SCOO, TbslaError, check, lib
from .matrix import (FORMATS, MPNN, Batch, Matrix, MatrixCOO, MatrixCSR, MatrixDENSE, MatrixELL, MatrixSCOO,
                     device_init, fill_uniform)

__all__ = ["MPNN", "Matrix", "MatrixCOO", "MatrixSCOO", "MatrixCSR", "MatrixELL", "MatrixDENSE", "FORMATS",
           "fill_uniform", "device_init", "TbslaError", "check", "lib", "COO", "SCOO", "CSR", "ELL",
           "DENSE", "F64", "F32", "BF16"]
