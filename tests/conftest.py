import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")
    # The native library and the oracle are built in-tree; build them once per
    # session if missing or stale (no-op when up to date).
    import importlib.util

    spec = importlib.util.spec_from_file_location("_tbsla_build", os.path.join(ROOT, "tbsla_gb300", "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.build()
    from oracle import build as ob

    ob.build_oracle()


def has_gpu() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def golden():
    def load(name):
        return np.load(os.path.join(GOLDEN, name))

    return {n: load(n + ".npz") for n in ("gen", "ops", "files", "cfg1", "spmm")}


META = "n_row n_col ln_row ln_col f_row f_col pr pc NR NC max_col".split()


def info_of(arr):
    d = dict(zip(META, [int(v) for v in arr[:11]]))
    d["nnz"] = int(arr[11])
    return d


def golden_cases(npz, prefix):
    """{case_key: {"info": dict, arrays..., "ax": y}} for keys under prefix/."""
    out = {}
    for k in npz.files:
        if not k.startswith(prefix + "/"):
            continue
        case, field = k.rsplit("/", 1)
        out.setdefault(case, {})[field] = npz[k]
    for case in out.values():
        case["info"] = info_of(case["info"])
    return out


@pytest.fixture(scope="session")
def gpu():
    if not has_gpu():
        pytest.skip("no CUDA device")
    import tbsla_gb300 as T

    T.device_init(0)
    return T
