"""ORACLE — test infrastructure only.

Build recipe for the two CPU checkers:

* ``oracle/_build/liboracle.so``: the C restatement in ``tbsla_oracle.c``,
  compiled with ``-ffp-contract=off`` (every product rounded before it is
  added, as the reference's loops are evaluated by g++ on x86-64) and OpenMP
  for the timed CPU baseline.
* ``oracle/_ref/libtbsla_ref.so``: the unmodified reference core
  (``src/cpp/matrix/*.cpp`` + ``src/cpp/utils/*.cpp``), compiled straight
  from where those sources lie in the reference tree, together with
  ``ref_shim.cpp``.  Built only where the reference tree is named by the
  environment variable ``TBSLA_REFERENCE_ROOT`` (the TBSLA source tree's
  root); it is used to record the golden vectors under ``tests/golden/`` and
  to validate the restatement.  Nothing is copied out of the reference tree.
"""
from __future__ import annotations

import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def ref_root() -> str | None:
    """The reference tree's root from TBSLA_REFERENCE_ROOT; None when unset.
    A set variable that names no TBSLA tree is an error."""
    root = os.environ.get("TBSLA_REFERENCE_ROOT")
    if not root:
        return None
    if not os.path.isdir(os.path.join(root, "src", "cpp", "matrix")):
        raise RuntimeError(f"TBSLA_REFERENCE_ROOT={root!r} holds no src/cpp/matrix: not a TBSLA source tree")
    return root

ORACLE_SO = os.path.join(HERE, "_build", "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libtbsla_ref.so")


def _newer(target: str, sources: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build_oracle(force: bool = False) -> str:
    srcs = [os.path.join(HERE, "tbsla_oracle.c"), os.path.join(HERE, "tbsla_oracle.h")]
    if force or _newer(ORACLE_SO, srcs):
        os.makedirs(os.path.dirname(ORACLE_SO), exist_ok=True)
        cmd = ["gcc", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
               "-std=c99", srcs[0], "-o", ORACLE_SO, "-lm"]
        subprocess.check_call(cmd)
    return ORACLE_SO


def reference_sources() -> list[str]:
    root = ref_root()
    if root is None:
        return []
    cpp = os.path.join(root, "src", "cpp")
    return sorted(glob.glob(os.path.join(cpp, "matrix", "*.cpp")) +
                  glob.glob(os.path.join(cpp, "utils", "*.cpp")))


def build_reference(force: bool = False) -> str | None:
    """Compile the reference core where its tree is mounted; None otherwise."""
    srcs = reference_sources()
    if not srcs:
        return REF_SO if os.path.exists(REF_SO) else None
    shim = os.path.join(HERE, "ref_shim.cpp")
    if force or _newer(REF_SO, srcs + [shim]):
        os.makedirs(os.path.dirname(REF_SO), exist_ok=True)
        inc = os.path.join(ref_root(), "src", "cpp", "include")
        cmd = ["g++", "-O3", "-std=c++14", "-fopenmp", "-fPIC", "-shared", "-I", inc,
               *srcs, shim, "-o", REF_SO]
        subprocess.check_call(cmd)
    return REF_SO


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_reference(force="--force" in sys.argv))
