"""The C++ drop-in classes, used from C++ exactly as the reference's classes:
compiles tests/cpp/test_dropin.cpp against tbsla_gb300/cpp/include and
libtbsla.so, runs it on the GPU."""
import os
import subprocess

import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu


def test_cpp_dropin_known_answers(gpu, tmp_path):
    exe = tmp_path / "test_dropin"
    pkg = os.path.join(ROOT, "tbsla_gb300")
    subprocess.check_call(["g++", "-O2", "-std=c++14", "-I", os.path.join(pkg, "cpp", "include"), "-I",
                           os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "cpp", "test_dropin.cpp"),
                           "-L", pkg, "-ltbsla", "-ltbsla_gb300", f"-Wl,-rpath,{pkg}", "-o", str(exe)])
    res = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stdout + res.stderr
    assert "=== finished without error ===" in res.stdout
