"""The C++ PirServer mirror (include/inspire_pir.hpp) through a compiled C++
test program (tests/cpp/pir_server_test.cc), the way a reference maintainer
would call the library from C++."""
import os
import subprocess

import pytest

from inspire_gb300 import build
from oracle import build_oracle

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cpp_pir_server_mirror(tmp_path):
    lib = build.build()
    orc = build_oracle.build()
    exe = str(tmp_path / "pir_server_test")
    cmd = ["g++", "-std=c++17", "-O1",
           "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(ROOT, "oracle"),
           os.path.join(ROOT, "tests", "cpp", "pir_server_test.cc"),
           "-o", exe,
           "-L", os.path.dirname(lib), "-linspire_gb300",
           "-L", os.path.dirname(orc), "-lpir_oracle",
           "-Wl,-rpath," + os.path.dirname(lib),
           "-Wl,-rpath," + os.path.dirname(orc)]
    subprocess.run(cmd, check=True)
    r = subprocess.run([exe, str(tmp_path)], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "all checks passed" in r.stdout
