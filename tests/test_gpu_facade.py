"""The C++ facade drives a ch4/v3-style loop (examples/v3_loop.cpp) through the C ABI."""
import os
import subprocess

import pytest

from conftest import ROOT, PKG_NAME

pytestmark = pytest.mark.gpu


def test_v3_style_cpp_driver(pic, tmp_path):
    pic.library()  # builds lib/libpic_gb300.so
    pkg = os.path.join(ROOT, PKG_NAME)
    exe = str(tmp_path / "v3_loop")
    r = subprocess.run(["g++", "-std=c++17", "-O2", os.path.join(pkg, "examples", "v3_loop.cpp"),
                        "-I", os.path.join(ROOT, "include"), "-L", os.path.join(pkg, "lib"), "-lpic_gb300",
                        "-Wl,-rpath," + os.path.join(pkg, "lib"), "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe, "10"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    line = r.stdout.strip().splitlines()[-1]
    fields = dict(kv.split("=") for kv in line.split())
    assert int(fields["ts"]) == 11
    assert int(fields["electrons"]) >= 200000 and int(fields["ions"]) >= 200000
    assert int(fields["collisions"]) > 0
