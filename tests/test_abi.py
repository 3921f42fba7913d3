"""C-ABI boundary checks that need no GPU: the library builds for sm_103a, exports every
symbol include/pic_gb300.h declares, and refuses to run without a CUDA device (no CPU
fallback).  The C++ facade header compiles against the C ABI."""
import ctypes as C
import os
import re
import subprocess

import pytest

from conftest import ROOT, PKG_NAME


def header_symbols():
    text = open(os.path.join(ROOT, "include", "pic_gb300.h")).read()
    return sorted(set(re.findall(r"^int (pic_\w+)\(", text, flags=re.M)))


def test_library_exports_every_declared_symbol(pic):
    L = pic.library()
    syms = header_symbols()
    assert len(syms) >= 30
    missing = [s for s in syms if not hasattr(L, s)]
    assert not missing, missing


def test_no_cpu_fallback_without_device(pic):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(pic.PicError) as ei:
        pic.World(5, 5, 5, (0, 0, 0), (1, 1, 1))
    assert ei.value.code == pic.PIC_ERR_CUDA


def test_last_error_message_is_reported(pic):
    L = pic.library()
    rc = L.pic_world_set_time(None, 1.0, 1)
    assert rc == pic.PIC_ERR_ARG
    buf = C.create_string_buffer(256)
    L.pic_last_error(buf, 256)
    assert b"dt" in buf.value or b"null" in buf.value


@pytest.mark.parametrize("src", ["include/pic_gb300.hpp", "include/pic_gb300_outputs.hpp",
                                 PKG_NAME + "/examples/v3_loop.cpp"])
def test_cpp_facade_compiles(src):
    r = subprocess.run(["g++", "-std=c++17", "-Wall", "-Werror", "-fsyntax-only", "-x", "c++", os.path.join(ROOT, src),
                        "-I", os.path.join(ROOT, "include")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
