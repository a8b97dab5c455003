"""The C++ host side over the C ABI: a program written against
include/kgr_attachment.hpp (AttachmentRTX's member functions) compiles with
g++, links libkgr.so and behaves like the reference's option surface."""
import os
import subprocess

import pytest

from artemis_gb300 import build, kgr

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cpp_adapter_options(tmp_path):
    kgr.lib()
    exe = tmp_path / "adapter_options"
    src = os.path.join(ROOT, "tests", "cpp", "adapter_options.cpp")
    cmd = ["g++", "-std=c++17", "-O1", "-I" + os.path.join(ROOT, "include"), src, "-o", str(exe),
           "-L" + build.LIBDIR, "-lkgr", "-Wl,-rpath," + build.LIBDIR]
    subprocess.check_call(cmd)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.split() == ["1", "8", "threaded", "0", "1", "1"]
