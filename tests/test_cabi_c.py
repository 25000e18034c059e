"""The C ABI from a plain C99 caller (tests/cabi_smoke.c): the header
compiles as C (-std=c99 -pedantic -Werror) and as C++, and a C program
links the library and plans a network, gets a status and message for a bad
tree, and creates a program (a CUDA error without a GPU, success with one)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_c_caller(pkg, tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    libdir = os.path.dirname(pkg.native.LIB_PATH)
    exe = str(tmp_path / "cabi_smoke")
    subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cabi_smoke.c"), "-L", libdir, "-ltqec_gb300",
                    f"-Wl,-rpath,{libdir}", "-o", exe], check=True, capture_output=True, text=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "classes=2 syndrome=2" in r.stdout and "bad tree: -1" in r.stdout
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx:
        subprocess.run([cxx, "-std=c++17", "-Wall", "-Werror", "-fsyntax-only", "-x", "c++",
                        os.path.join(ROOT, "include", "tqec_gb300.h")], check=True)
