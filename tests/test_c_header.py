"""include/fermicc.h is a plain C header: a C99 program (tests/abi_check.c)
compiles against it with warnings as errors, links libfermicc.so and checks
the argument validation and status strings (no device needed)."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT


def test_c99_program_against_the_header(tmp_path):
    from fermicc import _lib
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    if not os.path.exists(_lib.LIB_PATH):
        import __graft_entry__
        __graft_entry__.build()
    libdir = os.path.dirname(_lib.LIB_PATH)
    exe = str(tmp_path / "abi_check")
    cmd = [cc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "abi_check.c"), "-o", exe, "-L", libdir, "-lfermicc",
           f"-Wl,-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "abi_check ok" in r.stdout
