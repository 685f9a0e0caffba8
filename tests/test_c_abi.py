"""The C ABI from plain C (CPU): tests/c_abi_host.c is compiled with gcc as
strict C99 against include/radis_gb300.h, linked against the built library
and run; it checks the host-only entry points (version, partition tables,
HITRAN-160 parsing, node grid) and that a context without a GPU is an error
status, not an abort."""
import os
import shutil
import subprocess

import pytest

from radis_gb300 import _lib as L

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_plain_c_caller(native_lib, tmp_path):
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("gcc not found")
    exe = str(tmp_path / "c_abi_host")
    libdir = os.path.dirname(L.LIB_PATH)
    cmd = [gcc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "c_abi_host.c"), "-o", exe, "-L", libdir, "-lradisgb",
           f"-Wl,-rpath,{libdir}", "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr
