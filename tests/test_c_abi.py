"""The C ABI from C: a program built with gcc against include/fmm_gb300.h
and linked with libfmm_gb300.so, as the BLIS-side shim would be, runs the
host-only entry points (no GPU needed)."""
import shutil
import subprocess

import pytest

from conftest import COEFFS, ROOT


def test_abi_from_c(fmm, tmp_path):
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    exe = tmp_path / "abi_from_c"
    libdir = fmm.LIB_PATH.parent
    cmd = ["gcc", "-std=c11", "-O1", "-Wall", "-Werror", str(ROOT / "tests" / "c" / "abi_from_c.c"),
           f"-I{ROOT / 'include'}", f"-L{libdir}", "-lfmm_gb300", f"-Wl,-rpath,{libdir}", "-o", str(exe)]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    out = subprocess.run([str(exe), str(COEFFS)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    assert out.stdout.strip() == "ok"
