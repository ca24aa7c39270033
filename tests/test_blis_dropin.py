"""The reference's own test driver on this library (the drop-in boundary).

test/test_strassen_oapi.c is compiled unchanged against the reference's
headers (frame/include/bli_fmm.h) and linked with the BLIS-side shim
(fmm_blis_gb300/blis/bli_strassen_ab_gpu.c, which defines bli_strassen_ab_ex
and bli_strassen_ab over fmm_gpu_strassen_ab_gen), libfmm_gb300.so and BLIS
(libblis.a from the reference build in oracle/_ref/) instead of the
reference's libfmm.a and fmm_blis plugin. Needs the reference build, so it
runs where the reference sources are mounted; the GPU machine has neither
BLIS nor the reference, so the binary's GPU run is not part of the GPU tests.
Without a GPU the driver reaches the library's entry point, which reports
its status through the reference's error path (message, bli_abort)."""
import os
import shutil
import subprocess

import pytest

from conftest import COEFFS, ROOT

REF = ROOT / "oracle" / "_ref"
BLIS_INC = REF / "blis-inst" / "include" / "blis"
LIBBLIS = REF / "blis-inst" / "lib" / "libblis.a"
DRIVER = REF / "src" / "test" / "test_strassen_oapi.c"
SHIM = ROOT / "fmm_blis_gb300" / "blis" / "bli_strassen_ab_gpu.c"

pytestmark = pytest.mark.skipif(not (LIBBLIS.exists() and DRIVER.exists()),
                                reason="reference build (oracle/build_ref.sh) not present")


def run(cmd, **kw):
    p = subprocess.run(cmd, capture_output=True, text=True, **kw)
    assert p.returncode == 0, " ".join(map(str, cmd)) + "\n" + p.stdout + p.stderr
    return p


@pytest.fixture(scope="module")
def driver(fmm, tmp_path_factory):
    d = tmp_path_factory.mktemp("oapi")
    from fmm_blis_gb300 import build
    lib = build.LIB
    run(["gcc", "-O2", "-Wall", "-Werror", "-c", str(SHIM), "-isystem", str(BLIS_INC), f"-I{ROOT / 'include'}", "-fopenmp",
         "-o", str(d / "shim.o")])
    run(["gcc", "-O2", "-w", "-fopenmp", "-c", str(DRIVER), f"-I{REF / 'src' / 'frame' / 'include'}",
         f"-I{REF / 'src' / 'plugin'}", f"-I{BLIS_INC}", "-o", str(d / "test.o")])
    run(["gcc", "-fopenmp", str(d / "test.o"), str(d / "shim.o"), f"-L{lib.parent}", "-lfmm_gb300",
         f"-Wl,-rpath,{lib.parent}", str(LIBBLIS), "-lm", "-lpthread", "-o", str(d / "test_strassen.x")])
    shutil.copyfile(COEFFS / "222.txt", d / "222.txt")
    return d / "test_strassen.x"


def test_driver_links_with_the_reference_symbol_names(driver):
    syms = run(["nm", str(driver)]).stdout.split("\n")
    defined = {ln.split()[-1] for ln in syms if len(ln.split()) == 3 and ln.split()[1] == "T"}
    undefined = {ln.split()[-1] for ln in syms if len(ln.split()) == 2 and ln.split()[0] == "U"}
    assert {"bli_strassen_ab_ex", "bli_strassen_ab", "bli_plugin_register_fmm_blis"} <= defined   # the shim
    assert {"new_fmm", "free_fmm", "bl_clock", "fmm_gpu_strassen_ab_gen"} <= undefined   # libfmm_gb300.so
    dyn = run(["readelf", "-d", str(driver)]).stdout
    assert "libfmm_gb300.so" in dyn


def test_driver_reaches_the_gpu_entry_point(driver):
    p = subprocess.run([str(driver)], capture_output=True, text=True, cwd=driver.parent, timeout=120,
                       env=dict(os.environ, BLIS_NUM_THREADS="1"))
    import torch
    if torch.cuda.is_available():
        assert p.returncode == 0, p.stdout + p.stderr
        resid = float(p.stdout.split()[-2])
        assert resid < 1e-7
    else:
        assert p.returncode != 0
        assert "bli_strassen_ab_ex: fmm_gpu_strassen_ab_gen:" in p.stderr
