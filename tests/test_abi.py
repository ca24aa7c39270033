"""The C-ABI library loads without a GPU and exports every function the
public header declares."""
import re

from conftest import ROOT


def header_functions():
    text = (ROOT / "include" / "fmm_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = set(re.findall(r"\b([a-z_][a-z0-9_]*)\s*\(", text))
    return sorted(n for n in names if n not in {"if", "sizeof", "defined"})


def test_exports_every_declared_symbol(fmm):
    L = fmm.lib()
    names = header_functions()
    assert "fmm_gpu_dgemm" in names and "new_fmm" in names and "fmm_gpu_split_dgemm" in names
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert hasattr(L, "STRASSEN_FMM")


def test_library_is_sm103a_build(fmm):
    from fmm_blis_gb300 import build
    assert "arch=compute_103a,code=sm_103a" in " ".join(build.ARCH)
    assert fmm.LIB_PATH.exists()


def test_split_pair_rows_knob(fmm):
    """The pair-tile threshold is host state: no GPU needed; values below
    1024 are raised to 1024 and the previous value comes back."""
    prev = fmm.set_split_pair_rows(5000)
    try:
        assert fmm.set_split_pair_rows(10) == 5000
        assert fmm.set_split_pair_rows(2**40) == 1024
        assert fmm.set_split_pair_rows(1024) == 2**31 - 1
    finally:
        fmm.set_split_pair_rows(prev)


def test_split_host_call_rejects_bad_arguments(fmm):
    """Argument checks of the host-buffer split call come before any device
    work, so they hold without a GPU."""
    import numpy as np
    L = fmm.lib()
    A = np.zeros((4, 4), order="F")
    f = fmm.strassen_fmm()
    args = (1.0, A.ctypes.data, 4, A.ctypes.data, 4, 1.0, A.ctypes.data, 4, 4, 4, 4, f, 1)
    assert L.fmm_gpu_split_strassen_ab_ex(*args, 13, 1) == 1     # FP8 slices 2..12
    assert L.fmm_gpu_split_strassen_ab_ex(*args, 9, 0) == 1      # BF16 slices 2..8
    assert L.fmm_gpu_split_strassen_ab_ex(*args, 6, 2) == 1      # unknown format
    bad_ld = (1.0, A.ctypes.data, 3, A.ctypes.data, 4, 1.0, A.ctypes.data, 4, 4, 4, 4, f, 1, 6, 0)
    assert L.fmm_gpu_split_strassen_ab_ex(*bad_ld) == 1          # lda < m


def test_split_host_gen_rejects_bad_arguments(fmm):
    """The general-layout split host call checks strides, format and slices
    before any device work."""
    import numpy as np
    L = fmm.lib()
    A = np.zeros((4, 4))
    f = fmm.strassen_fmm()
    p = A.ctypes.data
    ok = (1.0, p, 4, 1, p, 4, 1, 1.0, p, 4, 1, 4, 4, 4, f, 1)
    assert L.fmm_gpu_split_strassen_ab_gen(*ok, 13, 1) == 1                            # slices
    assert L.fmm_gpu_split_strassen_ab_gen(*ok, 6, 3) == 1                             # format
    bad = (1.0, p, 0, 1, p, 4, 1, 1.0, p, 4, 1, 4, 4, 4, f, 1, 6, 0)                   # row stride 0
    assert L.fmm_gpu_split_strassen_ab_gen(*bad) == 1
    assert L.fmm_gpu_split_strassen_ab_gen(1.0, p, 4, 1, p, 4, 1, 1.0, p, 4, 1, -1, 4, 4, f, 1, 6, 0) == 1


def test_host_alloc_arguments_and_missing_gpu(fmm):
    """fmm_gpu_host_alloc checks its arguments before touching the GPU; where
    no GPU is present it fails with a status (no memory is handed out), and
    fmm.host_empty raises instead of returning unpinned memory."""
    import ctypes

    import pytest
    L = fmm.lib()
    p = ctypes.c_void_p(1234)
    assert L.fmm_gpu_host_alloc(0, ctypes.byref(p)) == 1 and not p.value       # zero bytes
    assert L.fmm_gpu_host_alloc(4096, None) == 1                              # no result pointer
    assert L.fmm_gpu_host_free(None) == 0                                     # freeing NULL is a no-op
    assert L.fmm_gpu_host_free(ctypes.c_void_p(4096)) == 1                    # not from fmm_gpu_host_alloc
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present: the allocation itself is covered by the GPU tests")
    assert L.fmm_gpu_host_alloc(1 << 20, ctypes.byref(p)) == 5 and not p.value
    with pytest.raises(RuntimeError):
        fmm.host_empty(16, 16)
