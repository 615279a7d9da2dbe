"""The C ABI library loads and exports every function that
include/haplo_gb300.h declares, and the ctypes binding covers all of them.
No compute call is made (no GPU needed)."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "haplo_gb300.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(hx_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_the_reference_runners():
    names = declared_functions()
    for must in ("hx_create", "hx_loglikelihood", "hx_em_accum", "hx_update_q_accum", "hx_update_p_accum",
                 "hx_qp_q", "hx_qp_p", "hx_project_q", "hx_project_p", "hx_zal", "hx_init_em",
                 "hx_admixture_qn", "hx_fit", "hx_census"):
        assert must in names


def test_library_exports_every_declared_symbol(built_lib):
    lib = ctypes.CDLL(built_lib)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_ctypes_binding_covers_header(hx):
    from haplo_gb300 import _lib
    assert set(declared_functions()) == set(_lib.SIGNATURES)


def test_status_strings_without_gpu(hx):
    lib = hx.load()
    assert lib.hx_status_string(0) == b"ok"
    assert lib.hx_status_string(7) == b"unsupported size"
    assert lib.hx_last_error(None) == b"null context"


def test_create_without_device_fails_loudly(hx):
    """No CPU fallback: where no CUDA device is usable, hx_create returns an
    error status (the ctypes wrapper raises)."""
    import numpy as np
    import pytest
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    bed = np.zeros((2, 1), dtype=np.uint8)
    with pytest.raises(hx.HxError):
        hx.GB300Admix(bed, 4, 1, 2)
