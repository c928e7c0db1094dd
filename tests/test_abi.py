"""The C-ABI library loads without a GPU and exports every entry point of
include/bskit_gb300.h with the signatures the ctypes binding declares."""
import ctypes
import os
import re

import pytest

from bskit_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "bskit_gb300.h")


def header_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:int|int64_t)\s+(bsk_\w+)\s*\(", src, flags=re.M)))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(_lib.LIB_PATH):
        from bskit_gb300 import build
        build.build()
    return _lib.load()


def test_header_declares_the_boundary():
    names = header_functions()
    for required in ("bsk_plan_create", "bsk_paint", "bsk_measure_b", "bsk_gridinfo",
                     "bsk_shell_mode_counts", "bsk_triset_create", "bsk_normalize"):
        assert required in names


def test_library_exports_every_header_symbol(lib):
    for name in header_functions():
        assert hasattr(lib, name), name


def test_binding_covers_header(lib):
    bound = {n for n, _, _ in _lib.SIGNATURES}
    assert bound == set(header_functions())


def test_version_and_error_text(lib):
    assert lib.bsk_version() >= 100
    # NULL out-pointer: rejected on the host before any CUDA call
    rc = lib.bsk_plan_create(64, 100.0, 1, None, 0, 0, None)
    assert rc == _lib.BSK_ERR_ARG
    assert "NULL" in _lib.last_error()
    assert lib.bsk_triset_size(None) == -1
    buf = ctypes.create_string_buffer(4)
    assert lib.bsk_last_error(buf, 4) == 0 and len(buf.value) <= 3


def test_bad_arguments_rejected_without_gpu(lib):
    out = ctypes.c_void_p()
    edges = (ctypes.c_double * 2)(0.1, 0.2)
    assert lib.bsk_plan_create(63, 100.0, 1, edges, 0, 0, ctypes.byref(out)) == _lib.BSK_ERR_ARG
    assert lib.bsk_plan_create(64, -1.0, 1, edges, 0, 0, ctypes.byref(out)) == _lib.BSK_ERR_ARG
    assert lib.bsk_plan_create(64, 100.0, 0, edges, 0, 0, ctypes.byref(out)) == _lib.BSK_ERR_ARG
    assert lib.bsk_plan_create(64, 100.0, 1, edges, 7, 0, ctypes.byref(out)) == _lib.BSK_ERR_ARG
    assert lib.bsk_normalize(-1, None, None, None, None) == _lib.BSK_ERR_ARG


def test_host_checks_reject_bad_buffers():
    # buffers go to the kernels as raw pointers, so the object layer checks their size,
    # type, device and layout first (no GPU needed: these fail before any library call)
    import torch

    from bskit_gb300 import engine

    cpu = torch.device("cpu")
    good = torch.zeros(5, dtype=torch.float64)
    engine._check_tensor(good, "out", (5,), torch.float64, cpu)
    for bad in (torch.zeros(4, dtype=torch.float64), torch.zeros(5, dtype=torch.float32),
                torch.zeros(10, dtype=torch.float64)[::2], [0.0] * 5):
        with pytest.raises(ValueError):
            engine._check_tensor(bad, "out", (5,), torch.float64, cpu)
    with pytest.raises(ValueError):
        engine._check_tensor(good, "out", (5,), torch.float64, torch.device("cuda", 0))
    with pytest.raises(ValueError):
        engine.Plan.normalize(good, good)  # host tensors


def test_noalloc_arguments_rejected_without_gpu(lib):
    # checks that run before any CUDA call
    tri = (ctypes.c_int32 * 3)(0, 0, 0)
    f = ctypes.c_void_p(16)  # never dereferenced: every call below fails its checks first
    out = ctypes.c_void_p(16)
    P = _lib.PREC_BF16X3
    cases = [
        (0, 1, tri, f, 1024, P, out),        # no shells
        (256, 1, tri, f, 1024, P, out),      # more shells than a plan allows
        (1, 1, None, f, 1024, P, out),       # triangles missing
        (1, -1, tri, f, 1024, P, out),       # negative count
        (1, 1, tri, None, 1024, P, out),     # field missing
        (1, 1, tri, f, 1004, P, out),        # k_points not a multiple of 8
        (1, 1, tri, f, 1024, _lib.PREC_FP64, out),  # SIMT precisions are not offered here
        (1, 1, tri, ctypes.c_void_p(20), 1024, P, out),  # field not 16-byte aligned
    ]
    for n, t, tr, ff, k, prec, o in cases:
        rc = lib.bsk_contract_noalloc(n, t, tr, ff, ff if ff else f, ff if ff else f, k, prec,
                                      o, None)
        assert rc == _lib.BSK_ERR_ARG, (n, t, k, prec, _lib.last_error())
    # an empty list is a valid request that does nothing
    assert lib.bsk_contract_noalloc(1, 0, None, f, f, f, 1024, P, None, None) == _lib.BSK_OK
    # the plan-based entry points reject a missing plan before touching the device
    assert lib.bsk_measure_b(None, None, 0, 0, 0, P, None, None) == _lib.BSK_ERR_ARG
    assert lib.bsk_gridinfo(None, None, None, None, None) == _lib.BSK_ERR_ARG
    assert lib.bsk_contract(None, None, f, f, f, 1024, P, out, None) == _lib.BSK_ERR_ARG
    # a misaligned output pointer is rejected before the capture check or any device call
    assert lib.bsk_contract_noalloc(1, 1, tri, f, f, f, 1024, P, ctypes.c_void_p(20),
                                    None) == _lib.BSK_ERR_ARG
