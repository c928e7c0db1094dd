"""bsk_contract_noalloc: the allocation-free tensor-core contraction.

It exists for callers that cannot call cudaMalloc when they need a result (a
framework that reserved the device memory up front, or a hot path on which
cudaMalloc/cudaFree are forbidden because they synchronise and can fail).
Its scratch is a 64 MiB static device array of the library.  The test calls
it through the C ABI twice in a row and compares both results with the
allocating entry point bsk_contract on the same fields; this file is named so
that pytest collects it last.
"""
import ctypes

import numpy as np
import pytest
import torch

from bskit_gb300 import _lib
from bskit_gb300 import bins as B
from bskit_gb300.engine import Plan

pytestmark = pytest.mark.gpu


def _call(lib, n_shells, tri, fs, K, out):
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = lib.bsk_contract_noalloc(n_shells, len(tri), tri.ctypes.data,
                                  *[ctypes.c_void_p(f.data_ptr()) for f in fs], K,
                                  _lib.PREC_BF16X3, ctypes.c_void_p(out.data_ptr()), stream)
    assert rc == _lib.BSK_OK, _lib.last_error()
    assert lib.bsk_sync_check(stream) == _lib.BSK_OK, _lib.last_error()


@pytest.mark.parametrize("num_fields", [1, 3])
def test_noalloc_matches_allocating_contract_twice(cuda, num_fields):
    kf = 2 * np.pi / 100.0
    kw = dict(kmin=kf, kmax=16 * kf, dk=2 * kf)
    edges = B.generate_bin_edge_list(**kw)
    tri = np.ascontiguousarray(B.generate_triangle_bin_list(num_fields=num_fields,
                                                            return_indices=True, **kw),
                               dtype=np.int32)
    n = len(edges)
    K = 40 ** 3
    g = torch.Generator(device="cuda")
    g.manual_seed(5)
    fs = [torch.randn((n, K), generator=g, device="cuda") for _ in range(3)]
    if num_fields == 1:
        fs = [fs[0]] * 3
    plan = Plan(64, 100.0, edges)
    ref = plan.contract(plan.triangles(tri), *fs, precision="bf16x3").cpu().numpy()
    lib = _lib.load()
    scale = np.abs(ref).max()
    for _ in range(2):
        out = torch.full((len(tri),), float("nan"), dtype=torch.float64, device="cuda")
        _call(lib, n, tri, fs, K, out)
        got = out.cpu().numpy()
        assert np.all(np.isfinite(got))
        # same kernel and per-entry arithmetic; only the FP64 atomics' order differs
        assert np.abs(got - ref).max() <= 1e-12 * scale


def test_noalloc_rejects_requests_beyond_the_static_area(cuda):
    lib = _lib.load()
    tri = np.array([[0, 0, 0]], dtype=np.int32)
    big = 20 * (1 << 20)  # 1 shell x 20M points needs 80 MB > 64 MiB
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    f = torch.zeros(8, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = lib.bsk_contract_noalloc(1, 1, tri.ctypes.data, *[ctypes.c_void_p(f.data_ptr())] * 3,
                                  big, _lib.PREC_BF16X3, ctypes.c_void_p(out.data_ptr()), stream)
    assert rc == _lib.BSK_ERR_ARG and "scratch" in _lib.last_error()
