"""bsk_contract_noalloc: the allocation-free tensor-core contraction.

It exists for callers that cannot call cudaMalloc when they need a result (a
framework that reserved the device memory up front, or a hot path on which
cudaMalloc/cudaFree are forbidden because they synchronise and can fail).
Its scratch is a 64 MiB static device array of the library.  The tests call
it through the C ABI and compare with the allocating entry point bsk_contract
(twice in a row, then a smaller request with other shells and triangles, so
that stale contents of the shared array would show) and with the FP64
contraction of the same fields at the bf16x3 error bound.  This file is named
so that pytest collects it last.
"""
import ctypes

import numpy as np
import pytest
import torch

from bskit_gb300 import _lib
from bskit_gb300 import bins as B
from bskit_gb300.engine import Plan

pytestmark = pytest.mark.gpu

# bf16x3 bound of the parity tests: |B - B_fp64| <= 4e-6 * sum |f1 f2 f3| per bin
BF16X3_NORMALISED = 4e-6


def _call(lib, n_shells, tri, fs, K, out, stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    sp = ctypes.c_void_p(s.cuda_stream)
    return lib.bsk_contract_noalloc(n_shells, len(tri), tri.ctypes.data,
                                    *[ctypes.c_void_p(f.data_ptr()) for f in fs], K,
                                    _lib.PREC_BF16X3, ctypes.c_void_p(out.data_ptr()), sp)


def _run(lib, n_shells, tri, fs, K):
    out = torch.full((len(tri),), float("nan"), dtype=torch.float64, device="cuda")
    rc = _call(lib, n_shells, tri, fs, K, out)
    assert rc == _lib.BSK_OK, _lib.last_error()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert lib.bsk_sync_check(stream) == _lib.BSK_OK, _lib.last_error()
    got = out.cpu().numpy()
    assert np.all(np.isfinite(got))
    return got


def _case(kmax_kf, num_fields, n_points, seed):
    kf = 2 * np.pi / 100.0
    kw = dict(kmin=kf, kmax=kmax_kf * kf, dk=2 * kf)
    edges = B.generate_bin_edge_list(**kw)
    tri = np.ascontiguousarray(B.generate_triangle_bin_list(num_fields=num_fields,
                                                            return_indices=True, **kw),
                               dtype=np.int32)
    n = len(edges)
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    fs = [torch.randn((n, n_points), generator=g, device="cuda") for _ in range(3)]
    if num_fields == 1:
        fs = [fs[0]] * 3
    return edges, tri, fs


@pytest.mark.parametrize("num_fields", [1, 3])
def test_noalloc_matches_allocating_contract_twice(cuda, num_fields):
    K = 40 ** 3
    edges, tri, fs = _case(16, num_fields, K, 5)
    n = len(edges)
    plan = Plan(64, 100.0, edges)
    ts = plan.triangles(tri)
    ref = plan.contract(ts, *fs, precision="bf16x3").cpu().numpy()
    b64 = plan.contract(ts, *fs, precision="fp64").cpu().numpy()
    absf = [f.abs() for f in fs]
    babs = plan.contract(ts, *absf, precision="fp64").cpu().numpy()
    lib = _lib.load()
    scale = np.abs(ref).max()
    for _ in range(2):
        got = _run(lib, n, tri, fs, K)
        # same kernel and per-entry arithmetic; only the FP64 atomics' order differs
        assert np.abs(got - ref).max() <= 1e-12 * scale
        # and within the bf16x3 bound of the FP64 contraction of the same fields
        assert np.all(np.abs(got - b64) <= BF16X3_NORMALISED * babs)

    # a smaller request with other shells and triangles after the larger one: every
    # schedule entry and split value it reads must be its own, not the last call's
    K2 = 24 ** 3
    edges2, tri2, fs2 = _case(10, 2, K2, 9)
    plan2 = Plan(64, 100.0, edges2)
    ref2 = plan2.contract(plan2.triangles(tri2), *fs2, precision="bf16x3").cpu().numpy()
    got2 = _run(lib, len(edges2), tri2, fs2, K2)
    assert np.abs(got2 - ref2).max() <= 1e-12 * np.abs(ref2).max()


def test_noalloc_allocates_no_device_memory(cuda):
    K = 32 ** 3
    edges, tri, fs = _case(12, 1, K, 3)
    lib = _lib.load()
    out = torch.zeros(len(tri), dtype=torch.float64, device="cuda")
    assert _call(lib, len(edges), tri, fs, K, out) == _lib.BSK_OK  # warm-up: module, address
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        assert _call(lib, len(edges), tri, fs, K, out) == _lib.BSK_OK, _lib.last_error()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


def test_noalloc_rejects_a_capturing_stream(cuda):
    K = 16 ** 3
    edges, tri, fs = _case(8, 1, K, 4)
    lib = _lib.load()
    out = torch.zeros(len(tri), dtype=torch.float64, device="cuda")
    assert _call(lib, len(edges), tri, fs, K, out) == _lib.BSK_OK  # outside capture: fine
    torch.cuda.synchronize()
    side = torch.cuda.Stream()
    graph = torch.cuda.CUDAGraph()
    rc = None
    with torch.cuda.graph(graph, stream=side):
        rc = _call(lib, len(edges), tri, fs, K, out, stream=side)
        torch.zeros(1, device="cuda")  # one captured node so that the graph is not empty
    assert rc == _lib.BSK_ERR_STATE
    assert "capture" in _lib.last_error()
    # the rejected call left the stream and the context usable
    assert _call(lib, len(edges), tri, fs, K, out) == _lib.BSK_OK, _lib.last_error()
    torch.cuda.synchronize()


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
