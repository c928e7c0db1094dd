"""Thin object layer over the C ABI (plans, triangle sets, device buffers).

Tensors are torch CUDA tensors; every call is enqueued on the current torch
stream of the plan's device.  Nothing here computes on the CPU.
"""
import ctypes
import weakref

import numpy as np
import torch

from . import _lib

GRID_MODES = {"reduced": _lib.GRID_REDUCED, "native": _lib.GRID_NATIVE,
              "single": _lib.GRID_REDUCED_SINGLE}


def _stream_ptr(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def _require_cuda():
    if not torch.cuda.is_available():
        raise RuntimeError("bskit_gb300 computes on a CUDA device only (none is available)")


def _check_tensor(t, what, shape, dtype, device):
    """A device buffer handed to the C ABI as a raw pointer: the kernels trust its size, so
    the shape, dtype, device and layout are checked here."""
    if (not isinstance(t, torch.Tensor) or tuple(t.shape) != tuple(shape) or t.dtype != dtype
            or t.device != device or not t.is_contiguous()):
        raise ValueError("%s must be a contiguous %s tensor of shape %s on %s" %
                         (what, dtype, tuple(shape), device))


class TriangleSet:
    """A registered list of (i, j, l) shell-index triples (``k_indices`` rows)."""

    def __init__(self, plan, tri):
        tri = np.ascontiguousarray(np.asarray(tri, dtype=np.int32).reshape(-1, 3))
        self.plan = plan
        self.indices = tri
        self.T = len(tri)
        h = ctypes.c_void_p()
        with torch.cuda.device(plan.device):
            _lib.call("bsk_triset_create", plan.handle, self.T,
                      tri.ctypes.data if self.T else None, ctypes.byref(h))
        self.handle = h
        plan._sets.add(self)

    def schedule(self):
        """(tiles, sum of tile column counts, pair rows) of the contraction schedule."""
        out = (ctypes.c_int64 * 3)()
        _lib.call("bsk_triset_schedule", self.handle, out)
        return int(out[0]), int(out[1]), int(out[2])

    def levels(self):
        """The grid levels of the set's resident contraction: one dict per level with the
        grid side, tiles, sum of tile columns, pair rows, bins and shells synthesised (empty
        when every bin is contracted on the plan's grid)."""
        n = _lib.load().bsk_triset_levels(self.handle, None, 0)
        if n < 0:
            raise _lib.BskError(n, _lib.last_error())
        out = (ctypes.c_int64 * (6 * max(n, 1)))()
        _lib.load().bsk_triset_levels(self.handle, out, n)
        keys = ("ngrid", "tiles", "sum_nc", "pair_rows", "bins", "shells")
        return [dict(zip(keys, (int(v) for v in out[6 * k:6 * k + 6]))) for k in range(n)]

    def close(self):
        if getattr(self, "handle", None):
            with torch.cuda.device(self.plan.device):
                _lib.load().bsk_triset_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Plan:
    """Engine state for one (Nmesh, BoxSize, shell list) on one device.

    ``grid='reduced'`` contracts on the smallest FFT-friendly grid Ng > 3 q_max, and the bins
    of small shells on smaller grids (identical sums, see ``bsk_plan_create`` and
    ``bsk_triset_levels``); ``grid='single'`` keeps every bin on that one reduced grid;
    ``grid='native'`` uses Ng = Nmesh.
    """

    def __init__(self, nmesh, box_size, shell_edges, grid="reduced", mem_budget=0, device=None):
        _require_cuda()
        self._sets = weakref.WeakSet()
        idx = None if device is None else torch.device(device).index
        self.device = torch.device("cuda", torch.cuda.current_device() if idx is None else idx)
        edges = np.ascontiguousarray(np.asarray(shell_edges, dtype=np.float64).reshape(-1, 2))
        self.shell_edges = edges
        self.nmesh = int(nmesh)
        self.box_size = float(box_size)
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.call("bsk_plan_create", self.nmesh, self.box_size, len(edges), edges.ctypes.data,
                      GRID_MODES[grid], int(mem_budget), ctypes.byref(h))
        self.handle = h
        info = (ctypes.c_int64 * _lib.INFO_COUNT)()
        _lib.call("bsk_plan_query", self.handle, info)
        self.ngrid = int(info[_lib.INFO_NGRID])
        self.qmax = int(info[_lib.INFO_QMAX])
        self.n_shells = len(edges)

    # ------------------------------------------------------------------ info
    def footprint(self):
        info = (ctypes.c_int64 * _lib.INFO_COUNT)()
        _lib.call("bsk_plan_query", self.handle, info)
        return int(info[_lib.INFO_FOOTPRINT])

    def stream_chunk(self):
        """Shells per chunk of the last measurement's shell streaming (0 = fields resident)."""
        info = (ctypes.c_int64 * _lib.INFO_COUNT)()
        _lib.call("bsk_plan_query", self.handle, info)
        return int(info[_lib.INFO_STREAM])

    def mode_counts(self):
        out = np.zeros(self.n_shells, dtype=np.int64)
        _lib.call("bsk_shell_mode_counts", self.handle, out.ctypes.data)
        return out

    def triangles(self, tri):
        return TriangleSet(self, tri)

    # ------------------------------------------------------------------ compute
    def paint(self, slot, mesh, stream=None, cic_nmesh=None):
        """r2c of a real N^3 float32 CUDA tensor into field slot 0/1/2.

        cic_nmesh: deconvolve the CIC window of a mesh assigned on a cic_nmesh^3 grid."""
        m = self._as_mesh(mesh)
        with torch.cuda.device(self.device):
            if cic_nmesh:
                _lib.call("bsk_paint_cic", self.handle, int(slot), ctypes.c_void_p(m.data_ptr()),
                          int(cic_nmesh), _stream_ptr(stream))
            else:
                _lib.call("bsk_paint", self.handle, int(slot), ctypes.c_void_p(m.data_ptr()),
                          _stream_ptr(stream))
        return m

    def paint_subbox(self, slot, mesh, multi, stream=None):
        """r2c of the sub-box multi = (a, b, c) of a larger cubic float32 CUDA mesh whose side
        is a multiple of this plan's Nmesh (the block starting at (a N, b N, c N))."""
        m = self._as_mesh(mesh, full=True)
        a, b, c = (int(v) for v in multi)
        with torch.cuda.device(self.device):
            _lib.call("bsk_paint_subbox", self.handle, int(slot), ctypes.c_void_p(m.data_ptr()),
                      int(m.shape[0]), a, b, c, _stream_ptr(stream))
        return m

    def measure_b(self, tset, slots=(0, 0, 0), precision="bf16x3", out=None, stream=None):
        """Unnormalised bispectrum (float64 CUDA tensor of length T)."""
        prec = _lib.PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        if out is None:
            out = torch.empty(tset.T, dtype=torch.float64, device=self.device)
        _check_tensor(out, "out", (tset.T,), torch.float64, self.device)
        with torch.cuda.device(self.device):
            _lib.call("bsk_measure_b", self.handle, tset.handle, int(slots[0]), int(slots[1]),
                      int(slots[2]), prec, ctypes.c_void_p(out.data_ptr()), _stream_ptr(stream))
        return out

    def measure_b_range(self, tset, k_begin, k_end, slots=(0, 0, 0), precision="bf16x3",
                        out=None, stream=None):
        """Partial unnormalised B over contraction-grid points [k_begin, k_end)."""
        prec = _lib.PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        if out is None:
            out = torch.empty(tset.T, dtype=torch.float64, device=self.device)
        _check_tensor(out, "out", (tset.T,), torch.float64, self.device)
        with torch.cuda.device(self.device):
            _lib.call("bsk_measure_b_range", self.handle, tset.handle, int(slots[0]),
                      int(slots[1]), int(slots[2]), prec, int(k_begin), int(k_end),
                      ctypes.c_void_p(out.data_ptr()), _stream_ptr(stream))
        return out

    def gridinfo(self, tset, stream=None):
        """(N_tri (T,), k_mean (T, 3)) float64 CUDA tensors; k_mean NaN where N_tri == 0."""
        ntri = torch.empty(tset.T, dtype=torch.float64, device=self.device)
        kmean = torch.empty((tset.T, 3), dtype=torch.float64, device=self.device)
        with torch.cuda.device(self.device):
            _lib.call("bsk_gridinfo", self.handle, tset.handle, ctypes.c_void_p(ntri.data_ptr()),
                      ctypes.c_void_p(kmean.data_ptr()), _stream_ptr(stream))
        return ntri, kmean

    def contract(self, tset, f1, f2, f3, precision="bf16x3", stream=None):
        """Raw contraction of caller fields ([n][K] float32 CUDA): sum_k f1 f2 f3."""
        prec = _lib.PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        fs = [f.contiguous() for f in (f1, f2, f3)]
        if fs[0].dim() != 2:
            raise ValueError("fields must be float32 CUDA tensors of shape (n_shells, K)")
        K = fs[0].shape[1]
        for i, f in enumerate(fs):
            _check_tensor(f, "f%d" % (i + 1), (self.n_shells, K), torch.float32, self.device)
        out = torch.empty(tset.T, dtype=torch.float64, device=self.device)
        with torch.cuda.device(self.device):
            _lib.call("bsk_contract", self.handle, tset.handle, *[ctypes.c_void_p(f.data_ptr())
                                                                  for f in fs],
                      int(K), prec, ctypes.c_void_p(out.data_ptr()), _stream_ptr(stream))
        return out

    def field(self, slot, shell, stream=None):
        """FP32 real-space field of one shell on the contraction grid (Ng^3)."""
        out = torch.empty((self.ngrid,) * 3, dtype=torch.float32, device=self.device)
        with torch.cuda.device(self.device):
            _lib.call("bsk_copy_field", self.handle, int(slot), int(shell),
                      ctypes.c_void_p(out.data_ptr()), _stream_ptr(stream))
        return out

    def sync_check(self, stream=None):
        with torch.cuda.device(self.device):
            _lib.call("bsk_sync_check", _stream_ptr(stream))

    @staticmethod
    def normalize(b_unnorm, ntri, stream=None):
        """b_unnorm / ntri (float64 CUDA tensors of one length T)."""
        if not isinstance(b_unnorm, torch.Tensor) or not b_unnorm.is_cuda:
            raise ValueError("b_unnorm must be a float64 CUDA tensor")
        dev, T = b_unnorm.device, b_unnorm.numel()
        _check_tensor(b_unnorm, "b_unnorm", (T,), torch.float64, dev)
        _check_tensor(ntri, "ntri", (T,), torch.float64, dev)
        out = torch.empty_like(b_unnorm)
        with torch.cuda.device(dev):
            _lib.call("bsk_normalize", int(b_unnorm.numel()), ctypes.c_void_p(b_unnorm.data_ptr()),
                      ctypes.c_void_p(ntri.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                      _stream_ptr(stream))
        return out

    # ------------------------------------------------------------------ helpers
    def _as_mesh(self, mesh, full=False):
        if isinstance(mesh, np.ndarray):
            mesh = torch.from_numpy(np.ascontiguousarray(mesh, dtype=np.float32))
        if not isinstance(mesh, torch.Tensor):
            raise TypeError("mesh must be a numpy array or torch tensor")
        if full:
            n = mesh.shape[0] if mesh.dim() == 3 else -1
            if mesh.dim() != 3 or len(set(mesh.shape)) != 1 or n % self.nmesh:
                raise ValueError("mesh shape %s is not a cube whose side is a multiple of "
                                 "Nmesh=%d" % (tuple(mesh.shape), self.nmesh))
        elif tuple(mesh.shape) != (self.nmesh,) * 3:
            raise ValueError("mesh shape %s does not match Nmesh=%d" % (tuple(mesh.shape),
                                                                          self.nmesh))
        return mesh.to(device=self.device, dtype=torch.float32).contiguous()

    def close(self):
        if getattr(self, "handle", None):
            for ts in list(self._sets):
                ts.close()
            with torch.cuda.device(self.device):
                _lib.load().bsk_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def compensate_cic(mesh, nmesh_cic, out=None, stream=None):
    """CIC window deconvolution of a whole cubic float32 CUDA mesh assigned on an
    nmesh_cic^3 grid (returns ``out``, a new tensor unless given; may be ``mesh``)."""
    _require_cuda()
    if not isinstance(mesh, torch.Tensor) or mesh.dim() != 3 or len(set(mesh.shape)) != 1:
        raise ValueError("mesh must be a cubic torch tensor")
    m = mesh.to(dtype=torch.float32).contiguous()
    if not m.is_cuda:
        m = m.cuda()
    if out is None:
        out = torch.empty_like(m)
    _check_tensor(out, "out", tuple(m.shape), torch.float32, m.device)
    with torch.cuda.device(m.device):
        _lib.call("bsk_compensate_cic", int(m.shape[0]), int(nmesh_cic),
                  ctypes.c_void_p(m.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                  _stream_ptr(stream))
    return out
