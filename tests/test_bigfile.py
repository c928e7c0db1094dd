"""Bigfile grid reader (no GPU): files written here to the bigfile layout the reader
restates (header, attr-v2, hex-numbered data files), read back exactly.

No file written by the bigfile library itself exists here, so these tests pin the reader
to that restated layout, not to the library.
"""
import json
import os

import numpy as np
import pytest

from bskit_gb300 import BigFileMesh, as_mesh
from bskit_gb300.bigfile import read_block, read_block_attrs, read_block_header


def _hex(a):
    return np.ascontiguousarray(a).tobytes().hex().upper()


def write_block(path, dataset, data, attrs, nfile=1, nmemb=1):
    """Write ``data`` (rows) and ``attrs`` as one block in ``nfile`` data files."""
    block = os.path.join(path, dataset)
    os.makedirs(block)
    flat = np.ascontiguousarray(data).reshape(-1)
    rows = len(flat) // nmemb
    cuts = np.linspace(0, rows, nfile + 1).astype(int)
    lines = ["DTYPE: %s\n" % flat.dtype.str, "NMEMB: %d\n" % nmemb, "NFILE: %d\n" % nfile]
    for i in range(nfile):
        part = flat[cuts[i] * nmemb:cuts[i + 1] * nmemb]
        with open(os.path.join(block, "%06X" % i), "wb") as f:
            f.write(part.tobytes())
        s = int(np.frombuffer(part.tobytes(), np.uint8).astype(np.uint64).sum()) % 2 ** 32
        lines.append("%06X: %d : %d : %d\n" % (i, cuts[i + 1] - cuts[i], s, 0))
    with open(os.path.join(block, "header"), "w") as f:
        f.writelines(lines)
    with open(os.path.join(block, "attr-v2"), "w") as f:
        for name, value in attrs.items():
            if isinstance(value, str):
                raw = value.encode()
                f.write("%s S1 %d %s\n" % (name, len(raw), raw.hex().upper()))
            else:
                v = np.atleast_1d(value)
                f.write("%s %s %d %s\n" % (name, v.dtype.str, v.size, _hex(v)))
    return block


def _grid(n, seed=0):
    return np.random.default_rng(seed).standard_normal((n, n, n)).astype(np.float32)


def test_reads_a_saved_real_mesh(tmp_path):
    n = 16
    grid = _grid(n)
    attrs = {"Nmesh": np.array([n] * 3, np.int64), "BoxSize": np.array([250.0] * 3),
             "ndarray.shape": np.array([n] * 3, np.int64),
             "Omega0": np.array([0.3089]), "label": "z0",
             "extra": "json://" + json.dumps({"a": [1, 2]})}
    # three data files of unequal size: the rows concatenate in file order
    write_block(str(tmp_path), "Field", grid, attrs, nfile=3)
    mesh = BigFileMesh(str(tmp_path), "Field")
    assert np.array_equal(mesh.numpy(), grid)
    assert mesh.Nmesh == n
    assert np.array_equal(mesh.attrs["BoxSize"], [250.0] * 3)
    assert mesh.attrs["label"] == "z0" and mesh.attrs["extra"] == {"a": [1, 2]}
    assert np.allclose(mesh.attrs["Omega0"], 0.3089)
    # what FFTBispectrum's source handling accepts and checks
    assert as_mesh(mesh, Nmesh=n, BoxSize=250.0) is mesh
    with pytest.raises(ValueError):
        as_mesh(mesh, Nmesh=2 * n)


def test_float64_mesh_and_cic_option(tmp_path):
    n = 8
    grid = _grid(n, 1).astype(np.float64)
    write_block(str(tmp_path), "Field", grid,
                {"BoxSize": np.array([100.0]), "ndarray.shape": np.array([n] * 3, np.int64)})
    mesh = BigFileMesh(str(tmp_path), compensate_cic=32)
    assert mesh.numpy().dtype == np.float32
    assert np.array_equal(mesh.numpy(), grid.astype(np.float32))
    assert mesh.compensate_cic == 32 and np.array_equal(mesh.attrs["BoxSize"], [100.0] * 3)


def test_block_reader_rows_and_members(tmp_path):
    pos = np.arange(30, dtype=np.float32).reshape(10, 3)
    block = write_block(str(tmp_path), "Position", pos, {}, nfile=2, nmemb=3)
    dtype, nmemb, rows = read_block_header(block)
    assert dtype == np.float32 and nmemb == 3 and rows == [5, 5]
    assert np.array_equal(read_block(block), pos)
    out = np.empty((10, 3), np.float32)
    assert read_block(block, out=out) is not None and np.array_equal(out, pos)
    assert read_block_attrs(block) == {}


def test_rejects_what_is_not_a_real_mesh(tmp_path):
    n = 8
    shape = np.array([n] * 3, np.int64)
    root = str(tmp_path)
    write_block(root, "NoShape", _grid(n), {"BoxSize": np.array([1.0])})
    write_block(root, "Complex", np.zeros(n ** 3, np.complex64),
                {"BoxSize": np.array([1.0]), "ndarray.shape": shape})
    write_block(root, "Short", _grid(n).reshape(-1)[:100],
                {"BoxSize": np.array([1.0]), "ndarray.shape": shape})
    for name in ("NoShape", "Complex", "Short", "Missing"):
        with pytest.raises(ValueError):
            BigFileMesh(root, name)
    # a data file whose size disagrees with its header line
    block = write_block(root, "Truncated", _grid(n),
                        {"BoxSize": np.array([1.0]), "ndarray.shape": shape})
    with open(os.path.join(block, "000000"), "r+b") as f:
        f.truncate(40)
    with pytest.raises(ValueError):
        BigFileMesh(root, "Truncated")
