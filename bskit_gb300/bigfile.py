"""Real-space density grids stored in the bigfile format, the input of bskit's scripts.

bskit's measurement scripts read their grids with nbodykit's
``BigFileMesh(path, 'Field')`` (scripts/measure/measure_bs_fast.py:218-223,
scripts/measure/measure_subbox_bs_fast.py:235), grids that its conversion scripts wrote
with ``mesh.save(path, dataset='Field', mode='real')``
(scripts/grids/convert_npygrid_to_bigfile.py:56,
scripts/grids/convert_illustris_hdf5_particles_to_bigfile_grid.py:109).
``BigFileMesh`` here reads such a grid into an ``ArrayMesh`` (host memory, float32), which
``FFTBispectrum`` and ``SubboxBispectrum`` take as their source.

The layout is the bigfile library's (rainwoodman/bigfile, not part of bskit, absent here
and unpinned by bskit), restated:

* a file is a directory and a block (``Field``) a sub-directory of it, holding
  - ``header``: the lines ``DTYPE: <numpy dtype, e.g. <f4>``, ``NMEMB: <members per row>``,
    ``NFILE: <number of data files>``, then one line per data file,
    ``<index, 6 hex digits>: <rows> : <checksum> : <checksum>``;
  - ``attr-v2``: one attribute per line, ``<name> <numpy dtype> <count> <hex bytes>``,
    the value's raw bytes written as two hex digits each (strings as dtype ``S1``);
  - the data files, named by their index in 6 upper-case hex digits (``000000``, ...):
    raw rows, which concatenated in index order form the block;
* nbodykit's ``save(mode='real')`` stores the real field flattened in C order with the
  attributes ``Nmesh``, ``BoxSize`` and ``ndarray.shape``, and its ``BigFileMesh`` takes
  the mesh shape from ``ndarray.shape``; string attributes that start with ``json://``
  hold JSON.

The per-file checksums are not verified.  No file written by the bigfile library itself is
available here, so this reader is checked only against files written to the layout above.
"""
import json
import os
import re

import numpy as np

from .mesh import ArrayMesh

_FILE_LINE = re.compile(r"^([0-9A-Fa-f]+)\s*:\s*(\d+)\s*:\s*(\d+)\s*:\s*(\d+)\s*$")


def read_block_header(block_dir):
    """(dtype, nmemb, [rows per data file]) of a block directory."""
    path = os.path.join(block_dir, "header")
    if not os.path.isfile(path):
        raise ValueError("%s is not a bigfile block (no header)" % block_dir)
    fields, rows = {}, {}
    with open(path) as f:
        for line in f:
            line = line.strip()
            if not line:
                continue
            m = _FILE_LINE.match(line)
            if m:
                rows[int(m.group(1), 16)] = int(m.group(2))
                continue
            key, sep, value = line.partition(":")
            if not sep:
                raise ValueError("bad header line %r in %s" % (line, path))
            fields[key.strip()] = value.strip()
    try:
        dtype = np.dtype(fields["DTYPE"])
        nmemb = int(fields["NMEMB"])
        nfile = int(fields["NFILE"])
    except (KeyError, TypeError, ValueError) as e:
        raise ValueError("bad bigfile header %s: %s" % (path, e))
    if sorted(rows) != list(range(nfile)):
        raise ValueError("header %s lists data files %s, expected 0..%d" %
                         (path, sorted(rows), nfile - 1))
    return dtype, nmemb, [rows[i] for i in range(nfile)]


def _attr_value(dtype, count, hexdata):
    raw = bytes.fromhex(hexdata) if hexdata else b""
    dt = np.dtype(dtype)
    if len(raw) != count * dt.itemsize:
        raise ValueError("attribute holds %d bytes, expected %d x %d" % (len(raw), count,
                                                                         dt.itemsize))
    if dt.kind == "S":
        s = raw.decode("utf-8", errors="replace")
        return json.loads(s[len("json://"):]) if s.startswith("json://") else s
    return np.frombuffer(raw, dtype=dt).copy()


def read_block_attrs(block_dir):
    """The attribute dictionary of a block (``attr-v2``); empty when the block has none."""
    path = os.path.join(block_dir, "attr-v2")
    attrs = {}
    if not os.path.isfile(path):
        return attrs
    with open(path) as f:
        for line in f:
            parts = line.split()
            if not parts:
                continue
            if len(parts) not in (3, 4):
                raise ValueError("bad attribute line %r in %s" % (line.strip(), path))
            name, dtype, count = parts[0], parts[1], int(parts[2])
            attrs[name] = _attr_value(dtype, count, parts[3] if len(parts) == 4 else "")
    return attrs


def read_block(block_dir, out=None):
    """The rows of a block as one array (shape (rows,) or (rows, nmemb)).

    ``out``: an optional preallocated array of that size and dtype (e.g. a pinned host
    buffer's numpy view) to read into."""
    dtype, nmemb, rows = read_block_header(block_dir)
    total = sum(rows)
    shape = (total,) if nmemb == 1 else (total, nmemb)
    if out is None:
        out = np.empty(shape, dtype=dtype)
    elif out.dtype != dtype or out.size != total * nmemb or not out.flags.c_contiguous:
        raise ValueError("out must be a C-contiguous %s array of %d elements" %
                         (dtype, total * nmemb))
    flat = out.reshape(-1)
    pos = 0
    for i, n in enumerate(rows):
        path = os.path.join(block_dir, "%06X" % i)
        want = n * nmemb * dtype.itemsize
        have = os.path.getsize(path) if os.path.isfile(path) else -1
        if have != want:
            raise ValueError("data file %s holds %d bytes, the header says %d" %
                             (path, have, want))
        with open(path, "rb") as f:
            got = f.readinto(memoryview(flat[pos:pos + n * nmemb]).cast("B"))
        if got != want:
            raise ValueError("short read of %s (%d of %d bytes)" % (path, got, want))
        pos += n * nmemb
    return out.reshape(shape)


class BigFileMesh(ArrayMesh):
    """A real N^3 grid read from ``path``/``dataset`` (nbodykit's ``BigFileMesh``).

    ``attrs`` holds the block's attributes (``Nmesh``, ``BoxSize``, ``ndarray.shape`` and
    whatever else was saved) with ``Nmesh`` and ``BoxSize`` as three-vectors.
    ``compensate_cic``: as for ``ArrayMesh`` (the scripts' CIC correction of a bigfile grid,
    scripts/measure/measure_bs_fast.py:220-222).
    """

    def __init__(self, path, dataset="Field", compensate_cic=None):
        block = os.path.join(path, dataset)
        attrs = read_block_attrs(block)
        if "ndarray.shape" not in attrs:
            raise ValueError("%s has no ndarray.shape attribute: it does not hold a mesh "
                             "saved by mesh.save()" % block)
        shape = tuple(int(v) for v in np.atleast_1d(attrs["ndarray.shape"]))
        if len(shape) != 3 or len(set(shape)) != 1:
            raise ValueError("mesh shape %s is not a cube" % (shape,))
        if "BoxSize" not in attrs:
            raise ValueError("%s has no BoxSize attribute" % block)
        dtype, nmemb, rows = read_block_header(block)
        if dtype.kind == "c":
            raise ValueError("%s holds a complex (mode='complex') field; bskit's grids are "
                             "saved with mode='real'" % block)
        if dtype.kind != "f" or nmemb != 1 or sum(rows) != int(np.prod(shape)):
            raise ValueError("%s holds %d rows of %d x %s, not a real %s mesh" %
                             (block, sum(rows), nmemb, dtype, shape))
        data = read_block(block).reshape(shape)
        ArrayMesh.__init__(self, data, attrs["BoxSize"], compensate_cic=compensate_cic)
        for key, value in attrs.items():
            if key not in ("Nmesh", "BoxSize"):
                self.attrs[key] = value
        self.path = path
        self.dataset = dataset
