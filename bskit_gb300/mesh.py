"""Mesh sources accepted by ``FFTBispectrum``.

bskit takes nbodykit ``MeshSource`` objects and paints them on an MPI-decomposed
pmesh grid.  Here a source is a real N^3 density mesh held as a numpy array or a
torch tensor (host or device) together with its box size; any object with an
``attrs`` dict (``BoxSize``, ``Nmesh``) and a ``paint(mode='real')`` method
(the nbodykit MeshSource interface) is accepted too and painted once.
"""
import numpy as np
import torch


class ArrayMesh(object):
    """A real density mesh ``array`` (N^3) in a periodic cube of side ``BoxSize``.

    ``compensate_cic``: NmeshCIC of the grid the particles were CIC-assigned on;
    the CIC window is then deconvolved when the mesh is painted (the
    ``CompensateCICShotnoiseNgrid`` action of scripts/measure/measure_bs_fast.py:45-57).
    """

    def __init__(self, array, BoxSize, compensate_cic=None):
        if isinstance(array, torch.Tensor):
            if array.dim() != 3 or len(set(array.shape)) != 1:
                raise ValueError("mesh must be a cubic N^3 array")
            self._t = array
            self._np = None
            n = array.shape[0]
        else:
            a = np.asarray(array)
            if a.ndim != 3 or len(set(a.shape)) != 1:
                raise ValueError("mesh must be a cubic N^3 array")
            if np.iscomplexobj(a):
                raise ValueError("mesh must be real")
            self._np = np.ascontiguousarray(a, dtype=np.float32)
            self._t = None
            n = a.shape[0]
        box = np.atleast_1d(np.asarray(BoxSize, dtype=np.float64))
        if box.size == 1:
            box = np.repeat(box, 3)
        self.attrs = {'Nmesh': np.array([n] * 3), 'BoxSize': box}
        self.compensate_cic = int(compensate_cic) if compensate_cic else None
        self._cache = {}

    @property
    def Nmesh(self):
        return int(self.attrs['Nmesh'][0])

    def tensor(self, device):
        """float32 contiguous tensor on ``device`` (cached)."""
        key = str(device)
        t = self._cache.get(key)
        if t is None:
            src = self._t if self._t is not None else torch.from_numpy(self._np)
            t = src.to(device=device, dtype=torch.float32).contiguous()
            self._cache[key] = t
        return t

    def numpy(self):
        if self._np is not None:
            return self._np
        return self._t.detach().to("cpu", torch.float32).numpy()


def as_mesh(source, Nmesh=None, BoxSize=None):
    """Wrap ``source`` as an ``ArrayMesh`` and check it against Nmesh / BoxSize."""
    if isinstance(source, ArrayMesh):
        mesh = source
    elif isinstance(source, (np.ndarray, torch.Tensor)):
        if BoxSize is None:
            raise ValueError("BoxSize is required when the source is a bare array")
        mesh = ArrayMesh(source, BoxSize)
    elif hasattr(source, "attrs") and hasattr(source, "paint"):
        field = source.paint(mode='real')
        mesh = ArrayMesh(np.asarray(field[...] if hasattr(field, "__getitem__") else field),
                         source.attrs['BoxSize'] if BoxSize is None else BoxSize)
    else:
        raise TypeError("unsupported mesh source %r" % type(source))
    if Nmesh is not None:
        nm = np.atleast_1d(np.asarray(Nmesh))
        if not np.all(nm == mesh.attrs['Nmesh'][0]):
            raise ValueError("Nmesh %s differs from the mesh size %d (resampling is not "
                             "supported)" % (Nmesh, mesh.attrs['Nmesh'][0]))
    if BoxSize is not None:
        bs = np.atleast_1d(np.asarray(BoxSize, dtype=np.float64))
        if not np.allclose(bs, mesh.attrs['BoxSize'][0], rtol=0, atol=0):
            raise ValueError("BoxSize %s differs from the mesh's %s" % (BoxSize,
                                                                        mesh.attrs['BoxSize']))
    return mesh
