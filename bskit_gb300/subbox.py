"""Sub-box bispectra: bskit's error-bar workflow as one batched request.

bskit cuts each sub-box out of the full field with ``field_subbox_pm``
(bskit/main.py:83-147: a nearest-grid-point readout of the sub-region, i.e. an
array slice), builds one ``FFTBispectrum`` per sub-box and measures it
(scripts/measure/measure_subbox_bs_fast.py:253-295), writing one file per
sub-box.  Here every sub-box of a request shares one engine plan (Nmesh/nsub,
BoxSize/nsub and the binning) and one triangle set; each sub-box is transformed
where it lies in the full device mesh (``bsk_paint_subbox``, no copy), and the
grid information, which depends only on the binning, is computed once for all.
A CIC compensation, when the mesh asks for one, is applied to the full mesh
before the cut (as measure_subbox_bs_fast.py:236-246 does).
"""
import numpy as np
import torch

from .bispectrum import FFTBispectrum
from .engine import compensate_cic
from .mesh import ArrayMesh, as_mesh


def subbox_index_to_multiindex(i, nsub_per_side):
    """(a, b, c) with i = a*n^2 + b*n + c, n = nsub_per_side, as a float array
    (bskit/main.py:54-80)."""
    a, r = divmod(int(i), nsub_per_side ** 2)
    b, c = divmod(r, nsub_per_side)
    return np.array([a, b, c], dtype=np.float64)


def field_subbox(box_multiindex, nsub_per_side, source):
    """The sub-region of ``source`` with origin box_multiindex * Lsub, Lsub =
    BoxSize / nsub_per_side, as an ``ArrayMesh`` of side Nmesh / nsub_per_side
    (bskit/main.py:83-147; nearest-grid-point readout = the array slice)."""
    mesh = as_mesh(source)
    n_full = mesh.Nmesh
    if n_full % nsub_per_side:
        raise ValueError("Nmesh %d is not divisible by nsub_per_side %d" % (n_full, nsub_per_side))
    n = n_full // nsub_per_side
    a, b, c = (int(v) * n for v in box_multiindex)
    src = mesh._t if mesh._t is not None else mesh.numpy()
    block = src[a:a + n, b:b + n, c:c + n]
    block = block.contiguous() if isinstance(block, torch.Tensor) else np.ascontiguousarray(block)
    return ArrayMesh(block, mesh.attrs['BoxSize'] / nsub_per_side)


class SubboxBispectrum(object):
    """Bispectra of the sub-boxes of one snapshot (auto, <AAB> or <ABC>).

    source, second, third : full meshes (``ArrayMesh``, or cubic arrays with
        ``BoxSize``); ``compensate_cic`` on the first mesh applies to all.
    nsub_per_side : sub-boxes per side; each has Nmesh/nsub points and side
        BoxSize/nsub.
    The binning keywords are ``FFTBispectrum``'s, in the sub-box's k units.
    """

    def __init__(self, source, nsub_per_side, BoxSize=None, dk=None, kmin=None, kmax=None,
                 num_lowk_bins=0, dk_high=-1., pos_units_mpcoverh=1., second=None, third=None,
                 triangle_type='all', isos_mult=0, isos_tol=0.1, squeezed_bin_index=0,
                 precision='bf16x3', grid='reduced', device=None, mem_budget=0):
        self.full = [as_mesh(m, BoxSize=BoxSize) if m is not None else None
                     for m in (source, second, third)]
        self.full = [m for m in self.full if m is not None]
        self.nsub = int(nsub_per_side)
        n_full = self.full[0].Nmesh
        for m in self.full[1:]:
            if m.Nmesh != n_full or not np.array_equal(m.attrs['BoxSize'],
                                                       self.full[0].attrs['BoxSize']):
                raise ValueError("all meshes must share Nmesh and BoxSize")
        if n_full % self.nsub:
            raise ValueError("Nmesh %d is not divisible by nsub_per_side %d"
                             % (n_full, self.nsub))
        self.n = n_full // self.nsub
        self.box = self.full[0].attrs['BoxSize'] / self.nsub
        # binning and plan of one sub-box (a placeholder mesh of the sub-box's shape:
        # nothing is painted from it)
        first = ArrayMesh(torch.empty((self.n,) * 3, dtype=torch.float32), self.box)
        subs = [first] * len(self.full)
        self.fb = FFTBispectrum(subs[0], Nmesh=self.n, BoxSize=self.box, dk=dk, kmin=kmin,
                                kmax=kmax, num_lowk_bins=num_lowk_bins, dk_high=dk_high,
                                pos_units_mpcoverh=pos_units_mpcoverh,
                                second=subs[1] if len(subs) > 1 else None,
                                third=subs[2] if len(subs) > 2 else None,
                                triangle_type=triangle_type, isos_mult=isos_mult,
                                isos_tol=isos_tol, squeezed_bin_index=squeezed_bin_index,
                                for_grid_info_only=True, precision=precision, grid=grid,
                                device=device, mem_budget=mem_budget)
        self._dev_full = None

    @property
    def k_edges(self):
        return self.fb.k_edges

    @property
    def k_indices(self):
        return self.fb.k_indices

    def _device_meshes(self, device):
        """Full meshes on the device, CIC-compensated once when asked for."""
        if self._dev_full is None:
            out = []
            for m in self.full:
                t = m.tensor(device)
                if m.compensate_cic:
                    t = compensate_cic(t, m.compensate_cic)
                out.append(t)
            self._dev_full = out
        return self._dev_full

    def measure(self, subboxes=None, imin=None, imax=None, meas_type='unnorm_b_value',
                out_file_prefix=None):
        """Measure sub-boxes (indices, default all nsub^3) over bins imin..imax-1.

        meas_type 'unnorm_b_value': unnormalised B per sub-box (the rows of
        measure_bispectrum_faster); 'grid_info': triangle counts and mean |k|
        (the rows of measure_gridinfo_faster, identical for every sub-box);
        'full': both and B normalised by the counts.  Returns {index: dict with
        'index', 'k_edge', 'k_mean', 'B', 'N_tri'}; with out_file_prefix, writes
        '<prefix>_subbox<i>.dat' per sub-box as the reference script does.
        """
        if meas_type not in ('unnorm_b_value', 'grid_info', 'full'):
            raise ValueError("meas_type must be 'unnorm_b_value', 'grid_info' or 'full'")
        if subboxes is None:
            subboxes = range(self.nsub ** 3)
        subboxes = [int(i) for i in subboxes]
        for i in subboxes:
            if not 0 <= i < self.nsub ** 3:
                raise ValueError("sub-box index %d outside [0, %d)" % (i, self.nsub ** 3))
        fb = self.fb
        i0, i1 = fb._range(imin, imax, len(fb.k_indices))
        edges = np.asarray(fb.k_edges[i0:i1])
        triples = np.asarray(fb.k_indices[i0:i1])
        index = np.arange(i0, i1)
        plan = fb._plan(fb._shell_edges())
        tset = plan.triangles(triples) if len(triples) else None
        units = fb.attrs['pos_units_mpcoverh']
        ntri = kmean = None
        if meas_type in ('grid_info', 'full') and tset is not None:
            nt, km = plan.gridinfo(tset)
            ntri, kmean = nt.cpu().numpy(), km.cpu().numpy() / units
        fulls = None
        if meas_type in ('unnorm_b_value', 'full') and tset is not None:
            fulls = self._device_meshes(plan.device)
        results = {}
        for i in subboxes:
            multi = subbox_index_to_multiindex(i, self.nsub).astype(int)
            B = np.zeros(len(index))
            if fulls is not None:
                for s, t in enumerate(fulls):
                    plan.paint_subbox(s, t, multi)
                b = plan.measure_b(tset, fb._slots(), fb.attrs.get('precision', 'bf16x3'))
                plan.sync_check()
                B = b.cpu().numpy() * units ** 6
            if meas_type == 'full':
                with np.errstate(divide='ignore', invalid='ignore'):
                    B = B / ntri
            res = {'index': index, 'k_edge': edges,
                   'k_mean': kmean if kmean is not None else np.zeros((len(index), 3)),
                   'B': B, 'N_tri': ntri if ntri is not None else np.zeros(len(index))}
            results[i] = res
            if out_file_prefix is not None:
                self._write(out_file_prefix + '_subbox%d.dat' % i, res, meas_type)
        if tset is not None:
            tset.close()
        return results

    @staticmethod
    def _write(path, res, meas_type):
        idx, e, km, B, nt = res['index'], res['k_edge'], res['k_mean'], res['B'], res['N_tri']
        if meas_type == 'grid_info':
            rows = ['%d %e %e %e %e %e %e %e %e %e %e\n' % ((idx[t],) + tuple(km[t]) +
                                                             tuple(e[t]) + (nt[t],))
                    for t in range(len(idx))]
        elif meas_type == 'unnorm_b_value':
            rows = ['%d %e %e %e %e %e %e %e\n' % ((idx[t],) + tuple(e[t]) + (B[t],))
                    for t in range(len(idx))]
        else:
            rows = ['%d %e %e %e %e %e %e %e %e %e %e %e\n' % ((idx[t],) + tuple(km[t]) +
                                                                tuple(e[t]) + (B[t], nt[t]))
                    for t in range(len(idx))]
        FFTBispectrum._write_batched(path, rows)

    def close(self):
        self.fb.close()
