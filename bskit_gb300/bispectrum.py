"""Drop-in ``FFTBispectrum`` measurement API (bskit/main.py:1392-2161) on GB300.

Same constructor arguments, methods, ``b`` result dictionary, ``attrs``,
ASCII output rows and errors as bskit's class; the arithmetic runs in the
C-ABI CUDA library (``engine.Plan``):

* ``__init__``                  -> bin lists (main.py:1549-1584) + r2c of each source
                                   (``_paint_meshes``, main.py:1608-1621)
* ``measure_bispectrum_faster`` -> unnormalised B of an index range (main.py:1784-1938)
* ``measure_gridinfo_faster``   -> N_tri and k_mean of an index range (main.py:1941-2132)
* ``measure_bispectrum``        -> per-triangle 'full' / 'grid_info' / 'unnorm_b_value'
                                   (main.py:1637-1780), including cross spectra
* ``save_bispectrum``, ``set_k_edges``, pickling of ``b``/``k_edges``/``attrs``.

Differences from bskit, all deliberate:
* sources are real meshes given as arrays (``ArrayMesh`` or numpy / torch
  arrays) instead of nbodykit sources; one process, one GPU, no MPI;
* ``measure_bispectrum_faster`` also accepts cross spectra (<AAB> with two
  sources, <ABC> with three), which bskit raises NotImplementedError for;
* triangle counts are the rounded (exact integer) FFT sums, and k_mean is NaN
  exactly when the count is zero;
* ``save_bispectrum`` writes the file (bskit passes a ``zip`` to np.savetxt,
  which fails on Python 3).
"""
import logging

import numpy as np
import torch

from . import bins as _bins
from .engine import Plan
from .mesh import ArrayMesh, as_mesh

NUM_TRI_TO_WRITE = 100


def _cubic(v, name):
    a = np.atleast_1d(np.asarray(v, dtype=np.float64))
    if a.size == 1:
        a = np.repeat(a, 3)
    if a.size != 3 or not np.all(a == a[0]):
        raise ValueError("%s must be a scalar or three equal values (cubic boxes only)" % name)
    return a


class FFTBispectrum(object):
    """Bispectrum measurements from one mesh, or cross bispectra of 2-3 meshes.

    Extra keyword arguments beyond bskit's:
    precision : 'bf16x3' (default), 'fp32', 'bf16' or 'fp64' -- arithmetic of the
        triple-product contraction of B (grid information is exact: integer lattice
        enumeration, or FP64 fields where that does not apply);
    grid : 'reduced' (default: each bin on the smallest exact grid its shells allow),
        'single' (the reduced grid for every bin) or 'native' -- see ``engine.Plan``;
    device : CUDA device of the computation;
    mem_budget : bytes of device memory the engine plan may hold (0 = no limit); a
        measurement that would exceed it raises BskError (BSK_ERR_OOM) before allocating.
    """
    logger = logging.getLogger('FFTBispectrum')

    def __init__(self, source, Nmesh=None, BoxSize=None, dk=None, kmin=None, kmax=None,
                 num_lowk_bins=0, dk_high=-1., dmu=None, mu_min=None, mu_max=None,
                 pos_units_mpcoverh=1., k_edges=None, second=None, third=None,
                 triangle_type='all', isos_mult=0, isos_tol=0.1, squeezed_bin_index=0,
                 for_grid_info_only=False, precision='bf16x3', grid='reduced', device=None,
                 mem_budget=0):
        self.mesh = as_mesh(source, Nmesh=Nmesh, BoxSize=BoxSize)
        self.second = None
        self.third = None
        self.attrs = {}
        self.attrs['Nmesh'] = _cubic(self.mesh.attrs['Nmesh'], 'Nmesh').astype(int)
        self.attrs['BoxSize'] = _cubic(self.mesh.attrs['BoxSize'], 'BoxSize')

        self.num_fields = 1
        if second is not None:
            self.second = as_mesh(second, Nmesh=Nmesh, BoxSize=BoxSize)
            self.num_fields += 1
        if third is not None:
            if second is None:
                raise ValueError('Need second source defined if third source is defined!')
            self.third = as_mesh(third, Nmesh=Nmesh, BoxSize=BoxSize)
            self.num_fields += 1
        for other, nm in ((self.second, 'second'), (self.third, 'third')):
            if other is None:
                continue
            if not np.array_equal(_cubic(other.attrs['BoxSize'], 'BoxSize'), self.attrs['BoxSize']):
                raise ValueError('BoxSize mismatch between first and %s mesh' % nm)
            if not np.array_equal(_cubic(other.attrs['Nmesh'], 'Nmesh'), self.attrs['Nmesh']):
                raise ValueError('Nmesh mismatch between first and %s mesh' % nm)

        if dk is None:
            dk = 2 * np.pi / self.attrs['BoxSize'].min()
        if (kmin is None or kmax is None) and k_edges is None:
            raise ValueError('Must specify either {kmin,kmax} values or k_edges array!')

        self.attrs['dk'] = dk
        self.attrs['kmin'] = kmin
        self.attrs['kmax'] = kmax
        self.attrs['dmu'] = dmu
        self.attrs['mu_min'] = mu_min
        self.attrs['mu_max'] = mu_max
        self.attrs['pos_units_mpcoverh'] = pos_units_mpcoverh
        self.attrs['triangle_type'] = triangle_type
        self.attrs['num_lowk_bins'] = num_lowk_bins
        self.attrs['dk_high'] = dk_high
        self.attrs['isos_mult'] = isos_mult
        self.attrs['isos_tol'] = isos_tol
        self.attrs['squeezed_bin_index'] = squeezed_bin_index
        self.attrs['precision'] = precision
        self.attrs['grid'] = grid

        self._device = device
        self._mem_budget = mem_budget
        self._plans = {}

        if k_edges is not None:
            self.k_edges = k_edges
        else:
            kw = dict(num_lowk_bins=num_lowk_bins, dk_high=dk_high)
            if triangle_type == 'all':
                self.k_edges = _bins.generate_triangle_bin_list(
                    kmin=kmin, kmax=kmax, dk=dk, dmu=dmu, mu_min=mu_min, mu_max=mu_max,
                    num_fields=self.num_fields, **kw)
                self.k_indices = _bins.generate_triangle_bin_list(
                    kmin=kmin, kmax=kmax, dk=dk, dmu=dmu, mu_min=mu_min, mu_max=mu_max,
                    num_fields=self.num_fields, return_indices=True, **kw)
            elif triangle_type == 'equilateral':
                self.k_edges = _bins.generate_equilateral_triangle_bin_list(
                    kmin=kmin, kmax=kmax, dk=dk, **kw)
                self.k_indices = _bins.generate_equilateral_triangle_bin_list(
                    kmin=kmin, kmax=kmax, dk=dk, return_indices=True, **kw)
            elif triangle_type == 'squeezed':
                self.k_edges = _bins.generate_squeezed_triangle_bin_list(
                    kmin, kmax, dk, squeezed_bin_index=squeezed_bin_index, **kw)
                self.k_indices = _bins.generate_squeezed_triangle_bin_list(
                    kmin, kmax, dk, squeezed_bin_index=squeezed_bin_index, return_indices=True,
                    **kw)
            elif triangle_type == 'isosceles':
                self.k_edges = _bins.generate_isosceles_triangle_bin_list(
                    kmin, kmax, dk, isos_mult=isos_mult, isos_tol=isos_tol, **kw)
                self.k_indices = _bins.generate_isosceles_triangle_bin_list(
                    kmin, kmax, dk, isos_mult=isos_mult, isos_tol=isos_tol,
                    return_indices=True, **kw)

        self.b = None
        if not for_grid_info_only:
            self._paint_meshes()
        else:
            self.attrs['painted'] = False

    # ---------------------------------------------------------------- pickling
    def __getstate__(self):
        return dict(b=self.b, k_edges=self.k_edges, attrs=self.attrs)

    def __setstate__(self, state):
        self.attrs = state['attrs']
        self.k_edges = state['k_edges']
        self.b = state['b']
        self._plans = {}

    # ---------------------------------------------------------------- engine plumbing
    def _meshes(self):
        return [m for m in (self.mesh, self.second, self.third) if m is not None]

    def _plan(self, shell_edges):
        """Engine plan for a shell list (cached), with every source painted."""
        edges = np.ascontiguousarray(np.asarray(shell_edges, dtype=np.float64).reshape(-1, 2))
        key = edges.tobytes()
        plan = self._plans.get(key)
        if plan is None:
            plan = Plan(int(self.attrs['Nmesh'][0]), float(self.attrs['BoxSize'][0]), edges,
                        grid=self.attrs.get('grid', 'reduced'), mem_budget=self._mem_budget,
                        device=self._device)
            plan.painted = False
            self._plans[key] = plan
        return plan

    def _paint_plan(self, plan):
        if not plan.painted:
            for s, m in enumerate(self._meshes()):
                plan.paint(s, m.tensor(plan.device), cic_nmesh=m.compensate_cic)
            plan.painted = True

    def _paint_meshes(self):
        """r2c of every source on the plan of the regular shell list (bskit/main.py:1608)."""
        if self.attrs.get('kmin') is not None:
            self._paint_plan(self._plan(self._shell_edges()))
        self.attrs['painted'] = True

    def _shell_edges(self):
        if self.attrs.get('kmin') is None or self.attrs.get('kmax') is None:
            raise ValueError('kmin/kmax are needed for the fast methods (bskit derives the '
                             'shells from them, main.py:1828)')
        return _bins.generate_bin_edge_list(self.attrs['kmin'], self.attrs['kmax'],
                                            self.attrs['dk'], self.attrs['num_lowk_bins'],
                                            self.attrs['dk_high'])

    def _slots(self):
        return {1: (0, 0, 0), 2: (0, 0, 1), 3: (0, 1, 2)}[self.num_fields]

    def set_k_edges(self, k_edges):
        """Set the array of triangle-bin edges (bskit/main.py:1624)."""
        self.k_edges = k_edges

    # ---------------------------------------------------------------- results
    def _append(self, index, k_edge, k_mean, B, N_tri):
        index = np.asarray(index)
        if self.b is None:
            self.b = {'index': index, 'k_edge': np.asarray(k_edge), 'k_mean': np.asarray(k_mean),
                      'B': np.asarray(B, dtype=np.float64), 'N_tri': np.asarray(N_tri, dtype=np.float64)}
        else:
            self.b['index'] = np.append(self.b['index'], index, axis=0)
            self.b['k_edge'] = np.append(self.b['k_edge'], k_edge, axis=0)
            self.b['k_mean'] = np.append(self.b['k_mean'], k_mean, axis=0)
            self.b['B'] = np.append(self.b['B'], B, axis=0)
            self.b['N_tri'] = np.append(self.b['N_tri'], N_tri, axis=0)

    def _tail(self, n):
        if n == 0:
            return {k: v[:0] for k, v in self.b.items()} if self.b is not None else {
                'index': np.zeros(0, int), 'k_edge': np.zeros((0, 6)), 'k_mean': np.zeros(0),
                'B': np.zeros(0), 'N_tri': np.zeros(0)}
        return {k: v[-n:] for k, v in self.b.items()}

    @staticmethod
    def _write_batched(out_file, rows):
        """Append rows the way bskit's fast methods do (main.py:1909-1929): in
        blocks of 100 and a final partial block, and nothing at all when only
        one triangle was measured."""
        if out_file is None or len(rows) < 2:
            return
        with open(out_file, "a") as f:
            f.writelines(rows)

    def _range(self, imin, imax, n_total):
        imin = 0 if imin is None else imin
        imax = n_total if imax is None else imax
        return imin, min(imax, n_total)

    # ---------------------------------------------------------------- fast methods
    def measure_bispectrum_faster(self, imin=None, imax=None, kmeas_min=None, kmeas_max=None,
                                  out_file=None, verbose=0):
        """Unnormalised B of triangle bins imin..imax-1 (bskit/main.py:1784)."""
        if (kmeas_min is not None) and (kmeas_max is not None):
            raise NotImplementedError('kmeas_min/kmeas_max not implemented yet!')
        i0, i1 = self._range(imin, imax, len(self.k_indices))
        edges = np.asarray(self.k_edges[i0:i1])
        triples = np.asarray(self.k_indices[i0:i1])
        index = np.arange(i0, i1)
        if len(triples) == 0:
            return self._tail(0)
        plan = self._plan(self._shell_edges())
        self._paint_plan(plan)
        tset = plan.triangles(triples)
        B = plan.measure_b(tset, self._slots(), self.attrs.get('precision', 'bf16x3'))
        plan.sync_check()
        B = B.cpu().numpy() * self.attrs['pos_units_mpcoverh'] ** 6.
        tset.close()
        self._append(index, edges, np.zeros(len(index)), B, np.zeros(len(index)))
        if verbose > 0:
            for t in range(len(index)):
                print('FFT Bk: %d %d %g %g' % (t, index[t], B[t], 0.))
        rows = ['%d %e %e %e %e %e %e %e\n' % ((index[t],) + tuple(edges[t]) + (B[t],))
                for t in range(len(index))]
        self._write_batched(out_file, rows)
        return self._tail(len(index))

    def measure_gridinfo_faster(self, imin=None, imax=None, kmeas_min=None, kmeas_max=None,
                                out_file=None, verbose=0):
        """Triangle counts and mean |k_i| of bins imin..imax-1 (bskit/main.py:1941)."""
        if (kmeas_min is not None) and (kmeas_max is not None):
            raise NotImplementedError('kmeas_min/kmeas_max not implemented yet!')
        i0, i1 = self._range(imin, imax, len(self.k_indices))
        edges = np.asarray(self.k_edges[i0:i1])
        triples = np.asarray(self.k_indices[i0:i1])
        index = np.arange(i0, i1)
        if len(triples) == 0:
            return self._tail(0)
        plan = self._plan(self._shell_edges())
        tset = plan.triangles(triples)
        ntri, kmean = plan.gridinfo(tset)
        plan.sync_check()
        ntri = ntri.cpu().numpy()
        kmean = kmean.cpu().numpy() / self.attrs['pos_units_mpcoverh']
        tset.close()
        self._append(index, edges, kmean, np.zeros(len(index)), ntri)
        if verbose > 0:
            for t in range(len(index)):
                if (t + 1) % 100 == 0:
                    print('FFT Bk: %d %d %g %g %g %g %g' % (t, index[t], kmean[t, 0], kmean[t, 1],
                                                           kmean[t, 2], 0., ntri[t]))
        rows = ['%d %e %e %e %e %e %e %e %e %e %e\n' % ((index[t],) + tuple(kmean[t]) +
                                                         tuple(edges[t]) + (ntri[t],))
                for t in range(len(index))]
        self._write_batched(out_file, rows)
        return self._tail(len(index))

    # ---------------------------------------------------------------- slow method
    def measure_bispectrum(self, imin=None, imax=None, kmeas_min=None, kmeas_max=None,
                           out_file=None, verbose=0, meas_type='full'):
        """Per-triangle measurement over bins imin..imax-1 (bskit/main.py:1637).

        meas_type: 'full' (B, N_tri, k_mean), 'grid_info' (N_tri, k_mean) or
        'unnorm_b_value' (B not divided by N_tri).  Bin edges are scaled by
        pos_units_mpcoverh before masking, as bskit does (main.py:1708-1722).
        """
        if (kmeas_min is not None) and (kmeas_max is not None):
            raise NotImplementedError('kmeas_min/kmeas_max not implemented yet!')
        if meas_type not in ('full', 'grid_info', 'unnorm_b_value'):
            raise ValueError("meas_type must be 'full', 'grid_info' or 'unnorm_b_value'")
        k_edges = np.asarray(self.k_edges, dtype=np.float64).reshape(-1, 6)
        i0, i1 = self._range(imin, imax, len(k_edges))
        tri_list = k_edges[i0:i1]
        index = np.arange(i0, i1)
        T = len(tri_list)
        if T == 0:
            return self._tail(0)
        u = self.attrs['pos_units_mpcoverh']
        scaled = tri_list * u
        pairs = scaled.reshape(-1, 2)
        shells, inv = np.unique(pairs, axis=0, return_inverse=True)
        triples = inv.reshape(-1, 3)
        # shells sorted by (lo, hi): membership of a mode is a run of consecutive shells
        plan = self._plan(shells)
        tset = plan.triangles(triples)
        B = np.zeros(T)
        ntri = np.zeros(T)
        kmean = np.zeros((T, 3))
        if meas_type in ('full', 'grid_info'):
            nt, km = plan.gridinfo(tset)
            plan.sync_check()
            ntri = nt.cpu().numpy()
            kmean = km.cpu().numpy()
        if meas_type in ('full', 'unnorm_b_value'):
            self._paint_plan(plan)
            Bu = plan.measure_b(tset, self._slots(), self.attrs.get('precision', 'bf16x3'))
            plan.sync_check()
            B = Bu.cpu().numpy()
            if meas_type == 'full':
                with np.errstate(divide='ignore', invalid='ignore'):
                    B = B / ntri
        tset.close()
        kmean = kmean / u
        B = B * u ** 6.
        self._append(index, tri_list, kmean, B, ntri)
        for t in range(T):
            if verbose > 0:
                print('FFT Bk: %d %g %g %g %g %g' % (t, kmean[t, 0], kmean[t, 1], kmean[t, 2],
                                                    B[t], ntri[t]))
        if out_file is not None:
            with open(out_file, "a") as f:
                for t in range(T):
                    e = tuple(tri_list[t])
                    if meas_type == 'full':
                        f.write('%d %e %e %e %e %e %e %e %e %e %e %e\n' %
                                ((index[t],) + tuple(kmean[t]) + e + (B[t], ntri[t])))
                    elif meas_type == 'grid_info':
                        f.write('%d %e %e %e %e %e %e %e %e %e %e\n' %
                                ((index[t],) + tuple(kmean[t]) + e + (ntri[t],)))
                    else:
                        f.write('%d %e\n' % (index[t], B[t]))
        return self._tail(T)

    # ---------------------------------------------------------------- output
    def save_bispectrum(self, out_file):
        """Write the accumulated ``b`` dict as text (bskit/main.py:2135)."""
        b = self.b
        if b is None:
            return
        header = 'k1_mean k2_mean k3_mean k1_low k1_high k2_low k2_high k3_low k3_high ' \
                 + '[all h Mpc^-1] B [h^-6 Mpc^6] N_tri'
        km = np.asarray(b['k_mean'], dtype=np.float64)
        if km.ndim == 1:
            km = np.repeat(km[:, None], 3, axis=1)
        ke = np.asarray(b['k_edge'], dtype=np.float64).reshape(-1, 6)
        cols = np.column_stack([km, ke, b['B'], b['N_tri']])
        np.savetxt(out_file, cols, header=header)

    def close(self):
        for p in self._plans.values():
            p.close()
        self._plans = {}
