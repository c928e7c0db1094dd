"""bskit's bispectrum measurement scripts, on the GB300 engine.

    python -m bskit_gb300.measure bs_fast        <measure_bs_fast.py arguments>
    python -m bskit_gb300.measure bs_slow        <measure_bs_slow.py arguments>
    python -m bskit_gb300.measure subbox_bs_fast <measure_subbox_bs_fast.py arguments>

Same positional arguments, options, defaults, errors and output files as
scripts/measure/measure_bs_fast.py:58-262, measure_bs_slow.py and
measure_subbox_bs_fast.py:60-295, for grids stored as bigfile meshes
(``snap_type bigfile_grid``, read by ``BigFileMesh``).  The 'gadget' and 'illustris'
snapshot types paint particle catalogs with nbodykit, which is not part of this
package: they raise NotImplementedError naming the conversion to a bigfile grid.
One option is added: ``--precision`` (bf16x3, fp32, bf16, fp64) of the contraction.
No MPI: one process drives one GPU.
"""
import argparse
import sys
import time

import numpy as np

KINDS = ("bs_fast", "bs_slow", "subbox_bs_fast")


def make_parser(kind):
    """The reference script's argument parser (measure_bs_fast.py:58-111 and twins)."""
    p = argparse.ArgumentParser(prog="python -m bskit_gb300.measure " + kind)
    p.add_argument('snap_type', choices=['gadget', 'illustris', 'bigfile_grid'],
                   help='type of snapshot')
    p.add_argument('snap_prefix1',
                   help='complete file path to snapshot files for mesh 1, including file prefix')
    p.add_argument('nmesh', type=int, help='Nmesh for FFTs')
    p.add_argument('nmesh_cic', type=int, help='Nmesh to be used for CIC correction')
    p.add_argument('boxsize', type=float, help='BoxSize in Mpc/h')
    if kind == 'subbox_bs_fast':
        p.add_argument('nsub_per_side', type=int, help='number of subboxes per side')
    p.add_argument('start_bin_index', type=int, help='first bin index to use')
    p.add_argument('end_bin_index', type=int, help='last bin index to use')
    if kind == 'subbox_bs_fast':
        p.add_argument('start_subbox_index', type=int, help='first subbox index to use')
        p.add_argument('end_subbox_index', type=int, help='last subbox index to use')
        p.add_argument('out_file_prefix', help='prefix of the per-subbox output files')
    else:
        p.add_argument('out_file', help='file path to output file')
    p.add_argument('--k_bin_file',
                   help='complete file path to file containing k bin definitions '
                        '(can specify instead of kmin,kmax,dk values)')
    p.add_argument('--k_bin_info', type=float, nargs=3,
                   help='minimum and maximum k values for bispectrum triangles, and bin '
                        'width, in h/Mpc')
    p.add_argument('--high_k_bin_info', type=float, nargs=2,
                   help='number of bins with smaller dk, and dk for higher bins')
    p.add_argument('-pu', '--pos_units_mpcoverh', type=float,
                   help='units of particle positions in file, in Mpc/h')
    p.add_argument('-cic', '--cic_correction', action='store_true',
                   help='whether to apply extra CIC correction to input snapshot')
    p.add_argument('--snap_prefix2', help='snapshot files for mesh 2')
    p.add_argument('--snap_prefix3', help='snapshot files for mesh 3')
    p.add_argument('--triangle_type', choices=['all', 'equilateral', 'squeezed', 'isosceles'],
                   help='type of triangles to consider')
    p.add_argument('--squeezed_bin_index', type=int,
                   help='k bin index of k_long bin for squeezed triangles')
    p.add_argument('--isos_mult', type=float,
                   help='multiplier for isosceles triangles, such that k_S = mult * k_L')
    p.add_argument('--isos_tol', type=float,
                   help='tolerance for relationship between k_S and k_L to count as isosceles')
    if kind == 'bs_slow':
        p.add_argument('--meas_type', choices=['full', 'grid_info', 'unnorm_b_value'],
                       help='type of measurement to do (full, grid_info, or unnorm_b_value')
    else:
        p.add_argument('--meas_type', choices=['grid_info', 'unnorm_b_value'],
                       default='unnorm_b_value',
                       help='type of measurement to do (grid_info or unnorm_b_value')
    p.add_argument('--precision', choices=['bf16x3', 'fp32', 'bf16', 'fp64'], default='bf16x3',
                   help='arithmetic of the triple-product contraction (not in bskit)')
    return p


def binning(args):
    """FFTBispectrum binning keywords from the parsed arguments, with the scripts' checks
    and defaults (measure_bs_fast.py:113-193)."""
    if (args.k_bin_file and args.k_bin_info) or (not args.k_bin_file and not args.k_bin_info):
        raise RuntimeError('Must specify either a k-bin file or kmin/kmax/dk!')
    kw = dict(pos_units_mpcoverh=1. if args.pos_units_mpcoverh is None
              else args.pos_units_mpcoverh)
    if args.k_bin_file:
        kw['k_edges'] = np.loadtxt(args.k_bin_file).T
        return kw
    triangle_type = args.triangle_type or 'all'
    kw.update(kmin=args.k_bin_info[0], kmax=args.k_bin_info[1], dk=args.k_bin_info[2],
              num_lowk_bins=0, dk_high=-1., triangle_type=triangle_type,
              squeezed_bin_index=0, isos_mult=0, isos_tol=0.1)
    if args.high_k_bin_info is not None:
        kw['num_lowk_bins'] = int(args.high_k_bin_info[0])
        kw['dk_high'] = args.high_k_bin_info[1]
    if triangle_type == 'squeezed' and args.squeezed_bin_index is not None:
        kw['squeezed_bin_index'] = args.squeezed_bin_index
    elif triangle_type == 'isosceles':
        if args.isos_mult is None:
            raise ValueError('Need to set isos_mult for isosceles triangles!')
        kw['isos_mult'] = args.isos_mult
        if args.isos_tol is not None:
            kw['isos_tol'] = args.isos_tol
    return kw


def load_meshes(args):
    """Meshes 1..3 of the run (measure_bs_fast.py:196-224); the CIC correction is applied
    when each mesh is painted."""
    prefixes = [args.snap_prefix1, args.snap_prefix2, args.snap_prefix3]
    if prefixes[2] is not None and prefixes[1] is None:
        raise ValueError('need second mesh if third mesh is input!')
    if args.snap_type != 'bigfile_grid':
        raise NotImplementedError(
            "snap_type %r paints a particle catalog with nbodykit, which this package does "
            "not include; paint it to a bigfile grid first (bskit's scripts/grids "
            "converters) and pass snap_type bigfile_grid" % args.snap_type)
    from .bigfile import BigFileMesh
    cic = args.nmesh_cic if args.cic_correction else None
    return [BigFileMesh(p, 'Field', compensate_cic=cic) if p is not None else None
            for p in prefixes]


def run(kind, argv=None, out=None):
    """Parse ``argv`` as the reference script ``kind`` does and run its measurement;
    status lines go to ``out`` (standard output by default)."""
    from .bispectrum import FFTBispectrum
    from .subbox import SubboxBispectrum

    args = make_parser(kind).parse_args(argv)
    start = time.time()

    def status(msg):
        print('%d\ts: %s' % (time.time() - start, msg), file=out or sys.stdout)

    status('Starting script')
    kw = binning(args)
    meshes = load_meshes(args)
    status('Finished input')
    if kind == 'bs_slow':
        meas_type = args.meas_type or 'full'
    else:
        meas_type = args.meas_type
    grid_only = meas_type == 'grid_info'
    box = np.ones(3) * args.boxsize

    if kind == 'subbox_bs_fast':
        if 'k_edges' in kw:
            # bskit's fast methods need shell indices, which k_edges does not set
            # (bskit/main.py:1550-1551): the reference script fails there as well
            raise NotImplementedError('the fast sub-box measurement derives its shells from '
                                      '--k_bin_info, not from a k-bin file')
        if meshes[0].Nmesh != args.nmesh:
            raise ValueError('Nmesh %d differs from the mesh size %d (resampling is not '
                             'supported)' % (args.nmesh, meshes[0].Nmesh))
        sb = SubboxBispectrum(meshes[0], args.nsub_per_side, BoxSize=args.boxsize,
                              second=meshes[1], third=meshes[2], precision=args.precision,
                              **kw)
        status('Starting subbox measurements')
        sb.measure(subboxes=range(args.start_subbox_index, args.end_subbox_index + 1),
                   imin=args.start_bin_index, imax=args.end_bin_index, meas_type=meas_type,
                   out_file_prefix=args.out_file_prefix)
        sb.close()
        status('Finished FFT bispectrum')
        return 0

    status('Starting initial paints')
    fftb = FFTBispectrum(meshes[0], Nmesh=args.nmesh, BoxSize=box, second=meshes[1],
                         third=meshes[2], for_grid_info_only=grid_only,
                         precision=args.precision, **kw)
    status('Finished initial paints')
    if kind == 'bs_slow':
        status('Starting FFT binning info computation' if grid_only else 'Starting FFT bispectrum')
        fftb.measure_bispectrum(imin=args.start_bin_index, imax=args.end_bin_index,
                                out_file=args.out_file, verbose=0, meas_type=meas_type)
    elif grid_only:
        status('Starting FFT binning info computation')
        fftb.measure_gridinfo_faster(imin=args.start_bin_index, imax=args.end_bin_index,
                                     out_file=args.out_file, verbose=0)
    else:
        status('Starting FFT bispectrum')
        fftb.measure_bispectrum_faster(imin=args.start_bin_index, imax=args.end_bin_index,
                                       out_file=args.out_file, verbose=0)
    fftb.close()
    status('Finished FFT bispectrum')
    return 0


def main(argv=None):
    argv = sys.argv[1:] if argv is None else list(argv)
    if not argv or argv[0] not in KINDS:
        print("usage: python -m bskit_gb300.measure {%s} <the script's arguments>" %
              ",".join(KINDS), file=sys.stderr)
        return 2
    return run(argv[0], argv[1:])


if __name__ == "__main__":
    sys.exit(main())
