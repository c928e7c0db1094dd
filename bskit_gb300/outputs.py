"""Result-file tools downstream of the measurement (host side).

* ``combine_bispectrum_files`` -- joins a grid-info file (from
  ``measure_gridinfo_faster``) and an unnormalised-B file (from
  ``measure_bispectrum_faster``) into the normalised 12-column table;
  same checks, k_max cut, divide and format as
  scripts/process/process_fast_bs_measurement.py:37-82.
* ``transform_bininfo_file`` -- rescales a grid-info file to another box size
  (bins defined in units of k_f): scripts/process/transform_bininfo_file.py:30-36.

Both are also command-line tools:
    python -m bskit_gb300.outputs combine BIN_INFO B_FILE K_MAX OUT
    python -m bskit_gb300.outputs transform IN OUT OLD_LBOX NEW_LBOX
"""
import sys

import numpy as np

EDGE_TOL = 0.01

COMBINED_HEADER = ('triangle index [dimensionless] k1_mean [h Mpc^-1] k2_mean [h Mpc^-1] '
                   'k3_mean [h Mpc^-1] k1_min [h Mpc^-1] k1_max [h Mpc^-1] k2_min [h Mpc^-1] '
                   'k2_max [h Mpc^-1] k3_min [h Mpc^-1] k3_max [h Mpc^-1] B_bin [h^-6 Mpc^6] '
                   'N_modes')
COMBINED_FMT = '%d ' + ' '.join(['%.6e'] * 11)
BININFO_FMT = '%d ' + ' '.join(['%.6e'] * 10)


def combine_arrays(bin_info, b_vals, k_max):
    """(rows, 12) array: bin info columns 0-9, B_unnorm / N_tri, N_tri.

    Rows stop before the first bin whose k1_min exceeds k_max, minus one more
    row, as bskit's script does; index and edge mismatches raise ValueError.
    """
    bin_info = np.atleast_2d(np.asarray(bin_info, dtype=np.float64))
    b_vals = np.atleast_2d(np.asarray(b_vals, dtype=np.float64))
    k1min = bin_info.T[4]
    if k1min[-1] > k_max:
        i_from_k_max = np.where(k1min == k1min[k1min > k_max][0])[0][0] - 1
    else:
        i_from_k_max = len(k1min)
    i_max = int(np.min([len(bin_info), len(b_vals), i_from_k_max]))
    out = np.zeros((i_max, 12))
    for i in range(i_max):
        if bin_info[i][0] != b_vals[i][0]:
            raise ValueError('Bin index mismatch between bin_info and B files: line %d: %d vs %d'
                             % (i, bin_info[i][0], b_vals[i][0]))
        for j in range(6):
            if np.abs((bin_info[i][4 + j] - b_vals[i][1 + j]) / bin_info[i][4 + j]) > EDGE_TOL:
                raise ValueError('Bin bound mismatch between bin_info and B files: line %d: %e vs %e'
                                 % (i, bin_info[i][4 + j], b_vals[i][1 + j]))
        out[i, 0:10] = bin_info[i, 0:10]
        out[i, 10] = b_vals[i, 7] / bin_info[i, 10]
        out[i, 11] = bin_info[i, 10]
    return out


def combine_bispectrum_files(bin_info_file, b_file, k_max, out_file):
    out = combine_arrays(np.loadtxt(bin_info_file), np.loadtxt(b_file), k_max)
    np.savetxt(out_file, out, fmt=COMBINED_FMT, header=COMBINED_HEADER)
    return out


def transform_bininfo(bin_info, old_lbox, new_lbox):
    """Multiply the k columns (1-9) by old_lbox / new_lbox."""
    b = np.array(bin_info, dtype=np.float64, copy=True)
    for i in range(1, 10):
        b.T[i] *= old_lbox / new_lbox
    return b


def transform_bininfo_file(in_file, out_file, old_lbox, new_lbox):
    b = transform_bininfo(np.loadtxt(in_file), old_lbox, new_lbox)
    np.savetxt(out_file, b, fmt=BININFO_FMT)
    return b


def main(argv):
    if len(argv) == 5 and argv[0] == 'combine':
        combine_bispectrum_files(argv[1], argv[2], float(argv[3]), argv[4])
    elif len(argv) == 5 and argv[0] == 'transform':
        transform_bininfo_file(argv[1], argv[2], float(argv[3]), float(argv[4]))
    else:
        sys.stderr.write(__doc__)
        return 2
    return 0


if __name__ == '__main__':
    sys.exit(main(sys.argv[1:]))
