"""Shell and triangle-bin specifications (host side).

Same names, arguments, outputs and errors as bskit's generators so that code
written against ``bskit`` keeps working:

* ``generate_bin_edge_list``                 -- bskit/main.py:1008-1071
* ``generate_equilateral_triangle_bin_list`` -- bskit/main.py:1074-1118
* ``generate_squeezed_triangle_bin_list``    -- bskit/main.py:1121-1178
* ``generate_isosceles_triangle_bin_list``   -- bskit/main.py:1181-1269
* ``generate_triangle_bin_list``             -- bskit/main.py:1272-1389
* ``geometric_k_mean``                       -- bskit/main.py:408-428

The outputs are bit-identical to bskit's (the shell edges come from the same
``np.arange`` fill, so the well known quirk that the last shell below ``kmax``
is dropped is kept).  The triangle enumeration is vectorised instead of
filtering ``itertools`` tuples, but yields the same rows in the same order:
rows are sorted by the lower edges of (k1, k2, k3), i.e. by shell index
because shell lower edges increase strictly.
"""
import numpy as np

__all__ = [
    "generate_bin_edge_list",
    "generate_equilateral_triangle_bin_list",
    "generate_squeezed_triangle_bin_list",
    "generate_isosceles_triangle_bin_list",
    "generate_triangle_bin_list",
    "geometric_k_mean",
    "triangle_indices_to_edges",
]


def geometric_k_mean(kmin, kmax):
    """Volume-weighted mean |k| of a shell: 3/4 (kmax^4-kmin^4)/(kmax^3-kmin^3).

    Same float expression as bskit/main.py:428 (so isosceles matching is
    bit-identical)."""
    return 0.75 * (kmax ** 4 - kmin ** 4) / (kmax ** 3 - kmin ** 3)


def generate_bin_edge_list(kmin=-1., kmax=-1., dk=-1., num_lowk_bins=0, dk_high=-1.):
    """(n, 2) array of closed shell edges [k_lower, k_upper].

    Lower edges are ``np.arange(kmin, kmax - dk, dk)`` (bskit/main.py:1052),
    upper edges ``k_lower + dk``; with ``num_lowk_bins > 0`` the shells after
    the first ``num_lowk_bins`` restart at the last low-k upper edge with width
    ``dk_high`` (bskit/main.py:1059-1066).
    """
    if kmin <= 0.:
        raise ValueError('kmin must be > 0!')
    if kmax <= 0.:
        raise ValueError('kmax must be > 0!')
    if dk <= 0.:
        raise ValueError('dk must be > 0!')
    if num_lowk_bins > 0 and dk_high < 0.:
        raise ValueError('Must specify dk_high if num_lowk_bins > 0!')

    lower = np.arange(kmin, kmax - dk, dk)
    upper = lower + np.ones_like(lower) * dk
    if 0 < num_lowk_bins < len(lower):
        lower_hi = np.arange(upper[num_lowk_bins - 1], kmax - dk_high, dk_high)
        upper_hi = lower_hi + np.ones_like(lower_hi) * dk_high
        lower = np.hstack((lower[:num_lowk_bins], lower_hi))
        upper = np.hstack((upper[:num_lowk_bins], upper_hi))
    return np.vstack((lower, upper)).T


def triangle_indices_to_edges(shell_edges, idx):
    """(T, 3) shell indices -> (T, 6) edges [k1_lo, k1_hi, k2_lo, k2_hi, k3_lo, k3_hi]."""
    idx = np.asarray(idx, dtype=np.int64).reshape(-1, 3)
    e = np.asarray(shell_edges, dtype=np.float64)
    return np.hstack((e[idx[:, 0]], e[idx[:, 1]], e[idx[:, 2]]))


def generate_equilateral_triangle_bin_list(kmin=-1., kmax=-1., dk=-1., num_lowk_bins=0,
                                           dk_high=-1., return_indices=False):
    """Equilateral triangle bins (i, i, i) for every shell (bskit/main.py:1074)."""
    edges = generate_bin_edge_list(kmin, kmax, dk, num_lowk_bins, dk_high)
    idx = np.repeat(np.arange(len(edges), dtype=np.int64)[:, None], 3, axis=1)
    if return_indices:
        return idx
    return np.hstack((edges, edges, edges))


def generate_squeezed_triangle_bin_list(kmin=-1., kmax=-1., dk=-1., squeezed_bin_index=0,
                                        num_lowk_bins=0, dk_high=-1., return_indices=False):
    """Squeezed bins (s, i, i) for every shell i above ``squeezed_bin_index`` s
    (bskit/main.py:1121)."""
    edges = generate_bin_edge_list(kmin, kmax, dk, num_lowk_bins, dk_high)
    s = int(squeezed_bin_index)
    short = np.arange(s + 1, len(edges), dtype=np.int64)
    idx = np.stack((np.full_like(short, s), short, short), axis=1).reshape(-1, 3)
    if return_indices:
        return idx
    if len(short) == 0:
        return np.zeros((0,), dtype=np.float64)
    return triangle_indices_to_edges(edges, idx)


def generate_isosceles_triangle_bin_list(kmin=-1., kmax=-1., dk=-1., isos_mult=0, isos_tol=0.1,
                                         num_lowk_bins=0, dk_high=-1., return_indices=False):
    """Isosceles bins (k_L, k_S, k_S) (bskit/main.py:1181-1269).

    For every shell S, the partner L is the shell whose geometric mean |k| is
    nearest to mean(S)/isos_mult; S is kept when the fractional mismatch is
    below ``isos_tol``.
    """
    if isos_mult < 1.:
        raise ValueError('isos_mult must be greater than 1! Come on man...')
    edges = generate_bin_edge_list(kmin, kmax, dk, num_lowk_bins, dk_high)
    kmean = np.array([geometric_k_mean(e[0], e[1]) for e in edges])
    target = kmean / isos_mult
    dist = np.abs(kmean[None, :] - target[:, None])
    nearest = dist.argmin(axis=1)
    dev = dist.min(axis=1) / target
    keep = dev < isos_tol
    s_idx = np.arange(len(edges), dtype=np.int64)[keep]
    l_idx = nearest[keep].astype(np.int64)
    idx = np.stack((l_idx, s_idx, s_idx), axis=1).reshape(-1, 3)
    if return_indices:
        return idx
    return np.hstack((edges[l_idx], edges[s_idx], edges[s_idx]))


def _closed_triangle_ok(edges, a, b, c):
    """Bin-edge triangle inequality of bskit/main.py:1338-1340 (float64)."""
    lo, hi = edges[:, 0], edges[:, 1]
    return ((hi[a] + hi[b] >= lo[c]) & (hi[a] + hi[c] >= lo[b]) & (hi[b] + hi[c] >= lo[a]))


def generate_triangle_bin_list(kmin=-1., kmax=-1., dk=-1., mu_min=None, mu_max=None, dmu=None,
                               num_fields=1, num_lowk_bins=0, dk_high=-1., return_indices=False):
    """All triangle bins for 1, 2 or 3 correlated fields (bskit/main.py:1272).

    * 1 field:  (i, j, l) with i >= j >= l;
    * 2 fields: (i, j, l) with i >= j, l free (the <AAB> ordering);
    * 3 fields: every (i, j, l);

    each kept when the bin edges admit a closed triangle, sorted by
    (k1_lo, k2_lo, k3_lo).
    """
    if num_fields not in [1, 2, 3]:
        raise ValueError('num_fields must be 1, 2, or 3!')
    if mu_min is not None or mu_max is not None or dmu is not None:
        raise NotImplementedError('Mu binning not implemented yet!')
    edges = generate_bin_edge_list(kmin, kmax, dk, num_lowk_bins, dk_high)
    n = len(edges)
    a, b, c = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    a, b, c = a.ravel(), b.ravel(), c.ravel()
    if num_fields == 1:
        sel = (a >= b) & (b >= c)
    elif num_fields == 2:
        sel = a >= b
    else:
        sel = np.ones_like(a, dtype=bool)
    a, b, c = a[sel], b[sel], c[sel]
    ok = _closed_triangle_ok(edges, a, b, c)
    idx = np.stack((a[ok], b[ok], c[ok]), axis=1).astype(np.int64)
    if len(idx) == 0:
        raise ValueError('no triangle bin satisfies the closure condition')
    # sort by (k1_lo, k2_lo, k3_lo) == lexicographic shell index order
    order = np.lexsort((idx[:, 2], idx[:, 1], idx[:, 0]))
    idx = idx[order]
    if return_indices:
        return idx
    return triangle_indices_to_edges(edges, idx)
