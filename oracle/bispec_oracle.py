"""FP64 CPU oracle for the FFT bispectrum path -- TEST INFRASTRUCTURE ONLY.

This module is the oracle for the GPU path.  Only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may
import it; the product (``bskit_gb300``) never does.

It restates, in plain numpy/float64, what bskit computes on its "fast" and
"slow" paths (bskit/main.py):

* shell membership of a Fourier mode: ``kk = sum(ki**2. for ki in k)**0.5``
  closed on both edges (main.py:264-268, 314-320, 616-620, 1848-1852); the
  wavenumbers are ``q * (2*pi/L)`` with q the integer FFT frequency
  (``np.fft.fftfreq(N, 1/N)``; last axis ``0..N/2``);
* pmesh's transform convention: r2c scaled by 1/N^3, c2r unscaled, so a
  masked field is ``I(x) = sum_{k in shell} dhat_k exp(i k.x)``
  (the ``paint(mode='real')`` calls at main.py:275,327,646,1861);
* ``number_field`` / ``k_field`` (main.py:227-329): c2r of the indicator and
  of |k|^p times the indicator;
* shell mode counts ``sum(n_i**2)/N^3`` (``pk_FFT`` main.py:367-370);
* triangle sums: B_unnorm = sum_x I_a I_b I_c * L^6 / N^3 (main.py:1875-1877),
  N_tri = sum_x n_a n_b n_c / N^3 (main.py:2027-2029),
  k_mean_a = sum_x K_a n_b n_c / N^3 / N_tri with NaN on empty bins
  (main.py:2037-2057);
* field order for cross spectra: <AAB> / <ABC> (main.py:627-640);
* the final normalisation B = B_unnorm / N_tri
  (scripts/process/process_fast_bs_measurement.py:76);
* the brute-force "counting triangles" estimator ``bk_binned``
  (main.py:834-1004) used as a known-answer check on tiny grids.

Parity status: shell mode counts and grid info (N_tri, k_mean) are pinned
against bskit's own golden outputs (examples/tests/output_ref/
Lbox1000_512_kf_3kf_3lowkbins*.dat, test_grid_512_1_ps_kf_0.5kf.dat).  B
values are pinned by the brute-force estimator and by analytic plane-wave
fields; bskit's golden B files need input grids that are not distributed.
"""
import numpy as np

TWO_PI = 2.0 * np.pi


def freq_int(n, half=False):
    """Integer FFT frequencies of one axis (numpy/pmesh ordering)."""
    if half:
        return np.arange(n // 2 + 1, dtype=np.int64)
    return np.fft.fftfreq(n, 1.0 / n).astype(np.int64)


def mode_kk(n, box):
    """|k| of every half-complex mode of an n^3 grid, float64, shape (n, n, n//2+1).

    Evaluated exactly as ``sum(ki ** 2. for ki in k) ** 0.5`` over
    x, y, z with ki = q * (2 pi / L) (bskit/main.py:1850)."""
    kf = TWO_PI / box
    kx = (freq_int(n) * kf)[:, None, None]
    ky = (freq_int(n) * kf)[None, :, None]
    kz = (freq_int(n, half=True) * kf)[None, None, :]
    return ((kx * kx + ky * ky) + kz * kz) ** 0.5


def hermitian_weight(n):
    """Number of full-grid modes each half-complex mode stands for (1 or 2)."""
    w = np.full(n // 2 + 1, 2, dtype=np.int64)
    w[0] = 1
    if n % 2 == 0:
        w[-1] = 1
    return w


def shell_mask(kk, lo, hi):
    """Closed-edge membership (bskit/main.py:1852)."""
    return (kk <= hi) & (kk >= lo)


def shell_mode_counts(n, box, shell_edges):
    """Exact number of full-grid modes per shell (= pk_FFT's N_modes)."""
    kk = mode_kk(n, box)
    w = hermitian_weight(n)[None, None, :]
    return np.array([int((shell_mask(kk, lo, hi) * w).sum()) for lo, hi in shell_edges],
                    dtype=np.int64)


def spectrum(delta):
    """pmesh-normalised r2c of a real mesh: dhat = rfftn(delta) / N^3 (complex128)."""
    d = np.asarray(delta, dtype=np.float64)
    return np.fft.rfftn(d) / d.size


def cic_compensate(dhat, n, nmesh_cic):
    """Divide each mode by prod_c sqrt(1 - 2/3 sin^2(w_c Nmesh / (2 NmeshCIC))), w_c = 2 pi q_c / N
    (``CompensateCICShotnoiseNgrid``, scripts/measure/measure_bs_fast.py:45-57)."""
    out = np.array(dhat, dtype=np.complex128, copy=True)
    for axis, q in enumerate((freq_int(n), freq_int(n), freq_int(n, half=True))):
        w = 2 * np.pi * q / n
        f = (1 - 2. / 3 * np.sin(0.5 * w * n / nmesh_cic) ** 2) ** 0.5
        shape = [1, 1, 1]
        shape[axis] = len(q)
        out /= f.reshape(shape)
    return out


def c2r(spec, n):
    """Unnormalised c2r (pmesh ``paint(mode='real')``)."""
    return np.fft.irfftn(spec, s=(n, n, n), axes=(0, 1, 2)) * float(n) ** 3


def shell_fields(dhat, n, box, shell_edges):
    """Masked real-space fields I_i(x) for every shell, float64 (n_shells, n, n, n)."""
    kk = mode_kk(n, box)
    return np.stack([c2r(dhat * shell_mask(kk, lo, hi), n) for lo, hi in shell_edges])


def number_fields(n, box, shell_edges):
    kk = mode_kk(n, box)
    return np.stack([c2r(shell_mask(kk, lo, hi).astype(np.complex128), n)
                     for lo, hi in shell_edges])


def k_fields(n, box, shell_edges, p=1.0):
    kk = mode_kk(n, box)
    return np.stack([c2r((kk ** p * shell_mask(kk, lo, hi)).astype(np.complex128), n)
                     for lo, hi in shell_edges])


def triple_sums(fa, fb, fc, tri):
    """S[t] = sum_x fa[i_t] fb[j_t] fc[l_t] in float64, grouped by (i, j) pairs."""
    tri = np.asarray(tri, dtype=np.int64).reshape(-1, 3)
    out = np.zeros(len(tri), dtype=np.float64)
    flat_c = fc.reshape(fc.shape[0], -1)
    pairs = {}
    for t, (i, j, l) in enumerate(tri):
        pairs.setdefault((int(i), int(j)), []).append((t, int(l)))
    for (i, j), items in pairs.items():
        p = (fa[i] * fb[j]).ravel()
        ls = np.array([l for _, l in items])
        vals = flat_c[ls] @ p
        for (t, _), v in zip(items, vals):
            out[t] = v
    return out


def _irfftn3(spec, n, workers):
    """Unnormalised c2r through scipy.fft with host threads when available (same
    transform as ``c2r``; used for the large grids of the configuration tests)."""
    try:
        import scipy.fft as sf
        return sf.irfftn(spec, s=(n, n, n), axes=(0, 1, 2), workers=workers) * float(n) ** 3
    except ImportError:
        return c2r(spec, n)


def shell_fields_subset(dhat, n, box, shell_edges, shells, workers=-1):
    """I_i(x) (float64) of the listed shells only, as a dict shell -> (n, n, n) array.

    Same definition as ``shell_fields`` (masked pmesh c2r, main.py:1846-1861); for
    large grids where only the shells of a sample of triangle bins are needed."""
    kk = mode_kk(n, box)
    out = {}
    for s in sorted(set(int(v) for v in shells)):
        lo, hi = shell_edges[s]
        out[s] = _irfftn3(dhat * shell_mask(kk, lo, hi), n, workers)
    return out


def triple_sums_blocked(fa, fb, fc, tri, block=8, workers=None):
    """(S, A): S[t] = sum_x fa[i_t] fb[j_t] fc[l_t] and A[t] = sum_x |fa fb fc|, float64.

    fa / fb / fc map a shell index to its (n, n, n) field (arrays or dicts).  The
    sum over x runs in blocks of ``block`` x-planes on a pool of host threads
    (numpy releases the GIL), each block reusing its pair products for every third
    shell; the block partial sums are added in float64 (main.py:1875 sums the
    product over the whole grid; only the summation order differs)."""
    import concurrent.futures as cf
    import os

    tri = np.asarray(tri, dtype=np.int64).reshape(-1, 3)
    pairs = {}
    for t, (i, j, l) in enumerate(tri):
        pairs.setdefault((int(i), int(j)), []).append((t, int(l)))
    n = next(iter(fa.values())).shape[0] if isinstance(fa, dict) else fa.shape[1]

    def one(x0):
        x1 = min(n, x0 + block)
        S = np.zeros(len(tri))
        A = np.zeros(len(tri))
        for (i, j), items in pairs.items():
            p = (fa[i][x0:x1] * fb[j][x0:x1]).ravel()
            ap = np.abs(p)
            for t, l in items:
                c = fc[l][x0:x1].ravel()
                S[t] += p @ c
                A[t] += ap @ np.abs(c)
        return S, A

    S = np.zeros(len(tri))
    A = np.zeros(len(tri))
    with cf.ThreadPoolExecutor(max_workers=workers or os.cpu_count() or 4) as ex:
        for s_, a_ in ex.map(one, range(0, n, block)):
            S += s_
            A += a_
    return S, A


def bispectrum_unnormalized(meshes, box, shell_edges, tri, pos_units=1.0):
    """B_unnorm for every triangle (the ``measure_bispectrum_faster`` output).

    ``meshes`` is a list of 1-3 real meshes; 2 meshes give <AAB>, 3 give <ABC>.
    """
    n = meshes[0].shape[0]
    fields = [shell_fields(spectrum(m), n, box, shell_edges) for m in meshes]
    fa = fields[0]
    fb = fields[1] if len(fields) == 3 else fields[0]
    fc = fields[-1]
    s = triple_sums(fa, fb, fc, tri)
    return s * float(box) ** 6 / float(n) ** 3 * pos_units ** 6


def grid_info(n, box, shell_edges, tri, pos_units=1.0):
    """(N_tri, k_mean (T, 3)) as ``measure_gridinfo_faster`` computes them.

    N_tri is returned both raw (float64 sum) and rounded to the nearest
    integer; k_mean is NaN where the triangle count is zero."""
    nf = number_fields(n, box, shell_edges)
    kf = k_fields(n, box, shell_edges, 1.0)
    tri = np.asarray(tri, dtype=np.int64).reshape(-1, 3)
    n3 = float(n) ** 3
    ntri_raw = triple_sums(nf, nf, nf, tri) / n3
    s1 = triple_sums(kf, nf, nf, tri) / n3
    s2 = triple_sums(nf, kf, nf, tri) / n3
    s3 = triple_sums(nf, nf, kf, tri) / n3
    ntri = np.rint(ntri_raw)
    with np.errstate(divide="ignore", invalid="ignore"):
        km = np.stack([s1, s2, s3], axis=1) / ntri[:, None]
    km[ntri == 0] = np.nan
    return ntri_raw, ntri, km / pos_units


def normalize(b_unnorm, ntri):
    """B = B_unnorm / N_tri (process_fast_bs_measurement.py:76)."""
    with np.errstate(divide="ignore", invalid="ignore"):
        return np.asarray(b_unnorm, dtype=np.float64) / np.asarray(ntri, dtype=np.float64)


def bk_binned(delta, box, bin0, bin1, bin2):
    """Direct 'counting triangles' estimator (bskit/main.py:834-1004).

    Enumerates every full-grid mode whose k^2 falls in [kmin^2, kmax^2)
    (the ``np.digitize`` test of main.py:918-921), then sums
    dhat(k1) dhat(k2) dhat(k3) over k1+k2+k3 = 0 (no periodic wrap, as in
    main.py:974-979).  Returns (B, N_tri, k1_mean, k2_mean, k3_mean).
    """
    d = np.asarray(delta, dtype=np.float64)
    n = d.shape[0]
    kf = TWO_PI / float(box)
    dhat = np.fft.fftn(d) / d.size
    q = freq_int(n)
    qx, qy, qz = np.meshgrid(q, q, q, indexing="ij")
    k2 = (qx * kf) ** 2 + (qy * kf) ** 2 + (qz * kf) ** 2
    sets = []
    for b in (bin0, bin1, bin2):
        m = (k2 >= b[0] ** 2) & (k2 < b[1] ** 2)
        sets.append((np.stack([qx[m], qy[m], qz[m]], axis=1), dhat[m], np.sqrt(k2[m])))
    (q0, d0, k0), (q1, d1, k1), (q2, d2, k2v) = sets
    lut = {tuple(v): (dv, kv) for v, dv, kv in zip(q2.tolist(), d2, k2v)}
    B = 0.0 + 0.0j
    nt = 0
    km = np.zeros(3)
    for a in range(len(q0)):
        s = q0[a][None, :] + q1
        for b in range(len(q1)):
            hit = lut.get((-int(s[b, 0]), -int(s[b, 1]), -int(s[b, 2])))
            if hit is None:
                continue
            nt += 1
            B += d0[a] * d1[b] * hit[0]
            km += (k0[a], k1[b], hit[1])
    B = B * float(box) ** 6
    if nt > 0:
        B /= nt
        km /= nt
    return B, nt, km[0], km[1], km[2]


def lognormal_mesh_reference(n, box, seed):
    """Independent restatement of the synthetic lognormal input recipe, used by
    the tests to check ``bskit_gb300.synthetic.lognormal_mesh`` (float32 out)."""
    rng = np.random.default_rng(seed)
    white = rng.standard_normal((n, n, n))
    wk = np.fft.rfftn(white)
    kk = mode_kk(n, box)
    with np.errstate(divide="ignore"):
        pk = 1e3 * (kk / 0.1) ** -1.5 * np.exp(-(kk / 2.0) ** 2)
    pk[0, 0, 0] = 0.0
    amp = np.sqrt(pk * n ** 3 / box ** 3)
    g = np.fft.irfftn(wk * amp, s=(n, n, n), axes=(0, 1, 2))
    var = g.var()
    return (np.exp(g - var / 2.0) - 1.0).astype(np.float32)
