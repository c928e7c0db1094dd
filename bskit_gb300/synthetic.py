"""Seeded synthetic density meshes (stand-ins for simulation snapshots).

Lognormal field: Gaussian g with power spectrum
    P(k) = 1e3 (k/0.1)^-1.5 exp(-(k/2)^2)   [h^-3 Mpc^3, k in h/Mpc], P(0) = 0,
built from seeded real-space white noise (numpy PCG64) as
    g = irfftn( rfftn(white) * sqrt(P(k) N^3 / L^3) ),
then delta = exp(g - var(g)/2) - 1, returned as float32.

``lognormal_mesh`` uses numpy (bit-reproducible, the reference input of the
parity tests); ``lognormal_mesh_torch`` follows the same recipe on a CUDA
device with torch's generator for large benchmark meshes.
"""
import numpy as np


def power_law_pk(k):
    with np.errstate(divide="ignore"):
        return 1e3 * (k / 0.1) ** -1.5 * np.exp(-(k / 2.0) ** 2)


def _kk(n, box):
    kf = 2.0 * np.pi / box
    q = np.fft.fftfreq(n, 1.0 / n) * kf
    qz = np.arange(n // 2 + 1) * kf
    return np.sqrt(q[:, None, None] ** 2 + q[None, :, None] ** 2 + qz[None, None, :] ** 2)


def lognormal_mesh(n, box, seed):
    rng = np.random.default_rng(seed)
    white = rng.standard_normal((n, n, n))
    pk = power_law_pk(_kk(n, box))
    pk[0, 0, 0] = 0.0
    g = np.fft.irfftn(np.fft.rfftn(white) * np.sqrt(pk * n ** 3 / box ** 3), s=(n, n, n),
                      axes=(0, 1, 2))
    return (np.exp(g - g.var() / 2.0) - 1.0).astype(np.float32)


def noisy_copy(delta, seed, amplitude=1.5, noise_var_frac=0.1):
    """delta2 = amplitude * delta + white noise of variance noise_var_frac * var(delta)."""
    rng = np.random.default_rng(seed)
    sig = np.sqrt(noise_var_frac * float(np.var(delta, dtype=np.float64)))
    return (amplitude * delta + sig * rng.standard_normal(delta.shape)).astype(np.float32)


def lognormal_mesh_torch(n, box, seed, device="cuda"):
    import torch

    gen = torch.Generator(device=device)
    gen.manual_seed(int(seed))
    white = torch.randn((n, n, n), generator=gen, device=device, dtype=torch.float32)
    kf = 2.0 * np.pi / box
    q = torch.fft.fftfreq(n, 1.0 / n, device=device, dtype=torch.float64) * kf
    qz = torch.arange(n // 2 + 1, device=device, dtype=torch.float64) * kf
    kk = torch.sqrt(q[:, None, None] ** 2 + q[None, :, None] ** 2 + qz[None, None, :] ** 2)
    pk = 1e3 * (kk / 0.1) ** -1.5 * torch.exp(-(kk / 2.0) ** 2)
    pk[0, 0, 0] = 0.0
    amp = torch.sqrt(pk * n ** 3 / box ** 3).to(torch.float32)
    del kk, pk
    wk = torch.fft.rfftn(white)
    del white
    wk *= amp
    del amp
    g = torch.fft.irfftn(wk, s=(n, n, n))
    del wk
    var = g.double().var().item()
    return torch.exp(g - var / 2.0) - 1.0


def noisy_copy_torch(delta, seed, amplitude=1.5, noise_var_frac=0.1):
    import torch

    gen = torch.Generator(device=delta.device)
    gen.manual_seed(int(seed))
    sig = float(np.sqrt(noise_var_frac * delta.double().var().item()))
    return amplitude * delta + sig * torch.randn(delta.shape, generator=gen, device=delta.device,
                                                 dtype=delta.dtype)
