"""Seeded synthetic k-sparse signals (no public dataset is involved).

Locations: k distinct frequencies drawn uniformly without replacement;
coefficients exp(i*phi), phi ~ U[0, 2 pi); time signal = exact inverse DFT in
the unnormalised convention the reference uses (x[t] = sum_f X_f e^{+2 pi i f t/n},
cuExperiment.cu:90-111), computed in FP64; optional complex Gaussian noise with
per-component sigma = sqrt(k / (2 snr)) (experiment.c:69, utils.c:187-219).
"""
from __future__ import annotations

import numpy as np


def sparse_spectrum(n, k, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    loc = np.sort(rng.choice(n, size=k, replace=False)).astype(np.int64)
    phase = rng.uniform(0.0, 2.0 * np.pi, size=k)
    return loc, np.exp(1j * phase)


def noise_sigma(k, snr_db):
    snr = 10.0 ** (snr_db / 10.0)
    return float(np.sqrt(k / (2.0 * snr)))


def signal_numpy(n, k, seed, snr_db=None):
    """(x, loc, coef, X_oracle) on the host in complex128."""
    loc, coef = sparse_spectrum(n, k, seed)
    X = np.zeros(n, np.complex128)
    X[loc] = coef
    x = np.fft.ifft(X) * n
    if snr_db is not None:
        rng = np.random.Generator(np.random.PCG64(seed + 0x5EED))
        s = noise_sigma(k, snr_db)
        x = x + s * (rng.standard_normal(n) + 1j * rng.standard_normal(n))
        X = np.fft.fft(x) / n
    return x, loc, coef, X


def signal_torch(n, k, seed, snr_db=None, device="cuda"):
    """Same signal built on the GPU with torch (FP64); returns (x, loc, coef, X)."""
    import torch
    loc, coef = sparse_spectrum(n, k, seed)
    X = torch.zeros(n, dtype=torch.complex128, device=device)
    X[torch.as_tensor(loc, device=device)] = torch.as_tensor(coef, device=device)
    x = torch.fft.ifft(X) * n
    if snr_db is not None:
        g = torch.Generator(device=device)
        g.manual_seed(seed + 0x5EED)
        s = noise_sigma(k, snr_db)
        nr = torch.randn(n, generator=g, device=device, dtype=torch.float64)
        ni = torch.randn(n, generator=g, device=device, dtype=torch.float64)
        x = x + s * torch.complex(nr, ni)
        X = torch.fft.fft(x) / n
    return x, loc, coef, X


def draws(seed, n, W, rlfc_loops, loops):
    """RLFC offsets and odd permutations (a, a^-1 mod n) from a seeded generator.

    The reference draws these with glibc drand48()/random() (innerLoop.cu:123,
    outerLoop.cu:128-134); the native API takes them as inputs so both sides of
    a parity test use identical draws.
    """
    rng = np.random.Generator(np.random.PCG64(seed ^ 0xD2A5))
    sigma = n // W
    offs = rng.integers(0, sigma, size=rlfc_loops).astype(np.int32)
    a = (rng.integers(0, n // 2, size=loops) * 2 + 1).astype(np.int64)
    ai = np.array([pow(int(v), -1, n) for v in a], np.int64)
    return offs, a.astype(np.int32), ai.astype(np.int32)
