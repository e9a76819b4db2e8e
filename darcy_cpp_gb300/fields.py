"""Random permeability fields (input generation, runs on the host).

Same published construction as the reference's generator
(python/darcy/fields.py:31-83, after Li et al., "Fourier Neural Operator for
Parametric PDEs", ICLR 2021): a mean-zero Gaussian random field with spectral
square-root eigenvalues ``tau^(alpha-1) (pi^2 |k|^2 + tau^2)^(-alpha/2)`` (the
k = 0 mode dropped), synthesised with an orthonormal inverse DCT, and a
threshold at zero into a two-phase medium. The arithmetic is written in the
same order as the reference so that the same seed gives the same field bits;
tests/golden pins the SHA-256 of the fields the reference itself produced.
"""

from __future__ import annotations

from typing import Union

import numpy as np

__all__ = ["gaussian_random_field", "two_phase_permeability"]

SeedLike = Union[int, np.random.Generator, None]


def _generator(seed: SeedLike) -> np.random.Generator:
    return seed if isinstance(seed, np.random.Generator) else np.random.default_rng(seed)


def gaussian_random_field(
    n: int,
    alpha: float = 2.0,
    tau: float = 3.0,
    seed: SeedLike = None,
    rng: np.random.Generator | None = None,
) -> np.ndarray:
    """Mean-zero GRF on an n x n grid, covariance (-Laplacian + tau^2 I)^(-alpha).

    ``seed`` is an int or a ``numpy.random.Generator``; ``rng`` is accepted as
    an alias, as the reference does (fields.py:38, :62).
    """
    if n < 1:
        raise ValueError(f"n must be positive, got {n}")
    gen = _generator(rng if rng is not None else seed)
    wave = np.arange(n)
    kx, ky = np.meshgrid(wave, wave, indexing="ij")
    spectrum = (np.pi**2) * (kx**2 + ky**2) + tau**2
    amplitude = (tau ** (alpha - 1.0)) * spectrum ** (-alpha / 2.0)
    amplitude[0, 0] = 0.0
    noise = gen.standard_normal((n, n))
    from scipy.fft import idctn

    return np.asarray(idctn(amplitude * noise, norm="ortho"), dtype=np.float64)


def two_phase_permeability(grf: np.ndarray, hi: float = 12.0, lo: float = 3.0) -> np.ndarray:
    """``hi`` where the field is >= 0, ``lo`` elsewhere (fields.py:72-83)."""
    if hi <= 0 or lo <= 0:
        raise ValueError("permeability phases must be strictly positive")
    return np.where(np.asarray(grf) >= 0.0, hi, lo).astype(np.float64)
