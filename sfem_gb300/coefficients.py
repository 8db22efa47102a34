"""Heterogeneous coefficient fields k = exp(g) per macro element.

``g`` is a stationary Gaussian random field with standard deviation ``sigma``
and squared-exponential covariance of correlation length ``ell`` (in macro
elements), sampled by spectral synthesis on a zero-padded periodic grid
(circulant embedding of twice the size in every direction, then cropped), and
renormalised to the requested standard deviation.  One value per macro
element, so the Laplacian with this coefficient is the reference's affine
sshex8 operator with each macro element's metric scaled by ``k_e``
(``affine_sshex8_laplacian_stencil_apply_fff``, operators/sshex8/sshex8_laplacian.cpp:698-769).
"""

from __future__ import annotations

import numpy as np


def gaussian_random_field(shape, ell=8.0, sigma=1.0, seed=0) -> np.ndarray:
    nz, ny, nx = shape
    pz, py, px = 2 * nz, 2 * ny, 2 * nx
    rng = np.random.default_rng(seed)
    kz = np.fft.fftfreq(pz) * 2 * np.pi
    ky = np.fft.fftfreq(py) * 2 * np.pi
    kx = np.fft.fftfreq(px) * 2 * np.pi
    KZ, KY, KX = np.meshgrid(kz, ky, kx, indexing="ij")
    k2 = KZ**2 + KY**2 + KX**2
    # spectral density of exp(-r^2 / (2 ell^2)) (up to a constant)
    spec = np.exp(-0.5 * ell**2 * k2)
    noise = rng.standard_normal((pz, py, px))
    g = np.fft.ifftn(np.fft.fftn(noise) * np.sqrt(spec)).real[:nz, :ny, :nx]
    g = (g - g.mean()) / max(g.std(), 1e-300) * sigma
    return g


def lognormal_coefficient(nx, ny, nz, ell=8.0, sigma=1.0, seed=0) -> np.ndarray:
    """k_e = exp(g_e) for macro element e = a + nx*(b + ny*c), float32."""
    g = gaussian_random_field((nz, ny, nx), ell=ell, sigma=sigma, seed=seed)
    return np.exp(g).reshape(-1).astype(np.float32)
