"""Seeded synthetic input fields for the MMH reconstruction workloads.

The reference reads N-body density grids from disk (mmh/main.f90:60-65); those
files are not available, so every workload here uses a seeded lognormal field
with the reference's own input contract: a periodic n^3 density of mean 1
(mmh/main.f90:72-77 stops the run unless |mean - 1| <= 1e-5).

Recipe: white Gaussian noise in k-space shaped by sqrt(P(k)), P(k) ~ k^ns,
Gaussian smoothing exp(-k^2 R^2 / 2) with R in cells, k = 0 removed,
normalised to unit variance and scaled by sigma; rho = exp(g - sigma^2/2),
renormalised to mean 1.
"""
import numpy as np


def lognormal_density(n, sigma=1.0, ns=-1.5, smooth=2.0, seed=1000, dtype=np.float64):
    """Return rho with shape (n, n, n) in Fortran order (rho[i, j, k] = u(1,i+1,j+1,k+1))."""
    rng = np.random.Generator(np.random.PCG64(seed))
    w = rng.standard_normal((n, n, n))
    W = np.fft.rfftn(w)
    kx = 2 * np.pi * np.fft.rfftfreq(n)
    ky = 2 * np.pi * np.fft.fftfreq(n)
    k2 = ky[:, None, None] ** 2 + ky[None, :, None] ** 2 + kx[None, None, :] ** 2
    k = np.sqrt(k2)
    with np.errstate(divide="ignore"):
        amp = np.where(k > 0, k ** (ns / 2.0), 0.0) * np.exp(-k2 * smooth * smooth / 2.0)
    g = np.fft.irfftn(W * amp, s=(n, n, n), axes=(0, 1, 2))
    g = g / g.std() * sigma
    rho = np.exp(g - sigma * sigma / 2.0)
    rho = rho / rho.mean()
    # rfftn over C-order (z, y, x) axes: transpose to Fortran (x, y, z) indexing
    return np.asfortranarray(rho.transpose(2, 1, 0), dtype=dtype)


def initial_state(n, sigma=1.0, ns=-1.5, seed=1000, dtype=np.float64, nfluid=5):
    """u(nfluid, n, n, n) with u(1) = rho and u(2:5) = 0, def = 0 (mmh/main.f90:57-83)."""
    rho = lognormal_density(n, sigma=sigma, ns=ns, seed=seed, dtype=dtype)
    u = np.zeros((nfluid, n, n, n), dtype=dtype, order="F")
    u[0] = rho
    defpot = np.zeros((n, n, n), dtype=dtype, order="F")
    return defpot, u
