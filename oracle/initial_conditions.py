"""NumPy restatement of the reference's initial-condition pipeline.

TEST INFRASTRUCTURE: the oracle the parity tests compare the CUDA path with, never
the product.

Follows ``jax_cfd/base/initial_conditions.py:60-121`` and
``jax_cfd/base/filter_utils.py:25-42``.  The reference draws its noise with
``jax.random.normal``, whose bit stream cannot be reproduced without JAX, so the
noise here comes from ``numpy.random.default_rng(seed)`` (PCG64); the
filtering, projection and normalisation follow the reference line for line.
Parity on this boundary is therefore defined on identical noise arrays fed to
both sides (the PRNG itself is unpinned, as in the reference's own tests,
which only check divergence and the maximum speed).
"""
from __future__ import annotations

import numpy as np

from oracle import fvm


def log_normal_pdf(x, mode, variance=.25):
  """initial_conditions.py:60-64."""
  mean = np.log(mode) + variance
  logx = np.log(x)
  return np.exp(-(mean - logx) ** 2 / 2 / variance - logx)


def angular_frequency_magnitude(grid: fvm.Grid, dtype=np.float32):
  """filter_utils.py:25-29."""
  freqs = [2 * np.pi * fvm.fftfreq(n, s, dtype) for n, s in zip(grid.shape, grid.step)]
  mesh = np.stack(np.meshgrid(*freqs, indexing='ij'), axis=0)
  return np.sqrt(np.sum(mesh * mesh, axis=0)).astype(dtype)


def spectral_filter(spectral_density, array, grid: fvm.Grid):
  """filter_utils.py:32-42: ifftn(fftn(x) * filters).real."""
  k = angular_frequency_magnitude(grid, array.dtype)
  with np.errstate(divide='ignore', invalid='ignore'):
    filters = np.where(k > 0, spectral_density(k), 0.0).astype(array.dtype)
  return np.fft.ifftn(np.fft.fftn(array) * filters).real.astype(array.dtype)


def noise(seed: int, grid: fvm.Grid, dtype=np.float32):
  """Standard-normal noise per velocity component (stand-in for jax.random)."""
  rng = np.random.default_rng(seed)
  return tuple(rng.standard_normal(grid.shape).astype(dtype)
               for _ in range(grid.ndim))


def max_speed(v):
  """initial_conditions.py:67-68: max over cells of the norm across components."""
  return np.sqrt(np.sum(np.stack(v) ** 2, axis=0)).max()


def filtered_velocity_field(seed: int, grid: fvm.Grid, maximum_velocity=1.,
                            peak_wavenumber=3., iterations=3, dtype=np.float32,
                            noise_arrays=None):
  """initial_conditions.py:71-121."""
  def spectral_density(k):
    return log_normal_pdf(k, peak_wavenumber) / k ** (grid.ndim - 1)
  if noise_arrays is None:
    noise_arrays = noise(seed, grid, dtype)
  v = tuple(spectral_filter(spectral_density, n, grid) for n in noise_arrays)
  diag = fvm.pinv_diagonal(grid, dtype)
  for _ in range(iterations):
    v = fvm.projection(v, grid, diag)
    vmax = max_speed(v)
    v = tuple(maximum_velocity * u / vmax for u in v)
  return v
