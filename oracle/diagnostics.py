"""NumPy restatement of the reference's flow diagnostics.

TEST INFRASTRUCTURE: the oracle the tests compare the on-device diagnostics and the
long-horizon statistics with, never the product.  Follows
jax_cfd/data/xarray_utils.py (the reference computes these through xarray;
the arithmetic is the same on plain arrays):

* ``vorticity_2d`` (155-162) and ``enstrophy_2d`` (165-167);
* ``energy_spectrum`` (370-383): kinetic energy of the unnormalised ``fftn``
  of each velocity component, 0.5 (|u^|^2 + |v^|^2), at angular wavenumbers
  2 pi fftfreq(n, step) (``fourier_transform``, 191-209, before its fftshift,
  which only reorders);
* ``isotropize(..., method='binsum')`` (279-290, 253-275): the sum of the
  spectrum over shells of |k| with bounds k_spacing * (i - 0.5), i = 1 ..
  round(k_max / k_spacing) + 1, right-inclusive like ``pandas.cut``, labelled
  k_spacing * i.
"""
from __future__ import annotations

import numpy as np


def vorticity_2d(u: np.ndarray, v: np.ndarray, step) -> np.ndarray:
  """xarray_utils.py:155-162: (v[x+1] - v) / dx - (u[y+1] - u) / dy."""
  dx, dy = step
  return (np.roll(v, -1, axis=0) - v) / dx - (np.roll(u, -1, axis=1) - u) / dy


def enstrophy_2d(u, v, step) -> np.ndarray:
  """xarray_utils.py:165-167."""
  return vorticity_2d(u, v, step) ** 2 / 2


def wavenumbers(shape, step):
  return [2 * np.pi * np.fft.fftfreq(n, s) for n, s in zip(shape, step)]


def energy_spectrum(u, v, step) -> np.ndarray:
  """xarray_utils.py:370-383 (float64, unshifted order)."""
  uh = np.fft.fftn(np.asarray(u, np.float64))
  vh = np.fft.fftn(np.asarray(v, np.float64))
  return (np.abs(uh) ** 2 + np.abs(vh) ** 2) / 2


def shell_bins(shape, step):
  """Bounds and labels of the binsum isotropization (xarray_utils.py:279-290)."""
  ks = wavenumbers(shape, step)
  k_spacing = max(float(k[1] - k[0]) for k in ks)
  k_max = min(float(k.max()) for k in ks) - 0.5 * k_spacing
  count = round(k_max / k_spacing)
  bounds = k_spacing * (np.arange(1, count + 2) - 0.5)
  labels = k_spacing * np.arange(1, count + 1)
  return bounds, labels


def isotropic_energy_spectrum(u, v, step):
  """``isotropize(energy_spectrum(...), method='binsum')``: (labels, E(k))."""
  e = energy_spectrum(u, v, step)
  kx, ky = np.meshgrid(*wavenumbers(u.shape, step), indexing='ij')
  k = np.sqrt(kx * kx + ky * ky)
  bounds, labels = shell_bins(u.shape, step)
  # pandas.cut(k, bounds, labels=False): bin i holds bounds[i] < k <= bounds[i+1].
  idx = np.searchsorted(bounds, k.ravel(), side='left') - 1
  ok = (idx >= 0) & (idx < labels.size)
  out = np.zeros(labels.size)
  np.add.at(out, idx[ok], e.ravel()[ok])
  return labels, out
