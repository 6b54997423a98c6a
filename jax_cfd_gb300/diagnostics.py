"""On-device flow diagnostics (jax_cfd/data/xarray_utils.py).

* ``vorticity_2d`` (155-162) — native curl at offset (1, 1);
* ``enstrophy`` — the mean of ``enstrophy_2d`` (165-167), a double reduction;
* ``isotropic_energy_spectrum`` — ``isotropize(energy_spectrum(ds),
  method='binsum')`` (279-290, 370-401): shell sums of 0.5 (|u^|^2 + |v^|^2)
  with the reference's bin bounds and labels, from the native real FFT.

These are the statistics of the long-horizon checks and of serving health;
they run on the GPU and return small host values.
"""
from __future__ import annotations

import ctypes
from typing import Tuple

import numpy as np
import torch

from jax_cfd_gb300 import _native as nat
from jax_cfd_gb300 import plans


def _grid_of(grid):
  return tuple(int(n) for n in grid.shape), tuple(float(s) for s in grid.step)


def shell_bins(shape, step):
  """Bounds and labels of the binsum isotropization (xarray_utils.py:279-290):
  k_spacing = max over axes of the first angular-wavenumber step, k_max = min
  over axes of the largest wavenumber minus half a spacing."""
  ks = [2 * np.pi * np.fft.fftfreq(n, s) for n, s in zip(shape, step)]
  k_spacing = max(float(k[1] - k[0]) for k in ks)
  k_max = min(float(k.max()) for k in ks) - 0.5 * k_spacing
  count = round(k_max / k_spacing)
  labels = k_spacing * np.arange(1, count + 1)
  return k_spacing, labels


def vorticity_2d(u: torch.Tensor, v: torch.Tensor, grid) -> torch.Tensor:
  shape, step = _grid_of(grid)
  plan = plans.cached('fvm-diag', (u.device, shape, step),
                      lambda: plans.FvmPlan(shape, step, device=u.device))
  return plan.curl_2d(u, v)


def enstrophy(u: torch.Tensor, v: torch.Tensor, grid) -> float:
  """Spatial mean of vorticity^2 / 2 (synchronises to return a float)."""
  shape, step = _grid_of(grid)
  plans.require_field(u, shape, name='u')
  plans.require_field(v, shape, name='v')
  out = torch.empty((), dtype=torch.float64, device=u.device)
  nat.check(nat.load().cfd_enstrophy_sum(plans.current_stream_ptr(u.device), shape[0], shape[1],
                                         step[0], step[1], plans.ptr(u), plans.ptr(v),
                                         plans.ptr(out)), 'cfd_enstrophy_sum')
  return float(out) / (shape[0] * shape[1])


def isotropic_energy_spectrum(u: torch.Tensor, v: torch.Tensor,
                              grid) -> Tuple[np.ndarray, torch.Tensor]:
  """(wavenumber labels, float64 device tensor of shell energies)."""
  shape, step = _grid_of(grid)
  plans.require_field(u, shape, name='u')
  plans.require_field(v, shape, name='v')
  ks, labels = shell_bins(shape, step)
  plan = plans.cached('spec-fft', (u.device, shape, step),
                      lambda: plans.SpecPlan(shape, step, device=u.device))
  out = torch.empty(labels.size, dtype=torch.float64, device=u.device)
  nat.check(nat.load().cfd_energy_spectrum_shells(
      plan.handle, plans.current_stream_ptr(u.device), plans.ptr(u), plans.ptr(v),
      ctypes.c_double(shape[0] * step[0]), ctypes.c_double(shape[1] * step[1]),
      ctypes.c_double(ks), int(labels.size), plans.ptr(out)), 'cfd_energy_spectrum_shells')
  return labels, out
