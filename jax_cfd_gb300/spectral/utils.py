"""Spectral helpers, mirroring ``jax_cfd/spectral/utils.py:128-203``.

These build the tables and conversions callers use around the step (device
torch expressions); the step itself applies the same operations inside its
native kernels.
"""
from __future__ import annotations

import numpy as np
import torch

from jax_cfd_gb300 import plans
from jax_cfd_gb300.base import grids


def brick_wall_filter_2d(grid: grids.Grid, device=None) -> torch.Tensor:
  """spectral/utils.py:128-134 (2/3 rule, asymmetric negative-row slice)."""
  n, m = grid.shape
  f = np.zeros((n, m // 2 + 1), np.float32)
  f[:int(2 / 3 * n) // 2, :int(2 / 3 * (m // 2 + 1))] = 1
  f[-int(2 / 3 * n) // 2:, :int(2 / 3 * (m // 2 + 1))] = 1
  dev = grids.default_device() if device is None else device
  return torch.from_numpy(f).to(dev)


def vorticity_to_velocity(grid: grids.Grid):
  """spectral/utils.py:154-189: (vx_hat, vy_hat) from vorticity_hat."""
  kx, ky = np.meshgrid(*grid.rfft_axes_numpy(), indexing='ij')
  two_pi_i = 2 * np.pi * 1j
  laplace = (two_pi_i ** 2 * (abs(kx) ** 2 + abs(ky) ** 2)).astype(np.complex64)
  laplace[0, 0] = 1

  def ret(vorticity_hat: torch.Tensor):
    dev = vorticity_hat.device
    lap = torch.from_numpy(laplace).to(dev)
    kxt = torch.from_numpy(kx).to(dev)
    kyt = torch.from_numpy(ky).to(dev)
    psi_hat = -1 / lap * vorticity_hat
    vxhat = two_pi_i * kyt * psi_hat
    vyhat = -two_pi_i * kxt * psi_hat
    return vxhat, vyhat
  return ret


def spectral_curl_2d(mesh, velocity_hat):
  """spectral/utils.py:199-203."""
  kx, ky = mesh
  uhat, vhat = velocity_hat
  return 2j * np.pi * (vhat * kx - uhat * ky)


def _plan(grid: grids.Grid, device):
  return plans.cached('spec-fft', (device, grid.shape, grid.step),
                      lambda: plans.SpecPlan(grid.shape, grid.step, device=device))


def rfft2(x: torch.Tensor, grid: grids.Grid) -> torch.Tensor:
  """jnp.fft.rfftn of a real [nx, ny] field with the native transforms."""
  return _plan(grid, x.device).rfft2(x.contiguous())


def irfft2(xhat: torch.Tensor, grid: grids.Grid) -> torch.Tensor:
  """jnp.fft.irfftn back to a real [nx, ny] field with the native transforms."""
  return _plan(grid, xhat.device).irfft2(xhat.contiguous())
