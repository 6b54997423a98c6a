"""Explicit diffusion, mirroring ``jax_cfd/base/diffusion.py:35-57``.

The fused step recognises ``diffuse=diffusion.diffuse``; called on its own,
``diffuse`` is the device torch expression of ``nu * laplacian(c)``.
"""
from __future__ import annotations

from jax_cfd_gb300.base import finite_differences as fd
from jax_cfd_gb300.base import grids


def diffuse(c: grids.GridVariable, nu: float) -> grids.GridArray:
  """diffusion.py:35-37."""
  return nu * fd.laplacian(c)


def stable_time_step(viscosity: float, grid: grids.Grid) -> float:
  """diffusion.py:40-57."""
  if viscosity == 0:
    return float('inf')
  dx = min(grid.step)
  ndim = grid.ndim
  return dx ** 2 / (viscosity * 2 ** ndim)


def solve_fast_diag(v, nu, dt, implementation=None):
  """Implicit diffusion (diffusion.py:166-212) is not on the GB300 hot path."""
  raise NotImplementedError('implicit diffusion is outside the GB300 hot path')


def solve_cg(v, nu, dt, *args, **kwargs):
  raise NotImplementedError('implicit diffusion is outside the GB300 hot path')
