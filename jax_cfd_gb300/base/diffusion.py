"""Diffusion, mirroring ``jax_cfd/base/diffusion.py``.

The fused step recognises ``diffuse=diffusion.diffuse``; called on its own,
``diffuse`` is the device torch expression of ``nu * laplacian(c)``.
``solve_fast_diag`` (implicit diffusion, diffusion.py:166-212) runs on the
native real-FFT transforms of the pressure solve.
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
  """diffusion.py:166-212 for periodic velocity tuples on the native rfft
  transforms: u + irfftn(func(lambda) rfftn(u)) per component, func(x) =
  (dt nu) x / (1 - (dt nu) x).  ``implementation`` may be None or 'rfft'
  (the reference's default for periodic grids with an even last axis)."""
  # pylint: disable=import-outside-toplevel
  from jax_cfd_gb300 import plans
  from jax_cfd_gb300.base import boundaries
  if implementation not in (None, 'rfft'):
    raise NotImplementedError(f'implementation={implementation!r} is outside the GB300 path')
  if len(v) != 2 or v[0].grid.ndim != 2:
    raise NotImplementedError('only 2-D grids are on the GB300 hot path')
  if not boundaries.has_all_periodic_boundary_conditions(*v):
    raise NotImplementedError('Non-periodic boundary conditions are not implemented.')
  grid = v[0].grid
  dev = v[0].data.device
  plan = plans.cached('fvm-diffusion', (dev, grid.shape, grid.step),
                      lambda: plans.FvmPlan(grid.shape, grid.step, device=dev))
  uo, vo = plan.diffusion_solve(v[0].data, v[1].data, float(nu), float(dt))
  return tuple(grids.GridVariable(grids.GridArray(o, u.offset, grid), u.bc)
               for o, u in zip((uo, vo), v))


def solve_cg(v, nu, dt, *args, **kwargs):
  raise NotImplementedError('implicit diffusion is outside the GB300 hot path')
