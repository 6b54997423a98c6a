"""Advection, mirroring the hot-path part of ``jax_cfd/base/advection.py``.

The fused step recognises ``convect=None`` (Van Leer via
``advect_van_leer_using_limiters``, advection.py:387-395, the reference
default) and ``convect=convect_linear`` (advection.py:183-207).  Called on
their own these functions run the same native stencil with diffusion and
forcing switched off.
"""
from __future__ import annotations

from typing import Optional

from jax_cfd_gb300 import _native as nat
from jax_cfd_gb300 import plans
from jax_cfd_gb300.base import boundaries
from jax_cfd_gb300.base import grids

GridArray = grids.GridArray
GridVariable = grids.GridVariable


def _native_advection(c: GridVariable, v, dt: float, convect: int) -> GridArray:
  if not boundaries.has_all_periodic_boundary_conditions(c, *v):
    raise NotImplementedError('Non-periodic boundary conditions are not implemented.')
  grid = grids.consistent_grid(c, *v)
  if len(v) != 2 or grid.ndim != 2:
    raise NotImplementedError('only 2-D staggered velocities are on the GB300 path')
  index = next((i for i, u in enumerate(v) if u is c), None)
  if index is None:
    raise NotImplementedError('the fused stencil advects the velocity components themselves')
  dev = v[0].data.device
  plan = plans.cached('fvm-adv', (dev, grid.shape, grid.step, float(dt or 0.0), convect),
                      lambda: plans.FvmPlan(grid.shape, grid.step, dt=float(dt or 0.0),
                                            convect=convect, device=dev))
  du, dv = plan.explicit_terms(v[0].data, v[1].data)
  return GridArray((du, dv)[index], c.offset, grid)


def advect_van_leer_using_limiters(c: GridVariable, v, dt: float) -> GridArray:
  """advection.py:387-395."""
  return _native_advection(c, v, dt, nat.CONVECT_VAN_LEER)


def advect_linear(c: GridVariable, v, dt: Optional[float] = None) -> GridArray:
  """advection.py:119-126."""
  return _native_advection(c, v, dt, nat.CONVECT_LINEAR)


def convect_linear(v):
  """advection.py:183-207 (self-advection with linear interpolation)."""
  return tuple(advect_linear(u, v) for u in v)


def stable_time_step(max_velocity: float, max_courant_number: float,
                     grid: grids.Grid) -> float:
  """advection.py:398-416."""
  dx = min(grid.step)
  return max_courant_number * dx / max_velocity
