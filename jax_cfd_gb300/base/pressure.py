"""Pressure projection, mirroring ``jax_cfd/base/pressure.py``.

``solve_fast_diag`` (pressure.py:115-157) and ``projection`` (181-198) run the
native real-FFT fast-diagonalisation kernels: backward-difference divergence,
packed row rFFT, column FFT * pinv(lambda) * inverse column FFT, row irFFT,
then ``v - forward_difference(q)``.
"""
from __future__ import annotations

from typing import Callable, Optional

from jax_cfd_gb300 import plans
from jax_cfd_gb300.base import boundaries
from jax_cfd_gb300.base import grids

GridArray = grids.GridArray
GridVariable = grids.GridVariable


def _check_velocity(v):
  grid = grids.consistent_grid(*v)
  if grid.ndim != 2 or len(v) != 2:
    raise NotImplementedError('only 2-D grids are on the GB300 hot path')
  if not boundaries.has_all_periodic_boundary_conditions(*v):
    raise NotImplementedError('non-periodic pressure solves are outside the GB300 hot path')
  if tuple(v[0].offset) != (1.0, 0.5) or tuple(v[1].offset) != (0.5, 1.0):
    raise grids.InconsistentOffsetError(
        f'velocity must sit on the cell faces, got {v[0].offset}, {v[1].offset}')
  return grid


def _plan(grid: grids.Grid, device):
  return plans.cached('fvm-pressure', (device, grid.shape, grid.step),
                      lambda: plans.FvmPlan(grid.shape, grid.step, device=device))


def solve_fast_diag(v, q0: Optional[GridArray] = None, pressure_bc=None,
                    implementation: Optional[str] = None) -> GridArray:
  """Pressure correction q with div(v - grad q) = 0 (pressure.py:115-157).

  ``implementation`` is accepted for signature compatibility; periodic grids
  always use the real-FFT diagonalisation, which is the reference's default
  off-TPU (fast_diagonalization.py:101-108).
  """
  del q0, implementation
  grid = _check_velocity(v)
  if pressure_bc is not None and not all(
      t == (boundaries.BCType.PERIODIC,) * 2 for t in pressure_bc.types):
    raise NotImplementedError('non-periodic pressure boundary conditions')
  plan = _plan(grid, v[0].data.device)
  return GridArray(plan.pressure_solve(v[0].data, v[1].data), grid.cell_center, grid)


def solve_cg(v, q0, pressure_bc=None, rtol=1e-6, atol=1e-6, maxiter=None):
  """Conjugate-gradient pressure solves are outside the GB300 hot path."""
  raise NotImplementedError('solve_cg is outside the GB300 hot path; use solve_fast_diag')


def projection(v, solve: Callable = solve_fast_diag):
  """pressure.py:181-198."""
  if solve is not solve_fast_diag:
    raise NotImplementedError('the GB300 projection uses solve_fast_diag')
  grid = _check_velocity(v)
  plan = _plan(grid, v[0].data.device)
  uo, vo = plan.projection(v[0].data, v[1].data)
  return (GridVariable(GridArray(uo, v[0].offset, grid), v[0].bc),
          GridVariable(GridArray(vo, v[1].offset, grid), v[1].bc))
