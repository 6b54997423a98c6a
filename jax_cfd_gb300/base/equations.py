"""Navier-Stokes equations, mirroring ``jax_cfd/base/equations.py``.

``semi_implicit_navier_stokes`` (equations.py:120-151) and
``implicit_diffusion_navier_stokes`` (154-195) keep the reference signatures
and return step functions backed by the fused GB300 kernels.  The arguments are pattern-matched onto the kernels: the
default Van Leer convection (or ``advection.convect_linear``),
``diffusion.diffuse``, ``pressure.solve_fast_diag``, forcings built by
``forcings`` and ``time_stepping.forward_euler``.  Anything else raises
``NotImplementedError`` -- there is no non-native fallback.
"""
from __future__ import annotations

from typing import Callable, Optional

from jax_cfd_gb300 import _native as nat
from jax_cfd_gb300 import plans
from jax_cfd_gb300.base import advection
from jax_cfd_gb300.base import boundaries
from jax_cfd_gb300.base import diffusion
from jax_cfd_gb300.base import forcings as forcings_lib
from jax_cfd_gb300.base import grids
from jax_cfd_gb300.base import pressure
from jax_cfd_gb300.base import time_stepping

GridArray = grids.GridArray
GridVariable = grids.GridVariable


def sum_fields(*args):
  """equations.py:41-42: elementwise sum starting from 0."""
  out = []
  for comp in zip(*args):
    acc = 0
    for a in comp:
      acc = acc + a
    out.append(acc)
  return tuple(out)


def stable_time_step(max_velocity: float, max_courant_number: float,
                     viscosity: float, grid: grids.Grid,
                     implicit_diffusion: bool = False) -> float:
  """equations.py:45-59 (raises when explicit diffusion needs a smaller dt)."""
  dt = advection.stable_time_step(max_velocity, max_courant_number, grid)
  if not implicit_diffusion:
    diffusion_dt = diffusion.stable_time_step(viscosity, grid)
    if diffusion_dt < dt:
      raise ValueError(f'stable time step for diffusion is smaller than '
                       f'the chosen timestep: {diffusion_dt} vs {dt}')
  return dt


def dynamic_time_step(v, max_courant_number: float, viscosity: float,
                      grid: grids.Grid, implicit_diffusion: bool = False) -> float:
  """equations.py:62-70 (v_max from the native max-speed reduction)."""
  v_max = float(plans.max_speed(v[0].data, v[1].data))
  return stable_time_step(v_max, max_courant_number, viscosity, grid,
                          implicit_diffusion)


def _check_state(v, grid: grids.Grid):
  if len(v) != 2 or grid.ndim != 2:
    raise NotImplementedError('only 2-D grids are on the GB300 hot path')
  if not boundaries.has_all_periodic_boundary_conditions(*v):
    raise NotImplementedError('Non-periodic boundary conditions are not implemented.')
  for u, o in zip(v, grid.cell_faces):
    if tuple(u.offset) != tuple(o):
      raise grids.InconsistentOffsetError(f'expected offset {o}, got {u.offset}')
    if u.grid != grid:
      raise grids.InconsistentGridError('velocity lives on another grid')


class FvmStep:
  """One fused forward-Euler step of ``semi_implicit_navier_stokes``.

  Calling it advances a velocity tuple by one step; ``gb300_repeat`` (used by
  ``funcutils.repeated``) advances it by many steps in one native call, with
  the projection of step k folded into the stencil of step k + 1.
  """

  def __init__(self, grid: grids.Grid, tableau=None, implicit_viscosity=None,
               **plan_kwargs):
    self.grid = grid
    self._plan_kwargs = plan_kwargs
    self._key = tuple(sorted((k, _freeze(v)) for k, v in plan_kwargs.items()))
    # None: the fused forward-Euler step; else (a, b) of navier_stokes_rk.
    self.tableau = tableau
    # Not None: implicit_diffusion_navier_stokes with this viscosity (the
    # plan's explicit terms then carry no diffusion).
    self.implicit_viscosity = implicit_viscosity

  def plan(self, device) -> plans.FvmPlan:
    return plans.cached('fvm-step', (device, self.grid.shape, self.grid.step, self._key),
                        lambda: plans.FvmPlan(self.grid.shape, self.grid.step,
                                              device=device, **self._plan_kwargs))

  def gb300_repeat(self, v, steps: int):
    _check_state(v, self.grid)
    plan = self.plan(v[0].data.device)
    if self.implicit_viscosity is not None:
      uo, vo = plan.step_implicit(v[0].data, v[1].data, steps, self.implicit_viscosity)
    elif self.tableau is None:
      uo, vo = plan.step(v[0].data, v[1].data, steps)
    else:
      uo, vo = plan.step_rk(v[0].data, v[1].data, steps, *self.tableau)
    return (GridVariable(GridArray(uo, v[0].offset, self.grid), v[0].bc),
            GridVariable(GridArray(vo, v[1].offset, self.grid), v[1].bc))

  def explicit_terms(self, v):
    _check_state(v, self.grid)
    du, dv = self.plan(v[0].data.device).explicit_terms(v[0].data, v[1].data)
    return (GridVariable(GridArray(du, v[0].offset, self.grid), v[0].bc),
            GridVariable(GridArray(dv, v[1].offset, self.grid), v[1].bc))

  def __call__(self, v):
    return self.gb300_repeat(v, 1)


def _freeze(x):
  if x is None or isinstance(x, (int, float, str)):
    return x
  try:
    import numpy as np  # pylint: disable=import-outside-toplevel
    a = np.asarray(x)
    return (a.shape, a.tobytes())
  except Exception:  # pylint: disable=broad-except
    return id(x)


class _FusedEquation:
  """What ``semi_implicit_navier_stokes`` hands to its time stepper."""

  def __init__(self, grid, dt, plan_kwargs, explicit_terms, pressure_projection):
    self.grid = grid
    self.dt = dt
    self.plan_kwargs = plan_kwargs
    self.explicit_terms = explicit_terms
    self.pressure_projection = pressure_projection

  def gb300_step(self, tableau, time_step):
    if float(time_step) != float(self.dt):
      raise NotImplementedError('time_step must equal the dt given to the equation')
    a = [list(row) for row in tableau.a]
    b = list(tableau.b)
    if (a, b) == ([], [1]):
      # forward_euler: the fused step (projection folded into the next stencil).
      return FvmStep(self.grid, dt=float(time_step), **self.plan_kwargs)
    if not 1 <= len(b) <= 4:
      raise NotImplementedError('the GB300 Runge-Kutta step takes tableaux of 1 to 4 stages')
    return FvmStep(self.grid, tableau=(a, b), dt=float(time_step), **self.plan_kwargs)


def _convect_kind(convect) -> int:
  if convect is None:
    return nat.CONVECT_VAN_LEER
  if convect is advection.convect_linear:
    return nat.CONVECT_LINEAR
  raise NotImplementedError(
      'convect must be None (Van Leer via advect_van_leer_using_limiters) or '
      'advection.convect_linear on the GB300 path')


def _plan_kwargs(density, viscosity, convect, diffuse, forcing):
  if diffuse is not diffusion.diffuse:
    raise NotImplementedError('diffuse must be diffusion.diffuse on the GB300 path')
  kw = dict(density=float(density),
            viscosity=None if viscosity is None else float(viscosity),
            convect=_convect_kind(convect))
  kw.update(forcings_lib.fused_descriptor(forcing))
  return kw


def navier_stokes_explicit_terms(density: float, viscosity: float, dt: float,
                                 grid: grids.Grid, convect=None,
                                 diffuse=diffusion.diffuse,
                                 forcing=None) -> Callable:
  """equations.py:77-116: du/dt without the projection (native stencil)."""
  step = FvmStep(grid, dt=float(dt),
                 **_plan_kwargs(density, viscosity, convect, diffuse, forcing))
  return step.explicit_terms


def semi_implicit_navier_stokes(density: float, viscosity: float, dt: float,
                                grid: grids.Grid, convect=None,
                                diffuse=diffusion.diffuse,
                                pressure_solve: Callable = pressure.solve_fast_diag,
                                forcing=None,
                                time_stepper: Callable = time_stepping.forward_euler
                                ) -> Callable:
  """equations.py:120-151."""
  if pressure_solve is not pressure.solve_fast_diag:
    raise NotImplementedError('pressure_solve must be pressure.solve_fast_diag on the GB300 path')
  kw = _plan_kwargs(density, viscosity, convect, diffuse, forcing)
  explicit = navier_stokes_explicit_terms(density, viscosity, dt, grid, convect,
                                          diffuse, forcing)
  eq = _FusedEquation(grid, dt, kw, explicit,
                      lambda v: pressure.projection(v, pressure_solve))
  return time_stepper(eq, dt)


def implicit_diffusion_navier_stokes(density: float, viscosity: float, dt: float,
                                     grid: grids.Grid, convect=None,
                                     diffusion_solve: Callable = diffusion.solve_fast_diag,
                                     pressure_solve: Callable = pressure.solve_fast_diag,
                                     forcing=None) -> Callable:
  """equations.py:154-195: v + dt (convection + forcing / density), the
  projection, then diffusion_solve(v, viscosity, dt), as one native step
  (cfd_fvm_step_implicit)."""
  if diffusion_solve is not diffusion.solve_fast_diag:
    raise NotImplementedError('diffusion_solve must be diffusion.solve_fast_diag on the GB300 path')
  if pressure_solve is not pressure.solve_fast_diag:
    raise NotImplementedError('pressure_solve must be pressure.solve_fast_diag on the GB300 path')
  kw = _plan_kwargs(density, None, convect, diffusion.diffuse, forcing)
  return FvmStep(grid, implicit_viscosity=float(viscosity), dt=float(dt), **kw)
