"""Pseudospectral equations, mirroring ``jax_cfd/spectral/equations.py:129-220``.

``NavierStokes2D`` keeps the reference's fields and methods; its stepping is
done by the native plan built in ``spectral.time_stepping``.  The explicit,
implicit and implicit-solve terms are also callable on their own: the first
through the native kernels, the other two as device elementwise expressions.
"""
from __future__ import annotations

import dataclasses
import hashlib
from typing import Callable, Optional

import numpy as np
import torch

from jax_cfd_gb300 import plans
from jax_cfd_gb300.base import boundaries
from jax_cfd_gb300.base import forcings
from jax_cfd_gb300.base import grids
from jax_cfd_gb300.spectral import utils as spectral_utils


@dataclasses.dataclass
class NavierStokes2D:
  """spectral/equations.py:129-191.

  Attributes:
    viscosity: strength of the diffusion term
    grid: underlying grid of the process
    drag: strength of the drag. Set to zero for no drag.
    smooth: smooth the advection term using the 2/3-rule (applied unless
      ``smooth is None``, as in the reference).
    forcing_fn: function of the grid returning a velocity-independent forcing.
  """
  viscosity: float
  grid: grids.Grid
  drag: float = 0.
  smooth: bool = True
  forcing_fn: Optional[Callable[[grids.Grid], Callable]] = None

  def __post_init__(self):
    if self.grid.ndim != 2:
      raise NotImplementedError('only 2-D grids are on the GB300 hot path')
    self._forcing_fn_with_grid = (self.forcing_fn(self.grid)
                                  if self.forcing_fn is not None else None)

  # -- tables (host float32, like jnp with x64 off) ------------------------
  def kx_ky(self):
    kx, ky = np.meshgrid(*self.grid.rfft_axes_numpy(), indexing='ij')
    return kx, ky

  def linear_term_numpy(self) -> np.ndarray:
    kx, ky = self.kx_ky()
    laplace = (np.pi * 2j) ** 2 * (kx ** 2 + ky ** 2)
    return self.viscosity * laplace - self.drag

  def forcing_fields(self, device):
    """Velocity-independent forcing (fx, fy) as device float32 fields, or None."""
    f = self._forcing_fn_with_grid
    if f is None:
      return None
    if isinstance(f, forcings.ForcingFn):
      if not f.velocity_independent:
        raise NotImplementedError('the GB300 spectral step supports velocity-independent forcings')
      fu, fv = f.constant_fields()
    else:
      # Arbitrary forcing callables are evaluated once, on a zero velocity;
      # the spectral step treats the result as constant.
      nx, ny = self.grid.shape
      bc = boundaries.periodic_boundary_conditions(2)
      z = tuple(grids.GridVariable(grids.GridArray(
          torch.zeros(nx, ny, device=device), (0.5, 0.5), self.grid), bc) for _ in range(2))
      fx, fy = f(z)
      return fx.data.float().contiguous(), fy.data.float().contiguous()
    to = lambda a: None if a is None else torch.from_numpy(np.ascontiguousarray(a, np.float32)).to(device)
    return to(fu), to(fv)

  def forcing_key(self, device) -> Optional[str]:
    """Content fingerprint of the forcing fields (part of the plan cache key:
    equations with equal forcing share plans, and a plan is never reused for
    a different forcing)."""
    key = getattr(self, '_forcing_key', None)
    if key is None:
      fields = self.forcing_fields(device)
      if fields is None:
        key = 'none'
      else:
        h = hashlib.sha1()
        for f in fields:
          h.update(b'-' if f is None else f.detach().float().contiguous().cpu().numpy().tobytes())
        key = h.hexdigest()
      self._forcing_key = key
    return key

  def _plan(self, device) -> plans.SpecPlan:
    return plans.cached(
        'spec-terms', (device, self.grid.shape, self.grid.step, float(self.viscosity),
                       float(self.drag), self.smooth is not None, self.forcing_key(device)),
        lambda: _make_plan(self, device, 0.0, (0., 1.), (0.,), (1.,)))

  def explicit_terms(self, vorticity_hat: torch.Tensor) -> torch.Tensor:
    """spectral/equations.py:160-184 (native)."""
    return self._plan(vorticity_hat.device).explicit_terms(vorticity_hat)

  def implicit_terms(self, vorticity_hat: torch.Tensor) -> torch.Tensor:
    lin = torch.from_numpy(self.linear_term_numpy().astype(np.complex64)).to(vorticity_hat.device)
    return lin * vorticity_hat

  def implicit_solve(self, vorticity_hat: torch.Tensor, time_step: float) -> torch.Tensor:
    lin = torch.from_numpy(self.linear_term_numpy().astype(np.complex64)).to(vorticity_hat.device)
    return 1 / (1 - time_step * lin) * vorticity_hat


def _make_plan(eq: NavierStokes2D, device, dt, alphas, betas, gammas) -> plans.SpecPlan:
  plan = plans.SpecPlan(eq.grid.shape, eq.grid.step, viscosity=float(eq.viscosity),
                        drag=float(eq.drag), dt=float(dt),
                        smooth=eq.smooth is not None, alphas=alphas, betas=betas,
                        gammas=gammas, device=device)
  fields = eq.forcing_fields(device)
  if fields is not None:
    plan.set_forcing(*fields)
  return plan


def ForcedNavierStokes2D(viscosity, grid, smooth):  # pylint: disable=invalid-name
  """spectral/equations.py:194-220: Kolmogorov k=4 at offsets 0, drag 0.1."""
  wave_number = 4
  offsets = ((0, 0), (0, 0))
  forcing_fn = lambda grid: forcings.kolmogorov_forcing(grid, k=wave_number, offsets=offsets)
  return NavierStokes2D(viscosity, grid, drag=0.1, smooth=smooth, forcing_fn=forcing_fn)
