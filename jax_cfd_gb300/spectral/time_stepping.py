"""Implicit-explicit time stepping, mirroring ``jax_cfd/spectral/time_stepping.py``.

``low_storage_runge_kutta_crank_nicolson`` (time_stepping.py:117-170) and its
named tableaux return a native step: each stage is a row pass (four inverse
real FFTs, the advection product, one forward real FFT) and a column pass
(x-FFT, 2/3 filter, forcing, the stage update, and the next stage's inverse
x-FFTs).
"""
from __future__ import annotations

from typing import Callable, Sequence

import torch

from jax_cfd_gb300 import plans
from jax_cfd_gb300.spectral import equations as spectral_equations


class ImplicitExplicitODE:
  """time_stepping.py:23-53 (interface only)."""

  def explicit_terms(self, state):
    raise NotImplementedError

  def implicit_terms(self, state):
    raise NotImplementedError

  def implicit_solve(self, state, step_size):
    raise NotImplementedError


class SpectralStep:
  """A native low-storage RK/CN step of ``NavierStokes2D``."""

  def __init__(self, equation, time_step, alphas, betas, gammas):
    if not isinstance(equation, spectral_equations.NavierStokes2D):
      raise NotImplementedError('the GB300 spectral step runs NavierStokes2D')
    if len(alphas) - 1 != len(betas) or len(betas) != len(gammas):
      raise ValueError('number of RK coefficients does not match')
    self.equation = equation
    self.time_step = float(time_step)
    self.coefficients = (tuple(alphas), tuple(betas), tuple(gammas))

  def plan(self, device) -> plans.SpecPlan:
    eq = self.equation
    return plans.cached(
        'spec-step', (device, eq.grid.shape, eq.grid.step, float(eq.viscosity),
                      float(eq.drag), eq.smooth is not None, eq.forcing_key(device),
                      self.time_step,
                      self.coefficients),
        lambda: spectral_equations._make_plan(eq, device, self.time_step,
                                              *self.coefficients))

  def gb300_repeat(self, vorticity_hat: torch.Tensor, steps: int) -> torch.Tensor:
    return self.plan(vorticity_hat.device).step(vorticity_hat, steps)

  def __call__(self, vorticity_hat: torch.Tensor) -> torch.Tensor:
    return self.gb300_repeat(vorticity_hat, 1)


def low_storage_runge_kutta_crank_nicolson(alphas: Sequence[float],
                                           betas: Sequence[float],
                                           gammas: Sequence[float], equation,
                                           time_step: float) -> Callable:
  """time_stepping.py:117-170."""
  return SpectralStep(equation, time_step, alphas, betas, gammas)


def crank_nicolson_rk3(equation, time_step: float) -> Callable:
  """time_stepping.py:173-183 ("Williamson")."""
  return low_storage_runge_kutta_crank_nicolson(
      alphas=[0, 1 / 3, 3 / 4, 1], betas=[0, -5 / 9, -153 / 128],
      gammas=[1 / 3, 15 / 16, 8 / 15], equation=equation, time_step=time_step)


# (alphas, betas, gammas) of crank_nicolson_rk4 (time_stepping.py:186-197,
# "Carpenter-Kennedy").
CN_RK4_COEFFICIENTS = (
    (0, 0.1496590219993, 0.3704009573644, 0.6222557631345, 0.9582821306748, 1),
    (0, -0.4178904745, -1.192151694643, -1.697784692471, -1.514183444257),
    (0.1496590219993, 0.3792103129999, 0.8229550293869, 0.6994504559488, 0.1530572479681),
)


def crank_nicolson_rk4(equation, time_step: float) -> Callable:
  """time_stepping.py:186-197 ("Carpenter-Kennedy")."""
  alphas, betas, gammas = CN_RK4_COEFFICIENTS
  return low_storage_runge_kutta_crank_nicolson(
      alphas=list(alphas), betas=list(betas), gammas=list(gammas),
      equation=equation, time_step=time_step)
