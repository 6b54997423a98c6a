"""Explicit Runge-Kutta time stepping, mirroring ``jax_cfd/base/time_stepping.py``.

``forward_euler(equation, dt)`` applied to the equation built by
``equations.semi_implicit_navier_stokes`` returns the fused GB300 step
(the projection of step k folded into the stencil of step k + 1).  The other
explicit tableaux (``midpoint_rk2``, ``heun_rk2``, ``classic_rk4`` or any
``ButcherTableau`` of up to four stages) run ``navier_stokes_rk`` on the same
kernels: the stencil in explicit-terms mode, the stage combinations in the
reference's order and a projection per stage.
"""
from __future__ import annotations

import dataclasses
from typing import Callable, Sequence


class ExplicitNavierStokesODE:
  """time_stepping.py:26-45: explicit terms plus a projection."""

  def __init__(self, explicit_terms, pressure_projection):
    self.explicit_terms = explicit_terms
    self.pressure_projection = pressure_projection


@dataclasses.dataclass
class ButcherTableau:
  """time_stepping.py:48-57."""
  a: Sequence[Sequence[float]]
  b: Sequence[float]

  def __post_init__(self):
    if len(self.a) + 1 != len(self.b):
      raise ValueError('inconsistent Butcher tableau')


FORWARD_EULER = ButcherTableau(a=[], b=[1])
MIDPOINT_RK2 = ButcherTableau(a=[[1 / 2]], b=[0, 1])
HEUN_RK2 = ButcherTableau(a=[[1]], b=[1 / 2, 1 / 2])
CLASSIC_RK4 = ButcherTableau(a=[[1 / 2], [0, 1 / 2], [0, 0, 1]],
                             b=[1 / 6, 1 / 3, 1 / 3, 1 / 6])


def navier_stokes_rk(tableau: ButcherTableau, equation, time_step: float) -> Callable:
  """time_stepping.py:59-107."""
  builder = getattr(equation, 'gb300_step', None)
  if builder is None:
    raise NotImplementedError(
        'the GB300 time stepper runs equations built by '
        'equations.semi_implicit_navier_stokes')
  return builder(tableau, time_step)


def forward_euler(equation, time_step: float) -> Callable:
  """time_stepping.py:109-119."""
  return navier_stokes_rk(FORWARD_EULER, equation, time_step)


def midpoint_rk2(equation, time_step: float) -> Callable:
  """time_stepping.py:121-131."""
  return navier_stokes_rk(MIDPOINT_RK2, equation, time_step)


def heun_rk2(equation, time_step: float) -> Callable:
  """time_stepping.py:134-144."""
  return navier_stokes_rk(HEUN_RK2, equation, time_step)


def classic_rk4(equation, time_step: float) -> Callable:
  """time_stepping.py:147-158."""
  return navier_stokes_rk(CLASSIC_RK4, equation, time_step)
