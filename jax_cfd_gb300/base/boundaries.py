"""Boundary conditions, mirroring the periodic subset of
``jax_cfd/base/boundaries.py`` (the only boundary on the hot path).

Non-periodic types can be constructed (so callers that build them keep
working) but the GB300 step and projection reject them with
``NotImplementedError``, like ``advection.advect_general`` does in the
reference (advection.py:108-110).
"""
from __future__ import annotations

import dataclasses
from typing import Sequence, Tuple

import torch

from jax_cfd_gb300.base import grids


class BCType:
  PERIODIC = 'periodic'
  DIRICHLET = 'dirichlet'
  NEUMANN = 'neumann'


@dataclasses.dataclass(init=False, frozen=True)
class ConstantBoundaryConditions:
  """Boundary conditions with constant values (boundaries.py:47-180)."""
  types: Tuple[Tuple[str, str], ...]
  bc_values: Tuple[Tuple[float, float], ...]

  def __init__(self, types: Sequence[Tuple[str, str]],
               values: Sequence[Tuple[float, float]]):
    object.__setattr__(self, 'types', tuple(tuple(t) for t in types))
    object.__setattr__(self, 'bc_values', tuple(tuple(v) for v in values))

  def shift(self, u: grids.GridArray, offset: int, axis: int) -> grids.GridArray:
    """Periodic shift (pad 'wrap' then trim): result[i] = u[i + offset]."""
    if self.types[axis][0] != BCType.PERIODIC:
      raise NotImplementedError('only periodic shifts are on the GB300 path')
    new_offset = tuple(o + offset if i == axis else o for i, o in enumerate(u.offset))
    return grids.GridArray(torch.roll(u.data, -offset, dims=axis), new_offset, u.grid)

  def impose_bc(self, u: grids.GridArray) -> grids.GridVariable:
    """boundaries.py:514-530: a no-op for periodic boundaries."""
    return grids.GridVariable(u, self)

  def trim_boundary(self, u: grids.GridArray) -> grids.GridArray:
    return u


def periodic_boundary_conditions(ndim: int) -> ConstantBoundaryConditions:
  """boundaries.py:556-559."""
  return ConstantBoundaryConditions(((BCType.PERIODIC, BCType.PERIODIC),) * ndim,
                                    ((0.0, 0.0),) * ndim)


def dirichlet_boundary_conditions(ndim: int, bc_vals=None) -> ConstantBoundaryConditions:
  if bc_vals is None:
    bc_vals = ((0.0, 0.0),) * ndim
  return ConstantBoundaryConditions(((BCType.DIRICHLET, BCType.DIRICHLET),) * ndim, bc_vals)


def neumann_boundary_conditions(ndim: int, bc_vals=None) -> ConstantBoundaryConditions:
  if bc_vals is None:
    bc_vals = ((0.0, 0.0),) * ndim
  return ConstantBoundaryConditions(((BCType.NEUMANN, BCType.NEUMANN),) * ndim, bc_vals)


def has_all_periodic_boundary_conditions(*arrays) -> bool:
  """boundaries.py:693-700."""
  for array in arrays:
    for lower, upper in array.bc.types:
      if lower != BCType.PERIODIC or upper != BCType.PERIODIC:
        return False
  return True


def get_pressure_bc_from_velocity(v) -> ConstantBoundaryConditions:
  """boundaries.py:724-735 (periodic velocity gives periodic pressure)."""
  if not has_all_periodic_boundary_conditions(*v):
    raise NotImplementedError('only periodic velocity boundaries are supported')
  return periodic_boundary_conditions(len(v))
