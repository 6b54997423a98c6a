"""Finite differences, mirroring ``jax_cfd/base/finite_differences.py``.

``divergence`` and ``curl_2d`` of a periodic 2-D velocity run as native
kernels; the single-array differences are torch ops on the device.
"""
from __future__ import annotations

from typing import Sequence, Tuple

import numpy as np
import torch

from jax_cfd_gb300 import plans
from jax_cfd_gb300.base import boundaries
from jax_cfd_gb300.base import grids

GridArray = grids.GridArray
GridVariable = grids.GridVariable


def stencil_sum(*arrays: GridArray) -> GridArray:
  """finite_differences.py:44-54."""
  offset = grids.averaged_offset(*arrays)
  result = 0
  for a in arrays:
    result = result + a.data
  return GridArray(result, offset, grids.consistent_grid(*arrays))


def central_difference(u: GridVariable, axis=None):
  if axis is None:
    axis = range(u.grid.ndim)
  if not isinstance(axis, int):
    return tuple(central_difference(u, a) for a in axis)
  diff = stencil_sum(u.shift(+1, axis), -u.shift(-1, axis))
  return diff / (2 * u.grid.step[axis])


def backward_difference(u: GridVariable, axis=None):
  """finite_differences.py:95-102."""
  if axis is None:
    axis = range(u.grid.ndim)
  if not isinstance(axis, int):
    return tuple(backward_difference(u, a) for a in axis)
  diff = stencil_sum(u.array, -u.shift(-1, axis))
  return diff / u.grid.step[axis]


def forward_difference(u: GridVariable, axis=None):
  """finite_differences.py:117-124."""
  if axis is None:
    axis = range(u.grid.ndim)
  if not isinstance(axis, int):
    return tuple(forward_difference(u, a) for a in axis)
  diff = stencil_sum(u.shift(+1, axis), -u.array)
  return diff / u.grid.step[axis]


def laplacian(u: GridVariable) -> GridArray:
  """finite_differences.py:127-133."""
  scales = np.square(1 / np.array(u.grid.step, dtype=np.float32))
  result = -2 * u.array * float(np.sum(scales))
  for axis in range(u.grid.ndim):
    result = result + stencil_sum(u.shift(-1, axis), u.shift(+1, axis)) * float(scales[axis])
  return result


def _plan_for(grid: grids.Grid, device):
  return plans.cached('fvm-diag', (device, grid.shape, grid.step),
                      lambda: plans.FvmPlan(grid.shape, grid.step, device=device))


def _native_2d(v: Sequence[GridVariable]) -> bool:
  return (len(v) == 2 and v[0].grid.ndim == 2 and v[0].data.is_cuda
          and boundaries.has_all_periodic_boundary_conditions(*v)
          and tuple(v[0].offset) == (1.0, 0.5) and tuple(v[1].offset) == (0.5, 1.0))


def divergence(v: Sequence[GridVariable]) -> GridArray:
  """finite_differences.py:136-143 (backward differences)."""
  grid = grids.consistent_grid(*v)
  if len(v) != grid.ndim:
    raise ValueError('The length of `v` must be equal to `grid.ndim`.'
                     f'Expected length {grid.ndim}; got {len(v)}.')
  if _native_2d(v):
    plan = _plan_for(grid, v[0].data.device)
    return GridArray(plan.divergence(v[0].data, v[1].data), grid.cell_center, grid)
  differences = [backward_difference(u, axis) for axis, u in enumerate(v)]
  out = differences[0]
  for d in differences[1:]:
    out = out + d
  return out


def curl_2d(v: Sequence[GridVariable]) -> GridArray:
  """finite_differences.py:186-193; result at offset (1, 1)."""
  if len(v) != 2:
    raise ValueError(f'Length of `v` is not 2: {len(v)}')
  grid = grids.consistent_grid(*v)
  if grid.ndim != 2:
    raise ValueError(f'Grid dimensionality is not 2: {grid.ndim}')
  if _native_2d(v):
    plan = _plan_for(grid, v[0].data.device)
    return GridArray(plan.curl_2d(v[0].data, v[1].data), (1.0, 1.0), grid)
  return forward_difference(v[1], axis=0) - forward_difference(v[0], axis=1)
