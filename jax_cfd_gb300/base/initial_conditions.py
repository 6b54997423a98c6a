"""Initial conditions, mirroring ``jax_cfd/base/initial_conditions.py``.

``filtered_velocity_field`` runs on the GPU: the spectral filter
(filter_utils.py:32-42) through the native rfft2/irfft2, then ``iterations``
rounds of native projection and max-speed normalisation
(initial_conditions.py:112-121).  The noise source is NumPy's PCG64
(``numpy.random.default_rng(seed).standard_normal``, one draw per component
in component order): the reference's ``jax.random`` bit stream is not
available without JAX, so ``rng_key`` is an integer seed or a NumPy Generator.
"""
from __future__ import annotations

from typing import Callable, Optional, Sequence, Tuple, Union

import numpy as np
import torch

from jax_cfd_gb300 import plans
from jax_cfd_gb300.base import boundaries
from jax_cfd_gb300.base import grids
from jax_cfd_gb300.base import pressure

GridArray = grids.GridArray
GridVariable = grids.GridVariable


def wrap_variables(var, grid: grids.Grid, bcs, offsets=None, batch_dim: bool = False):
  """initial_conditions.py:40-57."""
  del batch_dim
  if offsets is None:
    offsets = grid.cell_faces
  return tuple(bc.impose_bc(GridArray(u, o, grid)) for u, o, bc in zip(var, offsets, bcs))


def log_normal_pdf(x, mode, variance=.25):
  """initial_conditions.py:60-64 (float32 NumPy on the host)."""
  mean = np.log(np.float32(mode)) + np.float32(variance)
  logx = np.log(x)
  return np.exp(-(mean - logx) ** 2 / np.float32(2) / np.float32(variance) - logx)


def angular_frequency_magnitude(grid: grids.Grid) -> np.ndarray:
  """filter_utils.py:25-29 in float32."""
  freqs = [np.float32(2 * np.pi) * f for f in grid.fft_axes_numpy()]
  mesh = np.stack(np.meshgrid(*freqs, indexing='ij'), axis=0)
  return np.sqrt(np.sum(mesh * mesh, axis=0)).astype(np.float32)


def spectral_filter_table(spectral_density: Callable, grid: grids.Grid) -> np.ndarray:
  """filters = where(k > 0, spectral_density(k), 0) on the rfft half grid."""
  k = angular_frequency_magnitude(grid)
  with np.errstate(divide='ignore', invalid='ignore'):
    f = np.where(k > 0, spectral_density(k), 0.0).astype(np.float32)
  return np.ascontiguousarray(f[:, : grid.shape[-1] // 2 + 1])


def _spec_plan(grid: grids.Grid, device):
  return plans.cached('spec-fft', (device, grid.shape, grid.step),
                      lambda: plans.SpecPlan(grid.shape, grid.step, device=device))


def _noise(rng_key, grid: grids.Grid):
  rng = rng_key if isinstance(rng_key, np.random.Generator) else np.random.default_rng(int(rng_key))
  return [rng.standard_normal(grid.shape).astype(np.float32) for _ in range(grid.ndim)]


def filtered_velocity_field(rng_key: Union[int, np.random.Generator],
                            grid: grids.Grid, maximum_velocity: float = 1,
                            peak_wavenumber: float = 3, iterations: int = 3,
                            device=None) -> Tuple[GridVariable, ...]:
  """initial_conditions.py:71-121."""
  if grid.ndim != 2:
    raise NotImplementedError('only 2-D grids are on the GB300 hot path')
  dev = grids.default_device() if device is None else torch.device(device)

  def spectral_density(k):
    return log_normal_pdf(k, peak_wavenumber) / k ** (grid.ndim - 1)
  table = torch.from_numpy(spectral_filter_table(spectral_density, grid)).to(dev)
  plan = _spec_plan(grid, dev)
  comps = [plan.spectral_filter(torch.from_numpy(n).to(dev), table)
           for n in _noise(rng_key, grid)]
  bcs = [boundaries.periodic_boundary_conditions(grid.ndim)] * grid.ndim
  v = wrap_variables(comps, grid, bcs)
  for _ in range(iterations):
    v = pressure.projection(v)
    vmax = plans.max_speed(v[0].data, v[1].data)
    plans.scale_to_max_speed(v[0].data, v[1].data, vmax, maximum_velocity)
  return v


def initial_velocity_field(velocity_fns, grid: grids.Grid, velocity_bc=None,
                           pressure_solve=pressure.solve_fast_diag,
                           iterations: Optional[int] = None):
  """initial_conditions.py:124-161."""
  if velocity_bc is None:
    velocity_bc = (boundaries.periodic_boundary_conditions(grid.ndim),) * grid.ndim
  v = tuple(GridVariable(grid.eval_on_mesh(fn, offset), bc)
            for fn, offset, bc in zip(velocity_fns, grid.cell_faces, velocity_bc))
  if iterations is not None:
    for _ in range(iterations):
      v = pressure.projection(v, pressure_solve)
  return v
