"""torch (float64, autograd) restatement of the FVM step for gradient checks.

TEST INFRASTRUCTURE: the oracle the tests compare the hand-written CUDA adjoint with, never the
product.  JAX is not installable here, so ``jax.grad`` of the reference is
replaced by torch autograd through this restatement, which follows the same
reference lines as ``oracle/fvm.py`` op for op and mirrors jnp's
differentiation semantics: ``torch.where`` sends the gradient only to the
selected branch, and ``safe_div`` divides by ``where(y != 0, y, 1)`` so the
replaced denominator gets none (interpolation.py:224-226).
"""
from __future__ import annotations

from typing import Optional, Sequence

import numpy as np
import torch

from oracle import fvm as ofvm


def shift(c: torch.Tensor, k: int, axis: int) -> torch.Tensor:
  """Periodic c.shift(k, axis): result[i] = c[i + k] (boundaries.py:81-104)."""
  return c if k == 0 else torch.roll(c, -k, dims=axis)


def _linear_along_axis(c, c_off, offset, axis):
  """interpolation.py:36-63."""
  delta = offset - c_off[axis]
  if delta == 0:
    return c, c_off
  new_off = tuple(offset if j == axis else o for j, o in enumerate(c_off))
  if int(delta) == delta:
    return shift(c, int(delta), axis), new_off
  floor = int(np.floor(delta))
  ceil = int(np.ceil(delta))
  floor_weight = ceil - delta
  ceil_weight = 1. - floor_weight
  return floor_weight * shift(c, floor, axis) + ceil_weight * shift(c, ceil, axis), new_off


def linear(c, c_off, offset):
  """interpolation.py:66-93."""
  for a, o in enumerate(offset):
    c, c_off = _linear_along_axis(c, c_off, o, a)
  return c, c_off


def safe_div(x, y, default_numerator=1):
  """interpolation.py:224-226."""
  return x / torch.where(y != 0, y, torch.full_like(y, default_numerator))


def van_leer_limiter(r):
  """interpolation.py:229-231."""
  return torch.where(r > 0, safe_div(2 * r, 1 + r), torch.zeros_like(r))


def tvd_interpolation(c, c_off, offset, v, dt, step):
  """apply_tvd_limiter(lax_wendroff, van_leer_limiter) (interpolation.py:96-303)
  for forward half-cell interpolation."""
  for axis, axis_offset in enumerate(offset):
    interp_off = tuple(co if i != axis else axis_offset for i, co in enumerate(c_off))
    if interp_off != tuple(c_off):
      u, u_off = v[axis]
      delta = u_off[axis] - c_off[axis]
      floor, ceil = int(np.floor(delta)), int(np.ceil(delta))
      c_f, c_c = shift(c, floor, axis), shift(c, ceil, axis)
      c_low = torch.where(u > 0, c_f, c_c)                        # upwind 96-155
      courant = (dt / step[axis]) * u                             # lax_wendroff 158-221
      pos = c_f + 0.5 * (1 - courant) * (c_c - c_f)
      neg = c_c - 0.5 * (1 + courant) * (c_c - c_f)
      c_high = torch.where(u > 0, pos, neg)
      c_left, c_right, c_next_right = shift(c, -1, axis), shift(c, 1, axis), shift(c, 2, axis)
      pos_r = safe_div(c - c_left, c_right - c)
      neg_r = safe_div(c_next_right - c_right, c_right - c)
      phi = torch.where(u > 0, van_leer_limiter(pos_r), van_leer_limiter(neg_r))
      c = c_low - (c_low - c_high) * phi
      c_off = interp_off
  return c, c_off


def backward_difference(c, axis, step):
  return (c - shift(c, -1, axis)) / step[axis]


def forward_difference(c, axis, step):
  return (shift(c, 1, axis) - c) / step[axis]


def laplacian(c, step):
  """finite_differences.py:127-133."""
  scales = [(1 / s) ** 2 for s in step]
  result = -2 * c * sum(scales)
  for axis in range(c.ndim):
    result = result + (shift(c, -1, axis) + shift(c, 1, axis)) * scales[axis]
  return result


def divergence(v, step):
  out = 0
  for axis, u in enumerate(v):
    out = out + backward_difference(u, axis, step)
  return out


def curl_2d(v, step):
  """finite_differences.py:186-193."""
  return forward_difference(v[1], 0, step) - forward_difference(v[0], 1, step)


def advect(c, c_off, v, v_offs, dt, step, convect='van_leer'):
  """advect_general with linear velocity interpolation and TVD (or linear)
  interpolation of c (advection.py:34-116,119-126,387-395)."""
  targets = ofvm.control_volume_offsets(c_off)
  aligned_v = tuple(linear(u, uo, t) for u, uo, t in zip(v, v_offs, targets))
  if convect == 'van_leer':
    aligned_c = tuple(tvd_interpolation(c, c_off, t, aligned_v, dt, step) for t in targets)
  else:
    aligned_c = tuple(linear(c, c_off, t) for t in targets)
  flux = tuple(ac[0] * av[0] for ac, av in zip(aligned_c, aligned_v))
  return -divergence(flux, step)


_DIAG = {}


def _pinv_diagonal(grid: ofvm.Grid, device) -> torch.Tensor:
  """float64 pseudoinverse diagonal of the periodic Laplacian on `device`."""
  key = (grid.shape, grid.step, str(device))
  if key not in _DIAG:
    _DIAG[key] = torch.from_numpy(ofvm.pinv_diagonal(grid, np.float64)).to(device)
  return _DIAG[key]


def projection(v, grid: ofvm.Grid):
  """pressure.py:115-198 with the rfft pseudoinverse (float64); runs on the
  device of `v` (CPU, or a GPU for large grids)."""
  rhs = divergence(v, grid.step)
  diag = _pinv_diagonal(grid, rhs.device)
  q = torch.fft.irfftn(diag * torch.fft.rfftn(rhs), s=rhs.shape)
  return tuple(u - forward_difference(q, axis, grid.step) for axis, u in enumerate(v))


def step_fn(density: float, viscosity, dt: float, grid: ofvm.Grid, convect='van_leer',
            linear_coefficient: Optional[float] = None, const_u=None, const_v=None):
  """One forward-Euler step of semi_implicit_navier_stokes (equations.py:77-151)
  with forcing (lin * v + const) / density; ``viscosity`` may be a tensor."""
  offs = grid.cell_faces
  step = grid.step

  def f(v):
    dv = [advect(u, o, v, offs, dt, step, convect) for u, o in zip(v, offs)]
    if viscosity is not None:
      nu = viscosity / density
      dv = [d + nu * laplacian(u, step) for d, u in zip(dv, v)]
    forcing = [0, 0]
    if linear_coefficient is not None:
      forcing = [linear_coefficient * u for u in v]
    for a, const in enumerate((const_u, const_v)):
      if const is not None:
        forcing[a] = forcing[a] + const
    dv = [d + fi / density for d, fi in zip(dv, forcing)]
    return projection(tuple(u + dt * d for u, d in zip(v, dv)), grid)
  return f


def rollout(f, v, steps: int):
  for _ in range(steps):
    v = f(v)
  return v
