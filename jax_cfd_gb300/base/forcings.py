"""Forcing functions, mirroring ``jax_cfd/base/forcings.py``.

Each builder returns a ``ForcingFn``: callable on a velocity tuple exactly like
the reference's closures, and carrying a descriptor (linear coefficient and/or
a velocity-independent field) that the fused GB300 step compiles into its
stencil.  Constant fields are evaluated once on the host in float32, the way
jnp evaluates them with x64 off.
"""
from __future__ import annotations

from typing import Callable, Optional, Sequence, Tuple

import numpy as np
import torch

from jax_cfd_gb300 import _native as nat
from jax_cfd_gb300.base import grids

GridArray = grids.GridArray


class ForcingFn:
  """A forcing function plus what the native step needs to fuse it.

  Attributes:
    linear: coefficient of a ``linear_forcing`` term, or None.
    const_kind: one of the ``_native.FORCE_*`` layouts, or FORCE_NONE.
    const_u, const_v: host float32 tables for that layout (or None).
    const_offsets: offsets of the constant components.
    spectral_const: (fx, fy) host float32 fields of a velocity-independent
      forcing, used by the spectral step (fx/fy may be None for zero).
  """

  def __init__(self, fn: Callable, *, grid: grids.Grid, linear=None,
               const_kind=nat.FORCE_NONE, const_u=None, const_v=None,
               const_offsets=None, terms=1):
    self._fn = fn
    self.grid = grid
    self.linear = linear
    self.const_kind = const_kind
    self.const_u = const_u
    self.const_v = const_v
    self.const_offsets = const_offsets
    self.terms = terms

  def __call__(self, v):
    return self._fn(v)

  @property
  def velocity_independent(self) -> bool:
    return self.linear is None

  def constant_fields(self) -> Tuple[Optional[np.ndarray], Optional[np.ndarray]]:
    """Full [nx, ny] float32 fields of the constant part (None for zero)."""
    nx, ny = self.grid.shape
    fu = fv = None
    if self.const_kind == nat.FORCE_U_OF_Y:
      fu = np.broadcast_to(self.const_u[None, :], (nx, ny)).copy()
    elif self.const_kind == nat.FORCE_V_OF_X:
      fv = np.broadcast_to(self.const_v[:, None], (nx, ny)).copy()
    elif self.const_kind == nat.FORCE_FULL:
      fu, fv = self.const_u, self.const_v
    return fu, fv


def _device_of(v):
  return v[0].data.device


def taylor_green_forcing(grid: grids.Grid, scale: float = 1, k: int = 2) -> ForcingFn:
  """forcings.py:36-60: constant Taylor-Green field (2-D)."""
  if grid.ndim != 2:
    raise NotImplementedError('only 2-D grids are on the GB300 hot path')
  offs = grid.cell_faces
  ux, uy = grid.mesh_numpy(offs[0])
  vx, vy = grid.mesh_numpy(offs[1])
  one = np.float32(1.0)  # exp(-2 nu t) at t = 0
  u = (one * np.cos(k * ux) * np.sin(k * uy)) * np.float32(scale)
  v = (-one * np.sin(k * vx) * np.cos(k * vy)) * np.float32(scale)
  u = u.astype(np.float32)
  v = v.astype(np.float32)

  def forcing(vel):
    dev = _device_of(vel)
    return (GridArray(torch.from_numpy(u).to(dev), offs[0], grid),
            GridArray(torch.from_numpy(v).to(dev), offs[1], grid))
  return ForcingFn(forcing, grid=grid, const_kind=nat.FORCE_FULL, const_u=u,
                   const_v=v, const_offsets=offs)


def kolmogorov_forcing(grid: grids.Grid, scale: float = 1, k: int = 2,
                       swap_xy: bool = False,
                       offsets: Optional[Tuple[Tuple[float, ...], ...]] = None) -> ForcingFn:
  """forcings.py:63-104: scale * sin(k y) on u (or sin(k x) on v if swapped)."""
  if grid.ndim != 2:
    raise NotImplementedError('only 2-D grids are on the GB300 hot path')
  if offsets is None:
    offsets = grid.cell_faces
  if swap_xy:
    x = grid.axes_numpy(offsets[1])[0]
    table = (scale * np.sin(k * x)).astype(np.float32)
    u_off, v_off = (1, 1 / 2), tuple(offsets[1])
    kind, cu, cv = nat.FORCE_V_OF_X, None, table
  else:
    y = grid.axes_numpy(offsets[0])[1]
    table = (scale * np.sin(k * y)).astype(np.float32)
    u_off, v_off = tuple(offsets[0]), (1 / 2, 1)
    kind, cu, cv = nat.FORCE_U_OF_Y, table, None
  nx, ny = grid.shape

  def forcing(vel):
    dev = _device_of(vel)
    t = torch.from_numpy(table).to(dev)
    if swap_xy:
      fv = t[:, None].expand(nx, ny).contiguous()
      return (GridArray(torch.zeros_like(fv), u_off, grid), GridArray(fv, v_off, grid))
    fu = t[None, :].expand(nx, ny).contiguous()
    return (GridArray(fu, u_off, grid), GridArray(torch.zeros_like(fu), v_off, grid))
  return ForcingFn(forcing, grid=grid, const_kind=kind, const_u=cu, const_v=cv,
                   const_offsets=(u_off, v_off))


def linear_forcing(grid: grids.Grid, coefficient: float) -> ForcingFn:
  """forcings.py:107-113."""
  def forcing(v):
    return tuple(coefficient * u.array for u in v)
  return ForcingFn(forcing, grid=grid, linear=float(coefficient))


def no_forcing(grid: grids.Grid) -> ForcingFn:
  """forcings.py:116-122: 0 * u."""
  def forcing(v):
    return tuple(0 * u.array for u in v)
  return ForcingFn(forcing, grid=grid, linear=0.0)


def sum_forcings(*forcings: ForcingFn) -> ForcingFn:
  """forcings.py:125-129.  The fused step supports one linear term plus one
  constant term (any order: two-term float addition is commutative)."""
  from jax_cfd_gb300.base import equations  # pylint: disable=import-outside-toplevel

  def forcing(v):
    return equations.sum_fields(*[f(v) for f in forcings])
  linear = None
  kind, cu, cv, offs = nat.FORCE_NONE, None, None, None
  grid = forcings[0].grid if forcings else None
  fusable = len(forcings) <= 2
  for f in forcings:
    if not isinstance(f, ForcingFn):
      fusable = False
      continue
    if f.linear is not None:
      if linear is not None:
        fusable = False
      linear = f.linear
    if f.const_kind != nat.FORCE_NONE:
      if kind != nat.FORCE_NONE:
        fusable = False
      kind, cu, cv, offs = f.const_kind, f.const_u, f.const_v, f.const_offsets
  out = ForcingFn(forcing, grid=grid, linear=linear, const_kind=kind,
                  const_u=cu, const_v=cv, const_offsets=offs,
                  terms=len(forcings))
  out.fusable = fusable
  return out


FORCING_FUNCTIONS = dict(kolmogorov=kolmogorov_forcing,
                         taylor_green=taylor_green_forcing)


def simple_turbulence_forcing(grid: grids.Grid, constant_magnitude: float = 0,
                              constant_wavenumber: int = 2,
                              linear_coefficient: float = 0,
                              forcing_type: str = 'kolmogorov') -> ForcingFn:
  """forcings.py:136-178."""
  linear_force = linear_forcing(grid, linear_coefficient)
  constant_force_fn = FORCING_FUNCTIONS.get(forcing_type)
  if constant_force_fn is None:
    raise ValueError('Unknown `forcing_type`. '
                     f'Expected one of {list(FORCING_FUNCTIONS.keys())}; '
                     f'got {forcing_type}.')
  constant_force = constant_force_fn(grid, constant_magnitude, constant_wavenumber)
  return sum_forcings(linear_force, constant_force)


def fused_descriptor(forcing) -> dict:
  """Arguments of the native plan for `forcing` (None means no forcing)."""
  if forcing is None:
    return dict(linear_coefficient=None, const_forcing=nat.FORCE_NONE,
                force_u=None, force_v=None)
  if not isinstance(forcing, ForcingFn) or not getattr(forcing, 'fusable', True):
    raise NotImplementedError(
        'the GB300 step fuses forcings built from forcings.{kolmogorov,linear,'
        'taylor_green,no,simple_turbulence,sum}_forcing(s); got '
        f'{forcing!r}')
  return dict(linear_coefficient=forcing.linear, const_forcing=forcing.const_kind,
              force_u=forcing.const_u, force_v=forcing.const_v)
