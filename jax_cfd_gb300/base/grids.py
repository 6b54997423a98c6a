"""Staggered-grid data model, mirroring ``jax_cfd/base/grids.py``.

``Grid`` keeps the reference's constructor, attributes and offset conventions
(grids.py:499-675).  ``GridArray(data, offset, grid)`` and
``GridVariable(array, bc)`` (grids.py:40-108, 265-395) hold torch tensors
instead of jax arrays; the hot-path kernels read them in place (float32,
C-contiguous ``[nx, ny]``, axis 1 contiguous).
"""
from __future__ import annotations

import dataclasses
import numbers
import operator
from typing import Any, Callable, Optional, Sequence, Tuple, Union

import numpy as np
import torch

Array = Union[np.ndarray, torch.Tensor]
PyTree = Any


def _data(x):
  return x.data if isinstance(x, (GridArray, GridVariable)) else x


@dataclasses.dataclass(eq=False)
class GridArray:
  """Data with an alignment offset and an associated grid (grids.py:40-108)."""
  data: torch.Tensor
  offset: Tuple[float, ...]
  grid: 'Grid'

  @property
  def dtype(self):
    return self.data.dtype

  @property
  def shape(self) -> Tuple[int, ...]:
    return tuple(self.data.shape)

  def _binary(self, other, fn):
    arrays = [self] + ([other] if isinstance(other, GridArray) else [])
    offset = consistent_offset(*arrays)
    grid = consistent_grid(*arrays)
    return GridArray(fn(self.data, _data(other)), offset, grid)

  def __add__(self, o): return self._binary(o, operator.add)
  def __radd__(self, o): return self._binary(o, lambda a, b: b + a)
  def __sub__(self, o): return self._binary(o, operator.sub)
  def __rsub__(self, o): return self._binary(o, lambda a, b: b - a)
  def __mul__(self, o): return self._binary(o, operator.mul)
  def __rmul__(self, o): return self._binary(o, lambda a, b: b * a)
  def __truediv__(self, o): return self._binary(o, operator.truediv)
  def __rtruediv__(self, o): return self._binary(o, lambda a, b: b / a)
  def __neg__(self): return GridArray(-self.data, self.offset, self.grid)
  def __gt__(self, o): return self._binary(o, operator.gt)
  def __lt__(self, o): return self._binary(o, operator.lt)


GridArrayVector = Tuple[GridArray, ...]


@dataclasses.dataclass(eq=False)
class GridVariable:
  """Associates a GridArray with BoundaryConditions (grids.py:265-395)."""
  array: GridArray
  bc: Any

  def __post_init__(self):
    if not isinstance(self.array, GridArray):
      raise ValueError(
          f'Expected array type to be GridArray, got {type(self.array)}')
    if len(self.bc.types) != self.grid.ndim:
      raise ValueError(
          'Incompatible dimension between grid and bc, grid dimension = '
          f'{self.grid.ndim}, bc dimension = {len(self.bc.types)}')

  @property
  def dtype(self):
    return self.array.dtype

  @property
  def shape(self) -> Tuple[int, ...]:
    return self.array.shape

  @property
  def data(self) -> torch.Tensor:
    return self.array.data

  @property
  def offset(self) -> Tuple[float, ...]:
    return self.array.offset

  @property
  def grid(self) -> 'Grid':
    return self.array.grid

  def shift(self, offset: int, axis: int, mode: Optional[str] = 'extend') -> GridArray:
    """Periodic shift: result[i] = data[i + offset] (boundaries.py:81-104)."""
    del mode
    return self.bc.shift(self.array, offset, axis)

  def impose_bc(self) -> 'GridVariable':
    return self.bc.impose_bc(self.array)


GridVariableVector = Tuple[GridVariable, ...]


class InconsistentOffsetError(Exception):
  """Raised for cases of inconsistent offset in GridArrays."""


class InconsistentGridError(Exception):
  """Raised for cases of inconsistent grids between GridArrays."""


class InconsistentBoundaryConditionsError(Exception):
  """Raised for cases of inconsistent bc between GridVariables."""


def consistent_offset(*arrays) -> Tuple[float, ...]:
  """grids.py:460-467."""
  offsets = {tuple(a.offset) for a in arrays}
  if len(offsets) != 1:
    raise InconsistentOffsetError(f'arrays do not have a unique offset: {offsets}')
  offset, = offsets
  return offset


def consistent_grid(*arrays) -> 'Grid':
  """grids.py:474-482."""
  grids = {a.grid for a in arrays}
  if len(grids) != 1:
    raise InconsistentGridError(f'arrays do not have a unique grid: {grids}')
  grid, = grids
  return grid


def unique_boundary_conditions(*arrays):
  bcs = {a.bc for a in arrays}
  if len(bcs) != 1:
    raise InconsistentBoundaryConditionsError(f'arrays do not have a unique bc: {bcs}')
  bc, = bcs
  return bc


def averaged_offset(*arrays) -> Tuple[float, ...]:
  """grids.py:441-445."""
  return tuple(np.mean([a.offset for a in arrays], axis=0).tolist())


def control_volume_offsets(c) -> Tuple[Tuple[float, ...], ...]:
  """grids.py:448-454."""
  return tuple(
      tuple(o + .5 if i == j else o for i, o in enumerate(c.offset))
      for j in range(len(c.offset)))


def applied(func: Callable) -> Callable:
  """Wraps a tensor function so that it acts on GridArrays (grids.py:401-433)."""
  def wrapper(*args, **kwargs):
    for arg in args + tuple(kwargs.values()):
      if isinstance(arg, GridVariable):
        raise ValueError('grids.applied() cannot be used with GridVariable')
    gas = [a for a in args + tuple(kwargs.values()) if isinstance(a, GridArray)]
    offset = consistent_offset(*gas)
    grid = consistent_grid(*gas)
    raw_args = [_data(a) for a in args]
    raw_kwargs = {k: _data(v) for k, v in kwargs.items()}
    return GridArray(func(*raw_args, **raw_kwargs), offset, grid)
  return wrapper


where = applied(torch.where)

_DEFAULT_DEVICE = None


def default_device() -> torch.device:
  """Device that Grid.mesh and initial conditions allocate on (cuda:current)."""
  if _DEFAULT_DEVICE is not None:
    return _DEFAULT_DEVICE
  return torch.device('cuda', torch.cuda.current_device())


@dataclasses.dataclass(init=False, frozen=True)
class Grid:
  """Describes the size and shape for an Arakawa C-Grid (grids.py:499-568)."""
  shape: Tuple[int, ...]
  step: Tuple[float, ...]
  domain: Tuple[Tuple[float, float], ...]

  def __init__(self, shape: Sequence[int],
               step: Optional[Union[float, Sequence[float]]] = None,
               domain: Optional[Union[float, Sequence[Tuple[float, float]]]] = None):
    shape = tuple(operator.index(s) for s in shape)
    object.__setattr__(self, 'shape', shape)
    if step is not None and domain is not None:
      raise TypeError('cannot provide both step and domain')
    elif domain is not None:
      if isinstance(domain, (int, float)):
        domain = ((0, domain),) * len(shape)
      else:
        if len(domain) != self.ndim:
          raise ValueError('length of domain does not match ndim: '
                           f'{len(domain)} != {self.ndim}')
        for bounds in domain:
          if len(bounds) != 2:
            raise ValueError(f'domain is not sequence of pairs of numbers: {domain}')
      domain = tuple((float(lower), float(upper)) for lower, upper in domain)
    else:
      if step is None:
        step = 1
      if isinstance(step, numbers.Number):
        step = (step,) * self.ndim
      elif len(step) != self.ndim:
        raise ValueError('length of step does not match ndim: '
                         f'{len(step)} != {self.ndim}')
      domain = tuple((0.0, float(step_ * size)) for step_, size in zip(step, shape))
    object.__setattr__(self, 'domain', domain)
    step = tuple((upper - lower) / size for (lower, upper), size in zip(domain, shape))
    object.__setattr__(self, 'step', step)

  @property
  def ndim(self) -> int:
    return len(self.shape)

  @property
  def cell_center(self) -> Tuple[float, ...]:
    return self.ndim * (0.5,)

  @property
  def cell_faces(self) -> Tuple[Tuple[float, ...], ...]:
    """grids.py:567-572."""
    d = self.ndim
    offsets = (np.eye(d) + np.ones([d, d])) / 2.
    return tuple(tuple(float(o) for o in offset) for offset in offsets)

  def stagger(self, v: Tuple[Array, ...]) -> Tuple[GridArray, ...]:
    return tuple(GridArray(u, o, self) for u, o in zip(v, self.cell_faces))

  def center(self, v: PyTree) -> PyTree:
    if isinstance(v, (tuple, list)):
      return type(v)(self.center(u) for u in v)
    return GridArray(v, self.cell_center, self)

  def axes_numpy(self, offset: Optional[Sequence[float]] = None,
                 dtype=np.float32) -> Tuple[np.ndarray, ...]:
    """Host float32 axes: ``lower + (arange(n) + offset) * step`` with each op
    rounded to float32, as jnp computes them with x64 off (grids.py:588-610)."""
    if offset is None:
      offset = self.cell_center
    if len(offset) != self.ndim:
      raise ValueError(f'unexpected offset length: {len(offset)} vs {self.ndim}')
    t = np.dtype(dtype).type
    return tuple(t(lower) + (np.arange(length).astype(dtype) + t(o)) * t(step)
                 for (lower, _), o, length, step in zip(
                     self.domain, offset, self.shape, self.step))

  def axes(self, offset: Optional[Sequence[float]] = None, device=None):
    dev = default_device() if device is None else device
    return tuple(torch.from_numpy(a).to(dev) for a in self.axes_numpy(offset))

  def mesh_numpy(self, offset=None, dtype=np.float32):
    return tuple(np.meshgrid(*self.axes_numpy(offset, dtype), indexing='ij'))

  def mesh(self, offset: Optional[Sequence[float]] = None, device=None):
    """grids.py:640-653: per-axis positions, broadcast to the grid shape."""
    dev = default_device() if device is None else device
    return tuple(torch.from_numpy(np.ascontiguousarray(m)).to(dev)
                 for m in self.mesh_numpy(offset))

  def fft_axes_numpy(self, dtype=np.float32):
    """grids.py:612-616 (jnp.fft.fftfreq in float32)."""
    return tuple(_fftfreq(n, s, dtype) for n, s in zip(self.shape, self.step))

  def rfft_axes_numpy(self, dtype=np.float32):
    """grids.py:618-638."""
    ax = tuple(_fftfreq(n, s, dtype) for n, s in zip(self.shape[:-1], self.step[:-1]))
    return ax + (_rfftfreq(self.shape[-1], self.step[-1], dtype),)

  def rfft_mesh(self, device=None):
    dev = default_device() if device is None else device
    return tuple(torch.from_numpy(np.ascontiguousarray(m)).to(dev) for m in
                 np.meshgrid(*self.rfft_axes_numpy(), indexing='ij'))

  def eval_on_mesh(self, fn: Callable[..., Array], offset=None) -> GridArray:
    if offset is None:
      offset = self.cell_center
    return GridArray(fn(*self.mesh(offset)), offset, self)


def _fftfreq(n, d, dtype=np.float32):
  k = np.concatenate([np.arange(0, (n - 1) // 2 + 1), np.arange(-(n // 2), 0)]).astype(dtype)
  return k / np.dtype(dtype).type(d * n)


def _rfftfreq(n, d, dtype=np.float32):
  return np.arange(0, n // 2 + 1).astype(dtype) / np.dtype(dtype).type(d * n)
