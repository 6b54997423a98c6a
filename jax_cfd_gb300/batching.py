"""Batched and ragged execution of many independent FVM trajectories.

The reference advances one trajectory per call (``funcutils.repeated`` over a
``semi_implicit_navier_stokes`` step, jax_cfd/base/funcutils.py:82-88,
equations.py:120-151); many trajectories mean a Python loop or ``vmap`` over
same-shape inputs.  Here:

* ``FvmBatch``: ``count`` slots of one grid shape, each with its own viscosity,
  dt, density and forcing, advanced by one launch per kernel kind per step for
  the whole batch (the slot index is a grid axis of every launch).  Each slot
  has its own step count per chunk, so trajectories with different horizons
  share launches; slot parameters can be replaced between chunks (continuous
  batching).
* ``FvmEnsemble``: members of any shapes, grouped into one batch per shape;
  the batches run on forked streams and a chunk is one CUDA-graph launch.
* ``Ensemble``: the same over the drop-in objects -- step functions returned
  by ``equations.semi_implicit_navier_stokes`` and ``GridVariable`` states.

A member's result does not depend on which other members share its launches:
every kernel reads and writes only its own member's buffers.
"""
from __future__ import annotations

import ctypes
from typing import List, Optional, Sequence

import numpy as np
import torch

from jax_cfd_gb300 import _native as nat
from jax_cfd_gb300 import plans


class _DeviceArray:
  """A device array owned by a native object, exposed to torch through
  ``__cuda_array_interface__`` (zero copy); holds a reference to its owner."""

  def __init__(self, owner, address: int, shape, typestr: str = '<f4'):
    self._owner = owner
    self.__cuda_array_interface__ = {
        'shape': tuple(int(s) for s in shape), 'typestr': typestr,
        'data': (int(address), False), 'version': 2, 'strides': None}


def _view(owner, address: int, shape, device, typestr: str = '<f4') -> torch.Tensor:
  return torch.as_tensor(_DeviceArray(owner, address, shape, typestr), device=device)


# Host layout of the native per-slot health records (cfd_health).
HEALTH_DTYPE = np.dtype([('flags', '<u4'), ('max_abs', '<f4')])


def decode_health(raw) -> np.ndarray:
  """Health records from their int32 [count, 2] image (device or host)."""
  a = raw.cpu().numpy() if isinstance(raw, torch.Tensor) else np.asarray(raw)
  a = np.ascontiguousarray(a, dtype=np.int32).reshape(-1, 2)
  rec = np.empty(a.shape[0], HEALTH_DTYPE)
  rec['flags'] = a[:, 0].view(np.uint32)
  rec['max_abs'] = a[:, 1].view(np.float32)
  return rec


def _set_mirror(fn, handle, name: str, host: Optional[torch.Tensor], count: int):
  """Points a batch's health mirror at `host` (pinned int32 [count, 2]) or
  turns it off (None)."""
  if host is not None:
    if not host.is_pinned() or host.dtype != torch.int32 or tuple(host.shape) != (count, 2):
      raise ValueError(f'{name}: the mirror must be a pinned int32 tensor of shape ({count}, 2)')
  nat.check(fn(handle, None if host is None else ctypes.c_void_p(host.data_ptr())), name)


def _health_view(owner, fn, handle, count: int, device, *index) -> torch.Tensor:
  """int32 [count, 2] device view of health records returned by `fn`."""
  ptr = ctypes.c_void_p()
  nat.check(fn(handle, *index, ctypes.byref(ptr)), getattr(fn, '__name__', 'health'))
  return _view(owner, ptr.value, (count, 2), device, '<i4')


class FvmBatch:
  """Slots of one grid shape stepped together (``cfd_fvm_batch``)."""

  def __init__(self, shape: Sequence[int], step: Sequence[float], count: int, *,
               convect: int = nat.CONVECT_VAN_LEER,
               device: Optional[torch.device] = None):
    self.shape = (int(shape[0]), int(shape[1]))
    self.step = (float(step[0]), float(step[1]))
    self.count = int(count)
    self.convect = int(convect)
    self.device = torch.device(device) if device is not None else torch.device(
        'cuda', torch.cuda.current_device())
    cfg, _ = plans.fvm_config(self.shape, self.step, convect=convect, dt=0.0)
    handle = ctypes.c_void_p()
    self._lib = nat.load()
    with torch.cuda.device(self.device):
      nat.check(self._lib.cfd_fvm_batch_create(ctypes.byref(cfg), self.count,
                                               ctypes.byref(handle)), 'cfd_fvm_batch_create')
    self._h = handle
    self._views = [None] * self.count

  def __del__(self):
    h = getattr(self, '_h', None)
    if h is not None and h.value:
      try:
        torch.cuda.synchronize(self.device)
        self._lib.cfd_fvm_batch_destroy(h)
      except Exception:  # pylint: disable=broad-except
        pass
      self._h = None

  @property
  def nbytes(self) -> int:
    return int(self._lib.cfd_fvm_batch_bytes(self._h))

  def _slot(self, slot: int) -> int:
    if not 0 <= slot < self.count:
      raise IndexError(f'slot {slot} out of range [0, {self.count})')
    return int(slot)

  def state(self, slot: int):
    """(u, v) of a slot: torch views of the batch's device memory."""
    slot = self._slot(slot)
    if self._views[slot] is None:
      u, v = ctypes.c_void_p(), ctypes.c_void_p()
      nat.check(self._lib.cfd_fvm_batch_state(self._h, slot, ctypes.byref(u), ctypes.byref(v)),
                'cfd_fvm_batch_state')
      self._views[slot] = (_view(self, u.value, self.shape, self.device),
                           _view(self, v.value, self.shape, self.device))
    return self._views[slot]

  def set_slot(self, slot: int, *, dt: float, density: float = 1.0,
               viscosity: Optional[float] = None,
               linear_coefficient: Optional[float] = None,
               const_forcing: int = nat.FORCE_NONE, force_u=None, force_v=None):
    """Gives a slot new step parameters (enqueued on the current stream)."""
    slot = self._slot(slot)
    cfg, keep = plans.fvm_config(self.shape, self.step, density=density, viscosity=viscosity,
                                 dt=dt, convect=self.convect,
                                 linear_coefficient=linear_coefficient,
                                 const_forcing=const_forcing, force_u=force_u,
                                 force_v=force_v)
    nat.check(self._lib.cfd_fvm_batch_set_slot(self._h, plans.current_stream_ptr(self.device),
                                               slot, ctypes.byref(cfg)), 'cfd_fvm_batch_set_slot')
    del keep

  def set_state(self, slot: int, u: torch.Tensor, v: torch.Tensor):
    su, sv = self.state(slot)
    su.copy_(u)
    sv.copy_(v)

  def set_steps(self, slot: int, steps: int):
    nat.check(self._lib.cfd_fvm_batch_set_steps(self._h, self._slot(slot), int(steps)),
              'cfd_fvm_batch_set_steps')

  def run(self, chunk: int, graph: bool = True):
    """Advances every slot by min(its steps, chunk) steps, in place."""
    nat.check(self._lib.cfd_fvm_batch_run(self._h, plans.current_stream_ptr(self.device),
                                          int(chunk), 1 if graph else 0), 'cfd_fvm_batch_run')

  def autotune(self, steps: int = 10) -> int:
    """Times the launch configurations and keeps the fastest; returns its
    index (row shape + 2 * column scheme + 10 * stencil, or 20: each member's
    whole chunk resident in shared memory, for small grids, or 21 + the first
    form with the rows fed by bulk copies)."""
    chosen = ctypes.c_int(-1)
    nat.check(self._lib.cfd_fvm_batch_autotune(self._h, plans.current_stream_ptr(self.device),
                                               int(steps), ctypes.byref(chosen)),
              'cfd_fvm_batch_autotune')
    return int(chosen.value)

  # row shape + 2 * column scheme + 10 * stencil (0..19), 20 resident chunks,
  # 21 + (0..19) the same with bulk-copy row feed (cfd_fvm_batch_autotune).
  LAUNCH_CHOICES = 41

  def set_launch(self, choice: int):
    """Pins the launch configuration (see autotune); results do not change."""
    nat.check(self._lib.cfd_fvm_batch_set_launch(self._h, int(choice)),
              'cfd_fvm_batch_set_launch')

  def health_device(self) -> torch.Tensor:
    """The per-slot health records as an int32 [count, 2] device view
    (flags, bits of max_abs), written at the end of every run for the slots
    that ran; decode with ``decode_health``."""
    if getattr(self, '_health', None) is None:
      self._health = _health_view(self, self._lib.cfd_fvm_batch_health, self._h, self.count,
                                  self.device)
    return self._health

  def health(self) -> np.ndarray:
    """Host copy of the health records (ordered after the current stream's
    work): ``flags`` (HEALTH_NONFINITE when the state holds a NaN or an
    infinity) and ``max_abs`` (largest finite |u| or |v|)."""
    return decode_health(self.health_device())

  def set_health_mirror(self, host: Optional[torch.Tensor]):
    """Every run also writes the records into `host` (a pinned int32
    [count, 2] tensor, kept alive by the caller) from the device, readable
    once the run's stream has passed it; None stops it."""
    _set_mirror(self._lib.cfd_fvm_batch_set_health_mirror, self._h,
                'cfd_fvm_batch_set_health_mirror', host, self.count)
    self._mirror = host


class SpecBatch:
  """Slots of one grid shape running NavierStokes2D + a low-storage RK/CN
  integrator together (``cfd_spec_batch``)."""

  def __init__(self, shape: Sequence[int], step: Sequence[float], count: int, *,
               stages: int = 5, device: Optional[torch.device] = None):
    self.shape = (int(shape[0]), int(shape[1]))
    self.half_shape = (self.shape[0], self.shape[1] // 2 + 1)
    self.step = (float(step[0]), float(step[1]))
    self.count = int(count)
    self.stages = int(stages)
    self.device = torch.device(device) if device is not None else torch.device(
        'cuda', torch.cuda.current_device())
    zeros = [0.0] * self.stages
    cfg, _ = plans.spec_config(self.shape, self.step, alphas=[0.0] * (self.stages + 1),
                               betas=zeros, gammas=zeros)
    handle = ctypes.c_void_p()
    self._lib = nat.load()
    with torch.cuda.device(self.device):
      nat.check(self._lib.cfd_spec_batch_create(ctypes.byref(cfg), self.count,
                                                ctypes.byref(handle)), 'cfd_spec_batch_create')
    self._h = handle
    self._views = [None] * self.count
    self._forcing = [None] * self.count

  def __del__(self):
    h = getattr(self, '_h', None)
    if h is not None and h.value:
      try:
        torch.cuda.synchronize(self.device)
        self._lib.cfd_spec_batch_destroy(h)
      except Exception:  # pylint: disable=broad-except
        pass
      self._h = None

  @property
  def nbytes(self) -> int:
    return int(self._lib.cfd_spec_batch_bytes(self._h))

  def _slot(self, slot: int) -> int:
    if not 0 <= slot < self.count:
      raise IndexError(f'slot {slot} out of range [0, {self.count})')
    return int(slot)

  def state(self, slot: int) -> torch.Tensor:
    """The slot's vorticity spectrum (complex64 view of batch memory)."""
    slot = self._slot(slot)
    if self._views[slot] is None:
      w = ctypes.c_void_p()
      nat.check(self._lib.cfd_spec_batch_state(self._h, slot, ctypes.byref(w)),
                'cfd_spec_batch_state')
      flat = _view(self, w.value, (self.half_shape[0], 2 * self.half_shape[1]), self.device)
      self._views[slot] = flat.view(torch.complex64)
    return self._views[slot]

  def set_slot(self, slot: int, *, viscosity: float, drag: float, dt: float,
               smooth: bool = True, alphas, betas, gammas,
               forcing_plan: Optional[plans.SpecPlan] = None):
    """New step parameters for a slot; the forcing curl table is borrowed from
    `forcing_plan` (kept alive by the batch while the slot uses it)."""
    slot = self._slot(slot)
    cfg, keep = plans.spec_config(self.shape, self.step, viscosity=viscosity, drag=drag, dt=dt,
                                  smooth=smooth, alphas=alphas, betas=betas, gammas=gammas)
    fh = forcing_plan.handle if forcing_plan is not None else None
    nat.check(self._lib.cfd_spec_batch_set_slot(self._h, slot, ctypes.byref(cfg), fh),
              'cfd_spec_batch_set_slot')
    self._forcing[slot] = forcing_plan
    del keep

  def set_slot_from_step(self, slot: int, step_fn):
    """Slot parameters from a drop-in step (``crank_nicolson_rk4(eq, dt)``)."""
    from jax_cfd_gb300.spectral import time_stepping  # pylint: disable=import-outside-toplevel
    if not isinstance(step_fn, time_stepping.SpectralStep):
      raise NotImplementedError('spectral slots take time_stepping.SpectralStep steps')
    eq = step_fn.equation
    if tuple(eq.grid.shape) != self.shape or tuple(eq.grid.step) != self.step:
      raise ValueError('the step lives on another grid')
    forcing = eq._plan(self.device) if eq.forcing_fn is not None else None  # pylint: disable=protected-access
    a, b, g = step_fn.coefficients
    self.set_slot(slot, viscosity=float(eq.viscosity), drag=float(eq.drag),
                  dt=step_fn.time_step, smooth=eq.smooth is not None, alphas=a, betas=b,
                  gammas=g, forcing_plan=forcing)

  def set_state(self, slot: int, w_hat: torch.Tensor):
    self.state(slot).copy_(w_hat)

  def set_steps(self, slot: int, steps: int):
    nat.check(self._lib.cfd_spec_batch_set_steps(self._h, self._slot(slot), int(steps)),
              'cfd_spec_batch_set_steps')

  def run(self, chunk: int, graph: bool = True):
    nat.check(self._lib.cfd_spec_batch_run(self._h, plans.current_stream_ptr(self.device),
                                           int(chunk), 1 if graph else 0), 'cfd_spec_batch_run')

  def health_device(self) -> torch.Tensor:
    """As FvmBatch.health_device; max_abs is the largest finite component of
    the vorticity spectrum."""
    if getattr(self, '_health', None) is None:
      self._health = _health_view(self, self._lib.cfd_spec_batch_health, self._h, self.count,
                                  self.device)
    return self._health

  def health(self) -> np.ndarray:
    return decode_health(self.health_device())

  def set_health_mirror(self, host: Optional[torch.Tensor]):
    """As FvmBatch.set_health_mirror."""
    _set_mirror(self._lib.cfd_spec_batch_set_health_mirror, self._h,
                'cfd_spec_batch_set_health_mirror', host, self.count)
    self._mirror = host


class FvmEnsemble:
  """Members of any grid shapes (``cfd_fvm_ensemble``); ``members`` are dicts
  of ``plans.fvm_config`` arguments (shape, step, dt, viscosity, ...)."""

  def __init__(self, members: Sequence[dict], device: Optional[torch.device] = None):
    self.device = torch.device(device) if device is not None else torch.device(
        'cuda', torch.cuda.current_device())
    self.shapes = [tuple(int(n) for n in m['shape']) for m in members]
    cfgs = (nat.FvmConfig * len(members))()
    keep = []
    for i, m in enumerate(members):
      kw = dict(m)
      shape, step = kw.pop('shape'), kw.pop('step')
      cfg, k = plans.fvm_config(shape, step, **kw)
      cfgs[i] = cfg
      keep.append(k)
    handle = ctypes.c_void_p()
    self._lib = nat.load()
    with torch.cuda.device(self.device):
      nat.check(self._lib.cfd_fvm_ensemble_create(cfgs, len(members), ctypes.byref(handle)),
                'cfd_fvm_ensemble_create')
    del keep
    self._h = handle
    self._views = [None] * len(members)

  def __del__(self):
    h = getattr(self, '_h', None)
    if h is not None and h.value:
      try:
        torch.cuda.synchronize(self.device)
        self._lib.cfd_fvm_ensemble_destroy(h)
      except Exception:  # pylint: disable=broad-except
        pass
      self._h = None

  def __len__(self):
    return len(self.shapes)

  @property
  def num_batches(self) -> int:
    return int(self._lib.cfd_fvm_ensemble_batches(self._h))

  def state(self, index: int):
    if self._views[index] is None:
      u, v = ctypes.c_void_p(), ctypes.c_void_p()
      nat.check(self._lib.cfd_fvm_ensemble_state(self._h, int(index), ctypes.byref(u),
                                                 ctypes.byref(v)), 'cfd_fvm_ensemble_state')
      self._views[index] = (_view(self, u.value, self.shapes[index], self.device),
                            _view(self, v.value, self.shapes[index], self.device))
    return self._views[index]

  def set_state(self, index: int, u: torch.Tensor, v: torch.Tensor):
    su, sv = self.state(index)
    su.copy_(u)
    sv.copy_(v)

  def step(self, steps: int, graph: bool = True):
    nat.check(self._lib.cfd_fvm_ensemble_step(self._h, plans.current_stream_ptr(self.device),
                                              int(steps), 1 if graph else 0),
              'cfd_fvm_ensemble_step')

  def health(self) -> np.ndarray:
    """Health records of every member after its last step (see
    FvmBatch.health), in member order."""
    if getattr(self, '_health', None) is None:
      self._health = [_health_view(self, self._lib.cfd_fvm_ensemble_health, self._h, 1,
                                   self.device, i) for i in range(len(self))]
    return decode_health(torch.cat(self._health))

  def autotune(self, steps: int = 10):
    nat.check(self._lib.cfd_fvm_ensemble_autotune(self._h, plans.current_stream_ptr(self.device),
                                                  int(steps)), 'cfd_fvm_ensemble_autotune')


class Ensemble:
  """A ragged ensemble over drop-in step functions.

  ``step_fns[i]`` is what ``equations.semi_implicit_navier_stokes`` returned
  for member i (its grid, dt, viscosity and forcing); ``advance(steps)`` is
  ``funcutils.repeated(step_fns[i], steps)`` applied to every member at once.
  """

  def __init__(self, step_fns: Sequence, device: Optional[torch.device] = None):
    from jax_cfd_gb300.base import equations  # pylint: disable=import-outside-toplevel
    members = []
    for f in step_fns:
      if not isinstance(f, equations.FvmStep):
        raise NotImplementedError(
            'ensemble members must be step functions from '
            'equations.semi_implicit_navier_stokes on the GB300 path')
      members.append(dict(shape=f.grid.shape, step=f.grid.step, **f._plan_kwargs))  # pylint: disable=protected-access
    self.step_fns: List = list(step_fns)
    self.native = FvmEnsemble(members, device=device)

  def __len__(self):
    return len(self.step_fns)

  def set_velocity(self, index: int, v):
    from jax_cfd_gb300.base import equations  # pylint: disable=import-outside-toplevel
    equations._check_state(v, self.step_fns[index].grid)  # pylint: disable=protected-access
    self.native.set_state(index, v[0].data, v[1].data)

  def velocity(self, index: int, copy: bool = True):
    from jax_cfd_gb300.base.grids import GridArray, GridVariable  # pylint: disable=import-outside-toplevel
    from jax_cfd_gb300.base import boundaries  # pylint: disable=import-outside-toplevel
    grid = self.step_fns[index].grid
    bc = boundaries.periodic_boundary_conditions(2)
    u, v = self.native.state(index)
    if copy:
      u, v = u.clone(), v.clone()
    return tuple(GridVariable(GridArray(a, o, grid), bc)
                 for a, o in zip((u, v), grid.cell_faces))

  def advance(self, steps: int, graph: bool = True):
    self.native.step(steps, graph=graph)

  def health(self) -> np.ndarray:
    """Per-member health records after the last advance (flags, max_abs)."""
    return self.native.health()

  def finite(self) -> np.ndarray:
    """Whether each member's velocity is free of NaN and infinity."""
    return (self.health()['flags'] & nat.HEALTH_NONFINITE) == 0

  def autotune(self, steps: int = 10):
    self.native.autotune(steps)


def kolmogorov_member(shape, viscosity: float, dt: float, k: int,
                      linear: float = -0.1, domain=((0.0, 2 * np.pi), (0.0, 2 * np.pi))) -> dict:
  """Arguments of an FVM member with simple_turbulence_forcing(1, k, linear)
  (forcings.py:136-178): Kolmogorov sin(k y) on u at its staggered offset plus
  linear drag."""
  from jax_cfd_gb300.base import forcings, grids  # pylint: disable=import-outside-toplevel
  grid = grids.Grid(tuple(shape), domain=domain)
  f = forcings.simple_turbulence_forcing(grid, 1, k, linear)
  return dict(shape=grid.shape, step=grid.step, dt=float(dt), density=1.0,
              viscosity=float(viscosity), linear_coefficient=f.linear,
              const_forcing=f.const_kind, force_u=f.const_u, force_v=f.const_v)
