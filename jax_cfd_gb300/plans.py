"""Owning wrappers around the native FVM and spectral plans.

A plan holds one grid's precomputed tables (Laplacian eigenvalues, FFT
twiddles, wavenumbers, forcing) and its device workspace.  Entry points take
torch CUDA tensors and enqueue on the current torch stream; nothing here
synchronises except ``SpecPlan.set_forcing`` (documented in the C header).
"""
from __future__ import annotations

import ctypes
from typing import Optional, Sequence

import numpy as np
import torch

from jax_cfd_gb300 import _native as nat


def current_stream_ptr(device: Optional[torch.device] = None) -> int:
  return torch.cuda.current_stream(device).cuda_stream


def ptr(t: torch.Tensor) -> int:
  return t.data_ptr()


def require_field(t: torch.Tensor, shape, dtype=torch.float32, name='array'):
  """Validates a device field the kernels read or write."""
  if not isinstance(t, torch.Tensor):
    raise TypeError(f'{name} must be a torch.Tensor, got {type(t)}')
  if not t.is_cuda:
    raise ValueError(f'{name} must be a CUDA tensor (the native kernels run on the GPU)')
  if t.dtype != dtype:
    raise ValueError(f'{name}.dtype={t.dtype} does not match dtype={dtype}')
  if tuple(t.shape) != tuple(shape):
    raise ValueError(f'{name}.shape={tuple(t.shape)} does not match shape={tuple(shape)}')
  if not t.is_contiguous():
    raise ValueError(f'{name} must be contiguous')
  return t


def fvm_config(shape: Sequence[int], step: Sequence[float], *, density: float = 1.0,
               viscosity: Optional[float] = None, dt: float = 0.0,
               convect: int = nat.CONVECT_VAN_LEER,
               linear_coefficient: Optional[float] = None,
               const_forcing: int = nat.FORCE_NONE,
               force_u: Optional[np.ndarray] = None,
               force_v: Optional[np.ndarray] = None):
  """The C-ABI configuration of one FVM step; returns (config, arrays the
  config points into, which must stay alive while it is used)."""
  cfg = nat.FvmConfig()
  cfg.nx, cfg.ny = int(shape[0]), int(shape[1])
  cfg.hx, cfg.hy = float(step[0]), float(step[1])
  cfg.density = float(density)
  cfg.has_viscosity = 0 if viscosity is None else 1
  cfg.viscosity = 0.0 if viscosity is None else float(viscosity)
  cfg.dt = float(dt)
  cfg.convect = int(convect)
  cfg.has_linear_forcing = 0 if linear_coefficient is None else 1
  cfg.linear_coefficient = 0.0 if linear_coefficient is None else float(linear_coefficient)
  cfg.const_forcing = int(const_forcing)
  keep = []
  nx, ny = cfg.nx, cfg.ny
  lengths = {nat.FORCE_U_OF_Y: (ny, None), nat.FORCE_V_OF_X: (None, nx),
             nat.FORCE_FULL: (nx * ny, nx * ny)}.get(int(const_forcing), (None, None))
  for name, arr, want in (('force_u', force_u, lengths[0]), ('force_v', force_v, lengths[1])):
    if arr is not None:
      a = np.ascontiguousarray(arr, dtype=np.float32)
      if want is not None and a.size != want:
        raise ValueError(f'{name} has {a.size} values; this forcing layout on a '
                         f'{nx}x{ny} grid needs {want}')
      keep.append(a)
      setattr(cfg, name, a.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
  return cfg, keep


class FvmPlan:
  """Native plan for the staggered-grid step and pressure projection."""

  def __init__(self, shape: Sequence[int], step: Sequence[float], *,
               density: float = 1.0, viscosity: Optional[float] = None,
               dt: float = 0.0, convect: int = nat.CONVECT_VAN_LEER,
               linear_coefficient: Optional[float] = None,
               const_forcing: int = nat.FORCE_NONE,
               force_u: Optional[np.ndarray] = None,
               force_v: Optional[np.ndarray] = None,
               device: Optional[torch.device] = None):
    if len(shape) != 2:
      raise NotImplementedError('only 2-D grids are on the GB300 hot path')
    self.shape = (int(shape[0]), int(shape[1]))
    self.device = torch.device(device) if device is not None else torch.device(
        'cuda', torch.cuda.current_device())
    cfg, self._keep = fvm_config(self.shape, step, density=density, viscosity=viscosity,
                                 dt=dt, convect=convect,
                                 linear_coefficient=linear_coefficient,
                                 const_forcing=const_forcing, force_u=force_u,
                                 force_v=force_v)
    handle = ctypes.c_void_p()
    with torch.cuda.device(self.device):
      nat.check(nat.load().cfd_fvm_plan_create(ctypes.byref(cfg), ctypes.byref(handle)),
                'cfd_fvm_plan_create')
    self._h = handle
    self._lib = nat.load()

  def __del__(self):
    h = getattr(self, '_h', None)
    if h is not None and h.value:
      try:
        self._lib.cfd_fvm_plan_destroy(h)
      except Exception:  # pylint: disable=broad-except
        pass
      self._h = None

  @property
  def handle(self):
    return self._h

  @property
  def nbytes(self) -> int:
    return int(self._lib.cfd_fvm_plan_bytes(self._h))

  def _fields(self, *ts):
    for t in ts:
      require_field(t, self.shape)
    return [ptr(t) for t in ts]

  def step(self, u, v, steps: int, u_out=None, v_out=None):
    if steps < 0:
      raise ValueError('steps must be non-negative')
    u_out = torch.empty_like(u) if u_out is None else u_out
    v_out = torch.empty_like(v) if v_out is None else v_out
    a = self._fields(u, v, u_out, v_out)
    nat.check(self._lib.cfd_fvm_step(self._h, current_stream_ptr(u.device), *a, int(steps)),
              'cfd_fvm_step')
    return u_out, v_out

  def trajectory(self, u, v, inner: int, frames: int, frame_kind: int,
                 start_with_input: bool = False):
    """cfd_fvm_trajectory: (u_out, v_out, frames) with frames [frames, 2, nx,
    ny] (velocity) or [frames, nx, ny] (vorticity) on the device."""
    if inner < 0 or frames < 0:
      raise ValueError('inner and frames must be non-negative')
    u_out, v_out = torch.empty_like(u), torch.empty_like(v)
    shape = ((frames, 2) if frame_kind == nat.FRAME_VELOCITY else (frames,)) + tuple(self.shape)
    out = torch.empty(shape, dtype=torch.float32, device=u.device)
    a = self._fields(u, v)
    nat.check(self._lib.cfd_fvm_trajectory(self._h, current_stream_ptr(u.device), *a, int(inner),
                                           int(frames), int(frame_kind),
                                           int(bool(start_with_input)),
                                           ptr(out) if frames else None, ptr(u_out),
                                           ptr(v_out)), 'cfd_fvm_trajectory')
    return u_out, v_out, out

  def step_implicit(self, u, v, steps: int, viscosity: float, u_out=None, v_out=None):
    """implicit_diffusion_navier_stokes (equations.py:154-195); the plan is
    made without explicit viscosity."""
    if steps < 0:
      raise ValueError('steps must be non-negative')
    u_out = torch.empty_like(u) if u_out is None else u_out
    v_out = torch.empty_like(v) if v_out is None else v_out
    a = self._fields(u, v, u_out, v_out)
    nat.check(self._lib.cfd_fvm_step_implicit(self._h, current_stream_ptr(u.device), *a,
                                              int(steps), float(viscosity)),
              'cfd_fvm_step_implicit')
    return u_out, v_out

  def diffusion_solve(self, u, v, nu: float, dt: float, u_out=None, v_out=None):
    """diffusion.solve_fast_diag (diffusion.py:166-212) on periodic (u, v)."""
    u_out = torch.empty_like(u) if u_out is None else u_out
    v_out = torch.empty_like(v) if v_out is None else v_out
    a = self._fields(u, v, u_out, v_out)
    nat.check(self._lib.cfd_fvm_diffusion_solve(self._h, current_stream_ptr(u.device), *a,
                                                float(nu), float(dt)),
              'cfd_fvm_diffusion_solve')
    return u_out, v_out

  def step_rk(self, u, v, steps: int, a, b, u_out=None, v_out=None):
    """navier_stokes_rk with Butcher tableau (a, b) (time_stepping.py:59-107)."""
    if steps < 0:
      raise ValueError('steps must be non-negative')
    stages = len(b)
    if not 1 <= stages <= 4 or len(a) + 1 != stages:
      raise NotImplementedError('the GB300 Runge-Kutta step takes tableaux of 1 to 4 stages')
    if any(len(row) > i + 1 for i, row in enumerate(a)):
      raise ValueError('explicit tableaux only: row i has at most i + 1 entries')
    # Row i of the lower triangle, padded with zeros (which the reference's
    # sum skips, like the native combination).
    flat = [float(x) for i, row in enumerate(a)
            for x in list(row) + [0.0] * (i + 1 - len(row))]
    ca = (ctypes.c_double * len(flat))(*flat) if flat else None
    cb = (ctypes.c_double * stages)(*[float(x) for x in b])
    u_out = torch.empty_like(u) if u_out is None else u_out
    v_out = torch.empty_like(v) if v_out is None else v_out
    ptrs = self._fields(u, v, u_out, v_out)
    nat.check(self._lib.cfd_fvm_step_rk(self._h, current_stream_ptr(u.device), *ptrs, int(steps),
                                        stages, ctypes.cast(ca, ctypes.c_void_p) if ca else None,
                                        ctypes.cast(cb, ctypes.c_void_p)), 'cfd_fvm_step_rk')
    return u_out, v_out

  def autotune(self, u, v, steps: int = 20) -> int:
    """Times each transform launch configuration on (u, v) and keeps the
    fastest; returns its index (row block shape + 2 * column-pass scheme +
    12 * stencil scheme + 24 * row feed).  Synchronises the stream."""
    us, vs = torch.empty_like(u), torch.empty_like(v)
    chosen = ctypes.c_int(-1)
    a = self._fields(u, v, us, vs)
    nat.check(self._lib.cfd_fvm_plan_autotune(self._h, current_stream_ptr(u.device), *a,
                                              int(steps), ctypes.byref(chosen)),
              'cfd_fvm_plan_autotune')
    return int(chosen.value)

  LAUNCH_CHOICES = 144
  ROW_BLOCKS = ('wide', 'narrow')
  COLUMN_PASSES = ('blocks', 'cluster4', 'cluster8', 'pipelined4', 'pipelined2',
                   'pipelined4_tma')
  STENCILS = ('tiles', 'warp_streams')
  ROW_FEEDS = ('registers', 'bulk_copy')
  STREAM_ROWS = (16, 8, 32)

  @classmethod
  def describe_launch(cls, choice: int) -> dict:
    """Names of the parts of launch configuration `choice` (row block shape
    + 2 * column-pass scheme + 12 * stencil scheme + 24 * row feed + 48 *
    rows per stencil warp, the index cfd_fvm_plan_autotune reports)."""
    choice = int(choice)
    if not 0 <= choice < cls.LAUNCH_CHOICES:
      raise ValueError(f'launch choice {choice} outside [0, {cls.LAUNCH_CHOICES})')
    return {'row_blocks': cls.ROW_BLOCKS[choice & 1],
            'column_pass': cls.COLUMN_PASSES[(choice >> 1) % 6],
            'stencil': cls.STENCILS[(choice // 12) & 1],
            'row_feed': cls.ROW_FEEDS[(choice // 24) & 1],
            'stream_rows': cls.STREAM_ROWS[choice // 48]}

  def set_launch(self, choice: int):
    """Pins the launch configuration (see autotune); results do not change."""
    nat.check(self._lib.cfd_fvm_plan_set_launch(self._h, int(choice)), 'cfd_fvm_plan_set_launch')

  @property
  def launch(self) -> int:
    return int(self._lib.cfd_fvm_plan_get_launch(self._h))

  PROFILE_KINDS = ('explicit', 'div_rfft', 'col_pinv', 'irfft', 'project_out')

  def profile(self, u, v, steps: int):
    """Mean per-launch duration (ms) of each kernel kind over `steps` steps,
    from CUDA events recorded around every launch on the current stream."""
    uo, vo = torch.empty_like(u), torch.empty_like(v)
    ms = (ctypes.c_float * 5)()
    a = self._fields(u, v, uo, vo)
    nat.check(self._lib.cfd_fvm_profile(self._h, current_stream_ptr(u.device), *a, int(steps),
                                        ctypes.cast(ms, ctypes.c_void_p)), 'cfd_fvm_profile')
    return dict(zip(self.PROFILE_KINDS, (float(x) for x in ms)))

  def adjoint_step(self, u, v, gu, gv, want_nu: bool = True):
    """Cotangent of the state before one step, given the cotangent (gu, gv) of
    the state after it; with want_nu also the per-cell products whose sum
    times dt / density is the viscosity derivative."""
    gu_out, gv_out = torch.empty_like(gu), torch.empty_like(gv)
    nu_dot = torch.empty_like(u) if want_nu else None
    a = self._fields(u, v, gu, gv, gu_out, gv_out)
    nat.check(self._lib.cfd_fvm_adjoint_step(self._h, current_stream_ptr(u.device), *a,
                                             ptr(nu_dot) if want_nu else None),
              'cfd_fvm_adjoint_step')
    return gu_out, gv_out, nu_dot

  def adjoint_segment(self, u0, v0, steps: int, gu, gv, nu_acc=None):
    """Adjoint of `steps` steps from the checkpoint (u0, v0) in one native
    call: recomputes the segment's states, then runs its adjoint steps newest
    first, updating the cotangent (gu, gv) in place (contiguous float32 on the
    plan's device) from the state after the segment to the checkpoint.  With
    nu_acc (a float64 device scalar) adds the segment's sum of the per-cell
    viscosity products to it."""
    steps = int(steps)
    if steps < 1:
      raise ValueError('steps must be >= 1')
    a = self._fields(u0, v0, gu, gv)
    if nu_acc is not None and not (nu_acc.dtype == torch.float64 and nu_acc.numel() == 1
                                   and nu_acc.device == u0.device):
      raise ValueError('nu_acc must be a float64 device scalar')
    states = (torch.empty((steps - 1, 2) + tuple(u0.shape), dtype=torch.float32,
                          device=u0.device) if steps > 1 else None)
    scratch = torch.empty_like(u0) if nu_acc is not None else None
    opt = lambda t: None if t is None else ptr(t)
    nat.check(self._lib.cfd_fvm_adjoint_segment(
        self._h, current_stream_ptr(u0.device), a[0], a[1], steps, opt(states), a[2], a[3],
        opt(scratch), opt(nu_acc)), 'cfd_fvm_adjoint_segment')

  def explicit_terms(self, u, v):
    du, dv = torch.empty_like(u), torch.empty_like(v)
    a = self._fields(u, v, du, dv)
    nat.check(self._lib.cfd_fvm_explicit_terms(self._h, current_stream_ptr(u.device), *a),
              'cfd_fvm_explicit_terms')
    return du, dv

  def projection(self, u, v):
    uo, vo = torch.empty_like(u), torch.empty_like(v)
    a = self._fields(u, v, uo, vo)
    nat.check(self._lib.cfd_fvm_projection(self._h, current_stream_ptr(u.device), *a),
              'cfd_fvm_projection')
    return uo, vo

  def pressure_solve(self, u, v):
    q = torch.empty_like(u)
    a = self._fields(u, v, q)
    nat.check(self._lib.cfd_fvm_pressure_solve(self._h, current_stream_ptr(u.device), *a),
              'cfd_fvm_pressure_solve')
    return q

  def divergence(self, u, v):
    out = torch.empty_like(u)
    a = self._fields(u, v, out)
    nat.check(self._lib.cfd_fvm_divergence(self._h, current_stream_ptr(u.device), *a),
              'cfd_fvm_divergence')
    return out

  def curl_2d(self, u, v):
    out = torch.empty_like(u)
    a = self._fields(u, v, out)
    nat.check(self._lib.cfd_fvm_curl_2d(self._h, current_stream_ptr(u.device), *a),
              'cfd_fvm_curl_2d')
    return out


def max_speed(u: torch.Tensor, v: torch.Tensor) -> torch.Tensor:
  """Device scalar max over cells of sqrt(u^2 + v^2)."""
  require_field(u, u.shape, name='u')
  require_field(v, u.shape, name='v')
  out = torch.empty((), dtype=torch.float32, device=u.device)
  nat.check(nat.load().cfd_max_speed(current_stream_ptr(u.device), u.numel(), ptr(u), ptr(v),
                                     ptr(out)), 'cfd_max_speed')
  return out


def scale_to_max_speed(u, v, vmax: torch.Tensor, maximum_velocity: float):
  """In place: u = (maximum_velocity * u) / vmax (same for v)."""
  nat.check(nat.load().cfd_scale_to_max_speed(
      current_stream_ptr(u.device), u.numel(), ptr(u), ptr(v), ptr(vmax),
      float(maximum_velocity)), 'cfd_scale_to_max_speed')


def spec_config(shape: Sequence[int], step: Sequence[float], *, viscosity: float = 0.0,
                drag: float = 0.0, dt: float = 0.0, smooth: bool = True,
                alphas=(0., 1.), betas=(0.,), gammas=(1.,)):
  """The C-ABI configuration of one spectral step; returns (config, arrays the
  config points into)."""
  coef = [np.ascontiguousarray(c, dtype=np.float64) for c in (alphas, betas, gammas)]
  if len(coef[0]) != len(coef[1]) + 1 or len(coef[1]) != len(coef[2]):
    raise ValueError('number of RK coefficients does not match')
  cfg = nat.SpecConfig()
  cfg.nx, cfg.ny = int(shape[0]), int(shape[1])
  cfg.hx, cfg.hy = float(step[0]), float(step[1])
  cfg.viscosity = float(viscosity)
  cfg.drag = float(drag)
  cfg.dt = float(dt)
  cfg.smooth = 1 if smooth else 0
  cfg.num_stages = len(coef[1])
  cfg.alphas, cfg.betas, cfg.gammas = (
      c.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) for c in coef)
  return cfg, coef


class SpecPlan:
  """Native plan for the pseudospectral step and the 2-D real transforms."""

  def __init__(self, shape: Sequence[int], step: Sequence[float], *,
               viscosity: float = 0.0, drag: float = 0.0, dt: float = 0.0,
               smooth: bool = True, alphas=(0., 1.), betas=(0.,), gammas=(1.,),
               device: Optional[torch.device] = None):
    if len(shape) != 2:
      raise NotImplementedError('only 2-D grids are on the GB300 hot path')
    self.shape = (int(shape[0]), int(shape[1]))
    self.half_shape = (self.shape[0], self.shape[1] // 2 + 1)
    self.device = torch.device(device) if device is not None else torch.device(
        'cuda', torch.cuda.current_device())
    cfg, self._coef = spec_config(self.shape, step, viscosity=viscosity, drag=drag, dt=dt,
                                  smooth=smooth, alphas=alphas, betas=betas, gammas=gammas)
    handle = ctypes.c_void_p()
    with torch.cuda.device(self.device):
      nat.check(nat.load().cfd_spec_plan_create(ctypes.byref(cfg), ctypes.byref(handle)),
                'cfd_spec_plan_create')
    self._h = handle
    self._lib = nat.load()

  def __del__(self):
    h = getattr(self, '_h', None)
    if h is not None and h.value:
      try:
        self._lib.cfd_spec_plan_destroy(h)
      except Exception:  # pylint: disable=broad-except
        pass
      self._h = None

  @property
  def handle(self):
    return self._h

  @property
  def nbytes(self) -> int:
    return int(self._lib.cfd_spec_plan_bytes(self._h))

  LAUNCH_CHOICES = 15
  COLUMN_PASSES = ('blocks', 'cluster4', 'pipelined4', 'pipelined2', 'pipelined4_fused')
  ROW_PASSES = ('shared_memory', 'register_passes', 'register_passes_high_occupancy')

  def set_launch(self, choice: int):
    """choice = column scheme + 5 * row scheme.  Column passes: 0 per-block
    columns, 1 clusters of four one-column blocks (256 <= nx <= 2048), 2/3
    persistent register-pipelined groups of 4/2 columns (512 <= nx <= 4096),
    4 as 2 with each stage's update and the next stage's prep fused.  Row
    pass: 0 shared-memory engine, 1 register passes (512 <= ny <= 4096), 2
    register passes with registers for three blocks per multiprocessor (four
    at ny = 2048; 512 <= ny <= 2048).  Results do not change."""
    nat.check(self._lib.cfd_spec_plan_set_launch(self._h, int(choice)), 'cfd_spec_plan_set_launch')

  @property
  def launch(self) -> int:
    return int(self._lib.cfd_spec_plan_get_launch(self._h))

  def autotune(self, w_hat: torch.Tensor, steps: int = 4) -> int:
    """Times `steps` steps from w_hat under each column-pass scheme this grid
    supports (CUDA events on the current stream, one untimed step first) and
    keeps the fastest; returns its index.  Synchronises the stream."""
    stream = torch.cuda.current_stream(w_hat.device)
    best, best_ms = self.launch, None
    for choice in range(self.LAUNCH_CHOICES):
      try:
        self.set_launch(choice)
      except NotImplementedError:
        continue
      self.step(w_hat, 1)
      e0 = torch.cuda.Event(enable_timing=True)
      e1 = torch.cuda.Event(enable_timing=True)
      e0.record(stream)
      self.step(w_hat, steps)
      e1.record(stream)
      e1.synchronize()
      ms = e0.elapsed_time(e1)
      if best_ms is None or ms < best_ms:
        best, best_ms = choice, ms
    self.set_launch(best)
    return best

  def _real(self, t, name='x'):
    return require_field(t, self.shape, name=name)

  def _half(self, t, name='xhat'):
    return require_field(t, self.half_shape, dtype=torch.complex64, name=name)

  def set_forcing(self, fx: Optional[torch.Tensor], fy: Optional[torch.Tensor]):
    a = []
    for t, name in ((fx, 'fx'), (fy, 'fy')):
      if t is None:
        a.append(None)
      else:
        a.append(ptr(self._real(t, name)))
    dev = (fx if fx is not None else fy).device if (fx is not None or fy is not None) else self.device
    nat.check(self._lib.cfd_spec_set_forcing(self._h, current_stream_ptr(dev), *a),
              'cfd_spec_set_forcing')

  def step(self, w_hat: torch.Tensor, steps: int, out: Optional[torch.Tensor] = None):
    if steps < 0:
      raise ValueError('steps must be non-negative')
    self._half(w_hat, 'vorticity_hat')
    out = torch.empty_like(w_hat) if out is None else self._half(out, 'out')
    nat.check(self._lib.cfd_spec_step(self._h, current_stream_ptr(w_hat.device), ptr(w_hat),
                                      ptr(out), int(steps)), 'cfd_spec_step')
    return out

  PROFILE_KINDS = ('row', 'col_update', 'col_prep', 'col_stage')

  def profile(self, w_hat: torch.Tensor, steps: int):
    """Mean per-launch duration (ms) of each spectral kernel kind."""
    self._half(w_hat, 'vorticity_hat')
    out = torch.empty_like(w_hat)
    ms = (ctypes.c_float * 4)()
    nat.check(self._lib.cfd_spec_profile(self._h, current_stream_ptr(w_hat.device), ptr(w_hat),
                                         ptr(out), int(steps), ctypes.cast(ms, ctypes.c_void_p)),
              'cfd_spec_profile')
    return dict(zip(self.PROFILE_KINDS, (float(x) for x in ms)))

  def explicit_terms(self, w_hat: torch.Tensor) -> torch.Tensor:
    self._half(w_hat, 'vorticity_hat')
    out = torch.empty_like(w_hat)
    nat.check(self._lib.cfd_spec_explicit_terms(self._h, current_stream_ptr(w_hat.device),
                                                ptr(w_hat), ptr(out)),
              'cfd_spec_explicit_terms')
    return out

  def rfft2(self, x: torch.Tensor) -> torch.Tensor:
    self._real(x)
    out = torch.empty(self.half_shape, dtype=torch.complex64, device=x.device)
    nat.check(self._lib.cfd_rfft2(self._h, current_stream_ptr(x.device), ptr(x), ptr(out)),
              'cfd_rfft2')
    return out

  def irfft2(self, xhat: torch.Tensor) -> torch.Tensor:
    self._half(xhat)
    out = torch.empty(self.shape, dtype=torch.float32, device=xhat.device)
    nat.check(self._lib.cfd_irfft2(self._h, current_stream_ptr(xhat.device), ptr(xhat),
                                   ptr(out)), 'cfd_irfft2')
    return out

  def spectral_filter(self, x: torch.Tensor, table: torch.Tensor) -> torch.Tensor:
    self._real(x)
    require_field(table, self.half_shape, name='table')
    out = torch.empty_like(x)
    nat.check(self._lib.cfd_spectral_filter(self._h, current_stream_ptr(x.device), ptr(x),
                                            ptr(table), ptr(out)), 'cfd_spectral_filter')
    return out


_PLAN_CACHE = {}


def cached(kind, key, factory):
  """Per-process cache of plans keyed by (kind, device, parameters)."""
  k = (kind, key)
  plan = _PLAN_CACHE.get(k)
  if plan is None:
    plan = factory()
    _PLAN_CACHE[k] = plan
  return plan


def clear_cache():
  _PLAN_CACHE.clear()
