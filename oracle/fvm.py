"""NumPy restatement of the reference's staggered-grid (FVM) hot path.

TEST INFRASTRUCTURE: the oracle the parity tests compare the CUDA path with, never
the product.

Every function cites the reference line range (paths relative to the jax-cfd
project root) whose arithmetic it follows.  A "variable" here is a pair
``(data, offset)``; periodic boundary conditions are implied throughout, so
``shift(c, k, axis)`` is ``c[i + k]`` with wrap-around
(``jax_cfd/base/boundaries.py:81-104,193-198``: pad mode 'wrap' then trim).
"""
from __future__ import annotations

import dataclasses
from typing import Callable, Optional, Sequence, Tuple

import numpy as np

Offset = Tuple[float, ...]


# ---------------------------------------------------------------------------
# Grid (jax_cfd/base/grids.py:499-675)
# ---------------------------------------------------------------------------
@dataclasses.dataclass(frozen=True)
class Grid:
  """Shape/step/domain of a periodic grid (grids.py:499-568)."""
  shape: Tuple[int, ...]
  step: Tuple[float, ...]
  domain: Tuple[Tuple[float, float], ...]

  @classmethod
  def make(cls, shape, step=None, domain=None) -> 'Grid':
    shape = tuple(int(s) for s in shape)
    if domain is not None:
      if isinstance(domain, (int, float)):
        domain = ((0, domain),) * len(shape)
      domain = tuple((float(lo), float(hi)) for lo, hi in domain)
    else:
      if step is None:
        step = 1
      if isinstance(step, (int, float)):
        step = (step,) * len(shape)
      domain = tuple((0.0, float(s * n)) for s, n in zip(step, shape))
    step = tuple((hi - lo) / n for (lo, hi), n in zip(domain, shape))
    return cls(shape, step, domain)

  @property
  def ndim(self):
    return len(self.shape)

  @property
  def cell_faces(self) -> Tuple[Offset, ...]:
    """grids.py:567-572."""
    d = self.ndim
    offsets = (np.eye(d) + np.ones([d, d])) / 2.
    return tuple(tuple(float(o) for o in off) for off in offsets)

  @property
  def cell_center(self) -> Offset:
    return (0.5,) * self.ndim

  def axes(self, offset=None, dtype=np.float32):
    """grids.py:588-610, evaluated in ``dtype`` like jnp with x64 off.

    ``lower + (arange(n) + offset) * step``: arange is int32 and the Python
    scalars are weakly typed, so every operation rounds to ``dtype``.
    """
    if offset is None:
      offset = self.cell_center
    out = []
    for (lo, _), o, n, s in zip(self.domain, offset, self.shape, self.step):
      t = np.dtype(dtype).type
      a = np.arange(n).astype(dtype)
      out.append(t(lo) + (a + t(o)) * t(s))
    return tuple(out)

  def mesh(self, offset=None, dtype=np.float32):
    """grids.py:640-653."""
    return tuple(np.meshgrid(*self.axes(offset, dtype), indexing='ij'))


def fftfreq(n: int, d: float, dtype=np.float32) -> np.ndarray:
  """jnp.fft.fftfreq: integer ordinals divided by ``d * n`` in ``dtype``."""
  k = np.concatenate([np.arange(0, (n - 1) // 2 + 1),
                      np.arange(-(n // 2), 0)]).astype(dtype)
  return k / np.dtype(dtype).type(d * n)


def rfftfreq(n: int, d: float, dtype=np.float32) -> np.ndarray:
  k = np.arange(0, n // 2 + 1).astype(dtype)
  return k / np.dtype(dtype).type(d * n)


def rfft_mesh(grid: Grid, dtype=np.float32):
  """grids.py:618-658 (rfft_axes + meshgrid 'ij')."""
  axes = [fftfreq(n, s, dtype) for n, s in zip(grid.shape[:-1], grid.step[:-1])]
  axes.append(rfftfreq(grid.shape[-1], grid.step[-1], dtype))
  return tuple(np.meshgrid(*axes, indexing='ij'))


def shift(c: np.ndarray, k: int, axis: int) -> np.ndarray:
  """Periodic ``c.shift(k, axis)``: result[i] = c[i + k] (boundaries.py:81-104)."""
  if k == 0:
    return c
  return np.roll(c, -k, axis=axis)


def control_volume_offsets(offset: Offset) -> Tuple[Offset, ...]:
  """grids.py:448-454."""
  return tuple(tuple(o + .5 if i == j else o for i, o in enumerate(offset))
               for j in range(len(offset)))


# ---------------------------------------------------------------------------
# Interpolation (jax_cfd/base/interpolation.py)
# ---------------------------------------------------------------------------
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
  data = floor_weight * shift(c, floor, axis) + ceil_weight * shift(c, ceil, axis)
  return data, new_off


def linear(c, c_off, offset):
  """interpolation.py:66-93."""
  if len(offset) != len(c_off):
    raise ValueError('offset length mismatch')
  for a, o in enumerate(offset):
    c, c_off = _linear_along_axis(c, c_off, o, a)
  return c, c_off


def _interp_axis(c_off, offset):
  axes = tuple(a for a, (cur, tgt) in enumerate(zip(c_off, offset)) if cur != tgt)
  if len(axes) != 1:
    raise ValueError(f'offsets must differ in exactly one entry: {c_off} {offset}')
  return axes[0]


def upwind(c, c_off, offset, v):
  """interpolation.py:96-155. ``v`` is a tuple of (data, offset) or None."""
  if tuple(c_off) == tuple(offset):
    return c, c_off
  axis = _interp_axis(c_off, offset)
  u, u_off = v[axis]
  delta = u_off[axis] - c_off[axis]
  if int(delta) == delta:
    return shift(c, int(delta), axis), tuple(offset)
  floor = int(np.floor(delta))
  ceil = int(np.ceil(delta))
  return np.where(u > 0, shift(c, floor, axis), shift(c, ceil, axis)), tuple(offset)


def lax_wendroff(c, c_off, offset, v, dt, step):
  """interpolation.py:158-221."""
  if tuple(c_off) == tuple(offset):
    return c, c_off
  axis = _interp_axis(c_off, offset)
  u, u_off = v[axis]
  delta = u_off[axis] - c_off[axis]
  floor = int(np.floor(delta))
  ceil = int(np.ceil(delta))
  courant = (dt / step[axis]) * u
  c_f = shift(c, floor, axis)
  c_c = shift(c, ceil, axis)
  pos = c_f + 0.5 * (1 - courant) * (c_c - c_f)
  neg = c_c - 0.5 * (1 + courant) * (c_c - c_f)
  return np.where(u > 0, pos, neg), tuple(offset)


def safe_div(x, y, default_numerator=1):
  """interpolation.py:224-226."""
  with np.errstate(divide='ignore', invalid='ignore'):
    return x / np.where(y != 0, y, default_numerator)


def van_leer_limiter(r):
  """interpolation.py:229-231."""
  return np.where(r > 0, safe_div(2 * r, 1 + r), 0.0).astype(r.dtype)


def tvd_interpolation(c, c_off, offset, v, dt, step,
                      interpolation_fn=lax_wendroff, limiter=van_leer_limiter):
  """``apply_tvd_limiter(interpolation_fn, limiter)`` (interpolation.py:234-303)."""
  for axis, axis_offset in enumerate(offset):
    interp_off = tuple(co if i != axis else axis_offset for i, co in enumerate(c_off))
    if interp_off != tuple(c_off):
      if interp_off[axis] - c_off[axis] != 0.5:
        raise NotImplementedError('only forward interpolation to CV faces')
      c_low, _ = upwind(c, c_off, offset, v)
      c_high, _ = interpolation_fn(c, c_off, offset, v, dt, step)
      c_left = shift(c, -1, axis)
      c_right = shift(c, 1, axis)
      c_next_right = shift(c, 2, axis)
      pos_r = safe_div(c - c_left, c_right - c)
      neg_r = safe_div(c_next_right - c_right, c_right - c)
      pos_phi = limiter(pos_r)
      neg_phi = limiter(neg_r)
      u, _ = v[axis]
      phi = np.where(u > 0, pos_phi, neg_phi)
      c = c_low - (c_low - c_high) * phi
      c_off = interp_off
  return c, c_off


# ---------------------------------------------------------------------------
# Finite differences (jax_cfd/base/finite_differences.py)
# ---------------------------------------------------------------------------
def backward_difference(c, axis, step):
  """finite_differences.py:95-102: (0 + c + (-c[i-1])) / h."""
  return (c - shift(c, -1, axis)) / step[axis]


def forward_difference(c, axis, step):
  """finite_differences.py:117-124: (c[i+1] - c) / h."""
  return (shift(c, 1, axis) - c) / step[axis]


def laplacian(c, step):
  """finite_differences.py:127-133 (scales formed in the array dtype)."""
  scales = np.square(1 / np.array(step, dtype=c.dtype))
  result = -2 * c * np.sum(scales)
  for axis in range(c.ndim):
    result = result + (shift(c, -1, axis) + shift(c, 1, axis)) * scales[axis]
  return result


def divergence(v: Sequence[np.ndarray], step):
  """finite_differences.py:136-143: sum of backward differences (from 0)."""
  out = 0
  for axis, u in enumerate(v):
    out = out + backward_difference(u, axis, step)
  return out


def curl_2d(v, step):
  """finite_differences.py:186-193; result at offset (1, 1)."""
  return forward_difference(v[1], 0, step) - forward_difference(v[0], 1, step)


# ---------------------------------------------------------------------------
# Advection (jax_cfd/base/advection.py)
# ---------------------------------------------------------------------------
def advect_general(c, c_off, v, v_offs, dt, step, u_interp, c_interp):
  """advection.py:34-78 (_advect_aligned) and 81-116 (advect_general)."""
  targets = control_volume_offsets(c_off)
  aligned_v = tuple(u_interp(u, uo, t, dt, step, v, v_offs)
                    for u, uo, t in zip(v, v_offs, targets))
  aligned_c = tuple(c_interp(c, c_off, t, aligned_v, dt, step) for t in targets)
  flux = tuple(ac[0] * av[0] for ac, av in zip(aligned_c, aligned_v))
  return -divergence(flux, step)


def _linear_u(u, uo, target, dt, step, v, v_offs):
  return linear(u, uo, target)


def _tvd_c(c, c_off, target, aligned_v, dt, step):
  return tvd_interpolation(c, c_off, target, aligned_v, dt, step)


def _linear_c(c, c_off, target, aligned_v, dt, step):
  return linear(c, c_off, target)


def advect_van_leer_using_limiters(c, c_off, v, v_offs, dt, step):
  """advection.py:387-395."""
  return advect_general(c, c_off, v, v_offs, dt, step, _linear_u, _tvd_c)


def advect_linear(c, c_off, v, v_offs, dt, step):
  """advection.py:119-126 (linear interpolation of both c and v)."""
  return advect_general(c, c_off, v, v_offs, dt, step, _linear_u, _linear_c)


def advective_stable_time_step(max_velocity, max_courant_number, grid: Grid):
  """advection.py:398-416."""
  return max_courant_number * min(grid.step) / max_velocity


def diffusive_stable_time_step(viscosity, grid: Grid):
  """diffusion.py:40-57."""
  if viscosity == 0:
    return float('inf')
  return min(grid.step) ** 2 / (viscosity * 2 ** grid.ndim)


def stable_time_step(max_velocity, max_courant_number, viscosity, grid,
                     implicit_diffusion=False):
  """equations.py:45-59 (raises like the reference)."""
  dt = advective_stable_time_step(max_velocity, max_courant_number, grid)
  if not implicit_diffusion:
    ddt = diffusive_stable_time_step(viscosity, grid)
    if ddt < dt:
      raise ValueError(f'stable time step for diffusion is smaller than '
                       f'the chosen timestep: {ddt} vs {dt}')
  return dt


# ---------------------------------------------------------------------------
# Forcings (jax_cfd/base/forcings.py)
# ---------------------------------------------------------------------------
def kolmogorov_forcing(grid: Grid, scale=1, k=2, swap_xy=False, offsets=None,
                       dtype=np.float32):
  """forcings.py:63-104; returns a function of the velocity tuple."""
  if offsets is None:
    offsets = grid.cell_faces
  if swap_xy:
    x = grid.mesh(offsets[1], dtype)[0]
    fv = scale * np.sin(k * x)
    fu = np.zeros_like(fv)
  else:
    y = grid.mesh(offsets[0], dtype)[1]
    fu = scale * np.sin(k * y)
    fv = np.zeros_like(fu)
  f = (fu.astype(dtype), fv.astype(dtype))
  return lambda v: f


def linear_forcing(grid: Grid, coefficient: float):
  """forcings.py:107-113."""
  return lambda v: tuple(coefficient * u for u in v)


def sum_forcings(*forcings):
  """forcings.py:125-129 and equations.py:42 (``sum`` starts from 0)."""
  def forcing(v):
    parts = [f(v) for f in forcings]
    out = []
    for comp in zip(*parts):
      acc = 0
      for a in comp:
        acc = acc + a
      out.append(acc)
    return tuple(out)
  return forcing


def simple_turbulence_forcing(grid: Grid, constant_magnitude=0,
                              constant_wavenumber=2, linear_coefficient=0,
                              forcing_type='kolmogorov', dtype=np.float32):
  """forcings.py:136-178 (kolmogorov branch)."""
  if forcing_type != 'kolmogorov':
    raise NotImplementedError(forcing_type)
  lin = linear_forcing(grid, linear_coefficient)
  const = kolmogorov_forcing(grid, constant_magnitude, constant_wavenumber,
                             dtype=dtype)
  return sum_forcings(lin, const)


# ---------------------------------------------------------------------------
# Pressure (pressure.py, fast_diagonalization.py, array_utils.py)
# ---------------------------------------------------------------------------
def laplacian_matrix(size: int, step: float) -> np.ndarray:
  """array_utils.py:168-173 (circulant [-2, 1, 0, ..., 0, 1] / h^2)."""
  column = np.zeros(size)
  column[0] = -2 / step ** 2
  column[1] = column[-1] = 1 / step ** 2
  idx = (np.arange(size)[:, None] - np.arange(size)[None, :]) % size
  return column[idx]


def pinv_diagonal(grid: Grid, dtype=np.float32) -> np.ndarray:
  """Diagonal of the rfft pseudoinverse (fast_diagonalization.py:199-225,228-266).

  Eigenvalues are ``fft`` of each circulant's first column (``rfft`` on the
  last axis), summed by outer addition in float64; ``1/lambda`` where
  ``|lambda| > 10 * eps(dtype)`` else 0; then cast to the complex dtype
  (``jnp.asarray`` with x64 off gives complex64).
  """
  ops = [laplacian_matrix(n, s) for n, s in zip(grid.shape, grid.step)]
  eig = [np.fft.fft(op[:, 0]) for op in ops[:-1]] + [np.fft.rfft(ops[-1][:, 0])]
  summed = eig[0]
  for e in eig[1:]:
    summed = np.add.outer(summed, e)
  cutoff = 10 * np.finfo(dtype).eps
  with np.errstate(divide='ignore', invalid='ignore'):
    diag = np.where(abs(summed) > cutoff, 1 / summed, 0)
  cdtype = np.complex64 if dtype == np.float32 else np.complex128
  return diag.astype(cdtype)


def fast_diag_pinv(rhs, grid: Grid, diag=None):
  """Pseudoinverse of the periodic Laplacian applied to ``rhs`` through the
  rfft diagonalisation (fast_diagonalization.py:199-225, 228-266)."""
  if diag is None:
    diag = pinv_diagonal(grid, rhs.dtype)
  axes = tuple(range(rhs.ndim))
  out = np.fft.irfftn(diag * np.fft.rfftn(rhs), s=rhs.shape, axes=axes)
  return out.astype(rhs.dtype)


def solve_fast_diag(v, grid: Grid, diag=None):
  """pressure.py:115-157 with the periodic 'rfft' implementation."""
  rhs = divergence(v, grid.step)
  if grid.shape[-1] % 2:
    raise ValueError('rfft requires an even last axis')
  if diag is None:
    diag = pinv_diagonal(grid, rhs.dtype)
  axes = tuple(range(rhs.ndim))
  out = np.fft.irfftn(diag * np.fft.rfftn(rhs), s=rhs.shape, axes=axes)
  return out.real.astype(rhs.dtype) if np.iscomplexobj(out) else out.astype(rhs.dtype)


def projection(v, grid: Grid, diag=None):
  """pressure.py:181-198: v - forward_difference(q)."""
  q = solve_fast_diag(v, grid, diag)
  return tuple(u - forward_difference(q, axis, grid.step)
               for axis, u in enumerate(v))


# ---------------------------------------------------------------------------
# Implicit diffusion (diffusion.py, fast_diagonalization.py)
# ---------------------------------------------------------------------------
def diffusion_diagonal(grid: Grid, nu, dt, dtype=np.float32) -> np.ndarray:
  """diffusion.py:176-182 ``func`` on the summed eigenvalues of the periodic
  Laplacians (fast_diagonalization.py:199-225): ``x = (dt * nu) * lambda``,
  ``x / (1 - x)`` in float64, then cast to the complex dtype."""
  ops = [laplacian_matrix(n, s) for n, s in zip(grid.shape, grid.step)]
  eig = [np.fft.fft(op[:, 0]) for op in ops[:-1]] + [np.fft.rfft(ops[-1][:, 0])]
  summed = eig[0]
  for e in eig[1:]:
    summed = np.add.outer(summed, e)
  dt_nu_x = (dt * nu) * summed
  diag = dt_nu_x / (1 - dt_nu_x)
  cdtype = np.complex64 if dtype == np.float32 else np.complex128
  return diag.astype(cdtype)


def diffusion_solve_fast_diag(v, nu, dt, grid: Grid, diag=None):
  """diffusion.py:166-212 for periodic components: u + irfftn(diag * rfftn(u))
  (the 'rfft' transform, fast_diagonalization.py:199-225)."""
  if diag is None:
    diag = diffusion_diagonal(grid, nu, dt, v[0].dtype)
  out = []
  for u in v:
    axes = tuple(range(u.ndim))
    w = np.fft.irfftn(diag * np.fft.rfftn(u), s=u.shape, axes=axes).astype(u.dtype)
    out.append(u + w)
  return tuple(out)


# ---------------------------------------------------------------------------
# Equations and time stepping (equations.py, time_stepping.py)
# ---------------------------------------------------------------------------
ButcherTableau = Tuple[Sequence[Sequence[float]], Sequence[float]]
FORWARD_EULER: ButcherTableau = ([], [1])
MIDPOINT_RK2: ButcherTableau = ([[1 / 2]], [0, 1])
HEUN_RK2: ButcherTableau = ([[1]], [1 / 2, 1 / 2])
CLASSIC_RK4: ButcherTableau = ([[1 / 2], [0, 1 / 2], [0, 0, 1]],
                               [1 / 6, 1 / 3, 1 / 3, 1 / 6])


def explicit_terms_fn(density, viscosity, dt, grid: Grid, convect='van_leer',
                      forcing: Optional[Callable] = None):
  """equations.py:77-116 (``navier_stokes_explicit_terms``)."""
  offs = grid.cell_faces
  step = grid.step
  if convect == 'van_leer':
    adv = advect_van_leer_using_limiters
  elif convect == 'linear':
    adv = advect_linear
  else:
    raise ValueError(convect)

  def terms(v):
    dv = [adv(u, o, v, offs, dt, step) for u, o in zip(v, offs)]
    if viscosity is not None:
      nu = viscosity / density
      dv = [d + nu * laplacian(u, step) for d, u in zip(dv, v)]
    if forcing is not None:
      f = forcing(v)
      dv = [d + fi / density for d, fi in zip(dv, f)]
    return tuple(dv)
  return terms


def navier_stokes_rk(tableau: ButcherTableau, F, P, dt):
  """time_stepping.py:59-107 (reference method, eqs 16-21)."""
  a, b = tableau
  n = len(b)

  def combo(coeffs, ks):
    acc = 0
    for c_j, k_j in zip(coeffs, ks):
      if c_j:
        acc = acc + c_j * k_j
    return acc

  def step_fn(u0):
    k = [None] * n
    k[0] = F(u0)
    for i in range(1, n):
      u_star = tuple(u0[d] + dt * combo(a[i - 1], [kk[d] for kk in k[:i]])
                     for d in range(len(u0)))
      k[i] = F(P(u_star))
    u_star = tuple(u0[d] + dt * combo(b, [kk[d] for kk in k])
                   for d in range(len(u0)))
    return P(u_star)
  return step_fn


def semi_implicit_navier_stokes(density, viscosity, dt, grid: Grid,
                                convect='van_leer', forcing=None,
                                tableau: ButcherTableau = FORWARD_EULER,
                                diag=None):
  """equations.py:120-151 with pressure_solve=solve_fast_diag."""
  F = explicit_terms_fn(density, viscosity, dt, grid, convect, forcing)
  cache = {}

  def P(v):
    d = diag
    if d is None:
      key = v[0].dtype
      if key not in cache:
        cache[key] = pinv_diagonal(grid, v[0].dtype)
      d = cache[key]
    return projection(v, grid, d)
  return navier_stokes_rk(tableau, F, P, dt)


def implicit_diffusion_navier_stokes(density, viscosity, dt, grid: Grid,
                                     convect='van_leer', forcing=None):
  """equations.py:154-195 with diffusion_solve = pressure_solve =
  solve_fast_diag: v + dvdt * dt with dvdt = convection + forcing / density
  (sum_fields from 0), projection, then the implicit diffusion solve."""
  F = explicit_terms_fn(density, None, dt, grid, convect, forcing)
  cache = {}

  def step(v):
    dvdt = F(v)
    v = tuple(u + d * dt for u, d in zip(v, dvdt))
    key = v[0].dtype
    if key not in cache:
      cache[key] = (pinv_diagonal(grid, key), diffusion_diagonal(grid, viscosity, dt, key))
    pd, dd = cache[key]
    v = projection(v, grid, pd)
    return diffusion_solve_fast_diag(v, viscosity, dt, grid, dd)
  return step


def repeated(f, steps):
  """funcutils.py:82-88."""
  def run(x):
    for _ in range(steps):
      x = f(x)
    return x
  return run


def trajectory(step_fn, steps, post_process=lambda x: x, start_with_input=False):
  """funcutils.py:95-126 (frames stacked along a new leading axis)."""
  def run(x):
    frames = []
    for _ in range(steps):
      y = step_fn(x)
      frames.append(post_process(x if start_with_input else y))
      x = y
    if frames and isinstance(frames[0], tuple):
      stacked = tuple(np.stack(c) for c in zip(*frames))
    else:
      stacked = np.stack(frames) if frames else frames
    return x, stacked
  return run
