"""NumPy restatement of the reference's pseudospectral vorticity step.

TEST INFRASTRUCTURE: the oracle the parity tests compare the CUDA path with, never
the product.

Follows ``jax_cfd/spectral/equations.py:129-220``, ``spectral/utils.py:128-134,
154-203`` and ``spectral/time_stepping.py:117-197``.  The state is the
``rfftn`` of the vorticity, complex64 ``[nx, ny//2+1]`` (complex128 in the
float64 stand-in for ``jax_enable_x64``).  Expressions keep the reference's
association so that NumPy's NEP 50 weak-scalar rules round exactly where JAX's
do.
"""
from __future__ import annotations

from typing import Callable, Optional, Sequence

import numpy as np

from oracle import fvm

CN_RK4_ALPHAS = [0, 0.1496590219993, 0.3704009573644, 0.6222557631345,
                 0.9582821306748, 1]
CN_RK4_BETAS = [0, -0.4178904745, -1.192151694643, -1.697784692471,
                -1.514183444257]
CN_RK4_GAMMAS = [0.1496590219993, 0.3792103129999, 0.8229550293869,
                 0.6994504559488, 0.1530572479681]
CN_RK3_ALPHAS = [0, 1 / 3, 3 / 4, 1]
CN_RK3_BETAS = [0, -5 / 9, -153 / 128]
CN_RK3_GAMMAS = [1 / 3, 15 / 16, 8 / 15]


def brick_wall_filter_2d(grid: fvm.Grid, dtype=np.float32):
  """spectral/utils.py:128-134 (note the asymmetric negative-row slice)."""
  n, m = grid.shape
  f = np.zeros((n, m // 2 + 1), dtype)
  f[:int(2 / 3 * n) // 2, :int(2 / 3 * (m // 2 + 1))] = 1
  f[-int(2 / 3 * n) // 2:, :int(2 / 3 * (m // 2 + 1))] = 1
  return f


def vorticity_to_velocity(grid: fvm.Grid, dtype=np.float32):
  """spectral/utils.py:154-189."""
  kx, ky = fvm.rfft_mesh(grid, dtype)
  two_pi_i = 2 * np.pi * 1j
  laplace = two_pi_i ** 2 * (abs(kx) ** 2 + abs(ky) ** 2)
  laplace[0, 0] = 1

  def ret(vorticity_hat):
    psi_hat = -1 / laplace * vorticity_hat
    vxhat = two_pi_i * ky * psi_hat
    vyhat = -two_pi_i * kx * psi_hat
    return vxhat, vyhat
  return ret


def spectral_curl_2d(mesh, velocity_hat):
  """spectral/utils.py:199-203."""
  kx, ky = mesh
  uhat, vhat = velocity_hat
  return 2j * np.pi * (vhat * kx - uhat * ky)


class NavierStokes2D:
  """spectral/equations.py:129-191.

  ``forcing`` is a function ``grid -> (velocity -> (fx, fy))`` like the
  reference's ``forcing_fn``; the forcing used on the hot path
  (``kolmogorov_forcing``) ignores the velocity.
  """

  def __init__(self, viscosity, grid: fvm.Grid, drag=0., smooth=True,
               forcing_fn: Optional[Callable] = None, dtype=np.float32):
    self.viscosity = viscosity
    self.grid = grid
    self.drag = drag
    self.smooth = smooth
    self.dtype = dtype
    self.kx, self.ky = fvm.rfft_mesh(grid, dtype)
    self.laplace = (np.pi * 2j) ** 2 * (self.kx ** 2 + self.ky ** 2)
    self.filter_ = brick_wall_filter_2d(grid, dtype)
    self.linear_term = self.viscosity * self.laplace - self.drag
    self._forcing = forcing_fn(grid) if forcing_fn is not None else None
    self._velocity_solve = vorticity_to_velocity(grid, dtype)

  def explicit_terms(self, vorticity_hat):
    """spectral/equations.py:160-184."""
    s = self.grid.shape
    vxhat, vyhat = self._velocity_solve(vorticity_hat)
    ax = (0, 1)
    vx, vy = np.fft.irfftn(vxhat, s=s, axes=ax), np.fft.irfftn(vyhat, s=s, axes=ax)
    grad_x_hat = 2j * np.pi * self.kx * vorticity_hat
    grad_y_hat = 2j * np.pi * self.ky * vorticity_hat
    grad_x = np.fft.irfftn(grad_x_hat, s=s, axes=ax)
    grad_y = np.fft.irfftn(grad_y_hat, s=s, axes=ax)
    advection = -(grad_x * vx + grad_y * vy)
    advection_hat = np.fft.rfftn(advection)
    if self.smooth is not None:
      advection_hat = advection_hat * self.filter_
    terms = advection_hat
    if self._forcing is not None:
      fx, fy = self._forcing((vx, vy))
      fx_hat, fy_hat = np.fft.rfft2(fx), np.fft.rfft2(fy)
      terms = terms + spectral_curl_2d((self.kx, self.ky), (fx_hat, fy_hat))
    return terms

  def implicit_terms(self, vorticity_hat):
    return self.linear_term * vorticity_hat

  def implicit_solve(self, vorticity_hat, time_step):
    return 1 / (1 - time_step * self.linear_term) * vorticity_hat


def forced_navier_stokes_2d(viscosity, grid: fvm.Grid, smooth=True,
                            dtype=np.float32):
  """spectral/equations.py:194-220 (Kolmogorov k=4 at offset 0, drag 0.1)."""
  forcing_fn = lambda g: fvm.kolmogorov_forcing(
      g, k=4, offsets=((0, 0), (0, 0)), dtype=dtype)
  return NavierStokes2D(viscosity, grid, drag=0.1, smooth=smooth,
                        forcing_fn=forcing_fn, dtype=dtype)


def low_storage_runge_kutta_crank_nicolson(alphas, betas, gammas, equation,
                                           time_step):
  """spectral/time_stepping.py:117-170."""
  a, b, g = alphas, betas, gammas
  dt = time_step
  F, G, G_inv = (equation.explicit_terms, equation.implicit_terms,
                 equation.implicit_solve)
  if len(alphas) - 1 != len(betas) != len(gammas):
    raise ValueError('number of RK coefficients does not match')

  def step_fn(u):
    h = 0
    for k in range(len(b)):
      h = F(u) + b[k] * h
      mu = 0.5 * dt * (a[k + 1] - a[k])
      u = G_inv(u + g[k] * dt * h + mu * G(u), mu)
    return u
  return step_fn


def crank_nicolson_rk4(equation, time_step):
  """spectral/time_stepping.py:186-197."""
  return low_storage_runge_kutta_crank_nicolson(
      CN_RK4_ALPHAS, CN_RK4_BETAS, CN_RK4_GAMMAS, equation, time_step)


def crank_nicolson_rk3(equation, time_step):
  """spectral/time_stepping.py:173-183."""
  return low_storage_runge_kutta_crank_nicolson(
      CN_RK3_ALPHAS, CN_RK3_BETAS, CN_RK3_GAMMAS, equation, time_step)
