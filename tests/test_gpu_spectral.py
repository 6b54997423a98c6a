"""GPU parity of the pseudospectral path against the NumPy oracle.

Bar: per-step relative L2 <= 1e-5 on the vorticity spectrum (float32 state).
"""
import numpy as np
import pytest
import torch

from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu

STEP_TOL = 1e-5
TWO_PI = 2 * np.pi


def _vorticity_hat(shape, seed=0):
  from oracle import fvm as ofvm
  from oracle import initial_conditions as oic
  og = ofvm.Grid.make(shape, domain=((0, TWO_PI), (0, TWO_PI)))
  v0 = oic.filtered_velocity_field(seed, og, 2.0, 4)
  return og, np.fft.rfftn(ofvm.curl_2d(v0, og.step))


@pytest.mark.parametrize('shape', [(4, 4), (8, 16), (64, 64), (256, 128), (2048, 2048)])
def test_rfft2_irfft2(cuda_device, shape):
  import jax_cfd_gb300.base as cfd
  from jax_cfd_gb300.spectral import utils as su
  grid = cfd.grids.Grid(shape)
  x = np.random.default_rng(1).standard_normal(shape).astype(np.float32)
  xt = torch.from_numpy(x).to(cuda_device)
  xh = su.rfft2(xt, grid)
  want = np.fft.rfftn(x.astype(np.float64))
  assert rel_l2(xh.cpu().numpy(), want) <= 1e-6
  back = su.irfft2(xh, grid).cpu().numpy()
  assert rel_l2(back, x) <= 1e-6


@pytest.mark.parametrize('shape', [(16, 16), (64, 64), (128, 64), (64, 2048)])
@pytest.mark.parametrize('forced', [False, True])
def test_explicit_terms_match_oracle(cuda_device, shape, forced):
  import jax_cfd_gb300.base as cfd
  from jax_cfd_gb300.spectral import equations as seq
  from oracle import spectral as ospec
  og, w0 = _vorticity_hat(shape)
  grid = cfd.grids.Grid(shape, domain=((0, TWO_PI), (0, TWO_PI)))
  if forced:
    eq = seq.ForcedNavierStokes2D(1e-3, grid, smooth=True)
    oeq = ospec.forced_navier_stokes_2d(1e-3, og)
  else:
    eq = seq.NavierStokes2D(1e-3, grid, smooth=True)
    oeq = ospec.NavierStokes2D(1e-3, og, smooth=True)
  got = eq.explicit_terms(torch.from_numpy(w0).to(cuda_device)).cpu().numpy()
  assert rel_l2(got, oeq.explicit_terms(w0)) <= STEP_TOL


@pytest.mark.parametrize('shape', [(16, 16), (64, 64), (256, 256), (64, 128), (128, 512),
                                   (64, 1024), (256, 2048)])
def test_cn_rk4_step_matches_oracle(cuda_device, shape):
  import jax_cfd_gb300.base as cfd
  from jax_cfd_gb300.spectral import equations as seq
  from jax_cfd_gb300.spectral import time_stepping as sts
  from oracle import spectral as ospec
  og, w0 = _vorticity_hat(shape)
  grid = cfd.grids.Grid(shape, domain=((0, TWO_PI), (0, TWO_PI)))
  eq = seq.ForcedNavierStokes2D(1e-3, grid, smooth=True)
  step = sts.crank_nicolson_rk4(eq, 1e-3)
  got = step(torch.from_numpy(w0).to(cuda_device)).cpu().numpy()
  want = ospec.crank_nicolson_rk4(ospec.forced_navier_stokes_2d(1e-3, og), 1e-3)(w0)
  assert rel_l2(got, want) <= STEP_TOL


def test_repeated_steps_track_oracle(cuda_device):
  import jax_cfd_gb300.base as cfd
  from jax_cfd_gb300.spectral import equations as seq
  from jax_cfd_gb300.spectral import time_stepping as sts
  from oracle import fvm as ofvm
  from oracle import spectral as ospec
  og, w0 = _vorticity_hat((64, 64))
  grid = cfd.grids.Grid((64, 64), domain=((0, TWO_PI), (0, TWO_PI)))
  step = sts.crank_nicolson_rk4(seq.ForcedNavierStokes2D(1e-3, grid, smooth=True), 1e-3)
  got = cfd.funcutils.repeated(step, 20)(torch.from_numpy(w0).to(cuda_device)).cpu().numpy()
  want = ofvm.repeated(ospec.crank_nicolson_rk4(ospec.forced_navier_stokes_2d(1e-3, og), 1e-3),
                       20)(w0)
  assert rel_l2(got, want) <= 20 * STEP_TOL


def test_forced_turbulence_no_nan(cuda_device):
  """spectral/equations_test.py:213-233: 100 steps at dt=1e-5 stay finite."""
  import jax_cfd_gb300.base as cfd
  from jax_cfd_gb300.spectral import equations as seq
  from jax_cfd_gb300.spectral import time_stepping as sts
  _, w0 = _vorticity_hat((128, 128), seed=42)
  grid = cfd.grids.Grid((128, 128), domain=((0, TWO_PI), (0, TWO_PI)))
  eq = seq.NavierStokes2D(1e-3, grid, forcing_fn=cfd.forcings.kolmogorov_forcing, drag=0.1)
  _, traj = cfd.funcutils.trajectory(sts.crank_nicolson_rk4(eq, 1e-5), 100)(
      torch.from_numpy(w0).to(cuda_device))
  assert torch.isfinite(torch.view_as_real(traj)).all()


def test_taylor_green_spectral_analytic(cuda_device):
  """spectral/equations_test.py:235-270 analogue at 256^2."""
  import jax_cfd_gb300.base as cfd
  from jax_cfd_gb300.spectral import equations as seq
  from jax_cfd_gb300.spectral import time_stepping as sts
  from oracle import fvm as ofvm
  n, nu, t_end = 256, 1e-3, 0.11
  og = ofvm.Grid.make((n, n), domain=((0, TWO_PI), (0, TWO_PI)))
  grid = cfd.grids.Grid((n, n), domain=((0, TWO_PI), (0, TWO_PI)))

  def tg(t):
    s = np.float32(np.exp(-2 * nu * t))
    ux, uy = og.mesh(og.cell_faces[0])
    vx, vy = og.mesh(og.cell_faces[1])
    return (s * np.cos(ux) * np.sin(uy), -s * np.sin(vx) * np.cos(vy))
  w = ofvm.curl_2d(tg(0.0), og.step)
  dt = cfd.equations.stable_time_step(7, 0.5, nu, grid, implicit_diffusion=True)
  steps = int(np.ceil(t_end / dt))
  step = sts.crank_nicolson_rk4(seq.NavierStokes2D(nu, grid, drag=0), dt)
  out = cfd.funcutils.repeated(step, steps)(torch.from_numpy(np.fft.rfftn(w)).to(cuda_device))
  got = np.fft.irfftn(out.cpu().numpy(), s=(n, n), axes=(0, 1))
  want = ofvm.curl_2d(tg(steps * dt), og.step)
  assert np.abs(got - want).max() <= 1e-3


@pytest.mark.parametrize('shape', [(256, 256), (512, 256), (256, 1024), (2048, 2048)])
@pytest.mark.parametrize('forcing', ['smooth', 'kolmogorov'])
def test_cluster_column_passes_are_bitwise(cuda_device, shape, forcing):
  """Every column scheme (per-block, clusters, persistent pipelined, fused
  update + prep) and every row pass (shared memory, register passes at two or
  three blocks per multiprocessor) give exactly the per-block bits."""
  import jax_cfd_gb300.base as cfd
  from jax_cfd_gb300.spectral import equations as seq
  from jax_cfd_gb300.spectral import time_stepping as sts
  _, w0 = _vorticity_hat(shape, seed=3)
  grid = cfd.grids.Grid(shape, domain=((0, TWO_PI), (0, TWO_PI)))
  if forcing == 'smooth':
    eq = seq.ForcedNavierStokes2D(1e-3, grid, smooth=True)
  else:
    eq = seq.NavierStokes2D(1e-3, grid, forcing_fn=cfd.forcings.kolmogorov_forcing, drag=0.1)
  plan = sts.crank_nicolson_rk4(eq, 1e-3).plan(cuda_device)
  w = torch.from_numpy(w0.astype(np.complex64)).to(cuda_device)
  default = plan.launch
  results = {}
  try:
    for choice in range(plan.LAUNCH_CHOICES):
      try:
        plan.set_launch(choice)
      except NotImplementedError:
        continue
      assert plan.launch == choice
      results[choice] = plan.step(w, 3)
  finally:
    plan.set_launch(default)
  assert 0 in results and 1 in results
  for choice, got in results.items():
    assert torch.equal(torch.view_as_real(got), torch.view_as_real(results[0])), choice
