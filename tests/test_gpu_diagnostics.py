"""On-device diagnostics against the oracle, and the long-horizon statistics.

Long horizons: chaotic trajectories of different precisions separate after
about a thousand steps, so the GPU run is compared through time-averaged
statistics with tests/golden/long_horizon_64.npz (made by
tests/golden/make_long_horizon.py from the oracle's float32 run, the
reference's own precision, and its float64 run, the jax_enable_x64 stand-in):
the mean enstrophy and the isotropic energy spectrum, sampled every 100 steps
from step 2000 to step 20000, per seed, then averaged over the seeds (64 FVM
flows, 16 spectral ones; single-seed statistics scatter by several per cent).
The spectrum is compared as an energy-weighted relative L1 distance over all
shells.  The bar: within 2 % of the float32 oracle, and an error against
float64 no larger than 2 % or 1.5 times the float32 oracle's own, whichever is
larger.  Both implementations' errors against float64 are printed.
"""
import os

import numpy as np
import pytest
import torch

from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu

TWO_PI = 2 * np.pi
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden', 'long_horizon_64.npz')


def _weighted_l1(a, b):
  return float(np.abs(a - b).sum() / np.abs(b).sum())


@pytest.mark.parametrize('n', [32, 64, 256])
def test_diagnostics_match_oracle(cuda_device, n):
  import jax_cfd_gb300.base as cfd
  from jax_cfd_gb300 import diagnostics
  from oracle import diagnostics as od
  from oracle import fvm as ofvm
  from oracle import initial_conditions as oic
  og = ofvm.Grid.make((n, n), domain=((0, TWO_PI), (0, TWO_PI)))
  u, v = oic.filtered_velocity_field(n, og, 2.0, 4)
  grid = cfd.grids.Grid((n, n), domain=((0, TWO_PI), (0, TWO_PI)))
  ud, vd = (torch.from_numpy(a).to(cuda_device) for a in (u, v))
  labels, spec = diagnostics.isotropic_energy_spectrum(ud, vd, grid)
  want_labels, want = od.isotropic_energy_spectrum(u, v, og.step)
  np.testing.assert_allclose(labels, want_labels, rtol=0, atol=0)
  assert rel_l2(spec.cpu().numpy(), want) <= 1e-5
  ens = diagnostics.enstrophy(ud, vd, grid)
  want_ens = float(od.enstrophy_2d(u.astype(np.float64), v.astype(np.float64), og.step).mean())
  assert abs(ens - want_ens) <= 1e-5 * want_ens
  w = diagnostics.vorticity_2d(ud, vd, grid).cpu().numpy()
  assert rel_l2(w, od.vorticity_2d(u, v, og.step)) <= 1e-6


def test_single_mode_spectrum_lands_in_its_shell(cuda_device):
  import jax_cfd_gb300.base as cfd
  from jax_cfd_gb300 import diagnostics
  n = 64
  grid = cfd.grids.Grid((n, n), domain=((0, TWO_PI), (0, TWO_PI)))
  x, y = grid.mesh_numpy(grid.cell_faces[0])
  u = np.cos(3 * x).astype(np.float32)       # |k| = 3
  v = np.sin(4 * y + 2 * x).astype(np.float32)  # |k| = sqrt(20), shell 4
  labels, spec = diagnostics.isotropic_energy_spectrum(
      torch.from_numpy(u).to(cuda_device), torch.from_numpy(v).to(cuda_device), grid)
  spec = spec.cpu().numpy()
  # |fft2(cos)|^2: two peaks of (n^2 / 2)^2; energy 0.5 * that per component
  one = 0.5 * 2 * (n * n / 2) ** 2
  np.testing.assert_allclose(spec[2], one, rtol=1e-5)
  np.testing.assert_allclose(spec[3], one, rtol=1e-5)
  assert np.abs(np.delete(spec, [2, 3])).max() <= 1e-6 * one


def _gpu_fvm_statistics(dev, golden):
  """Per-seed time-averaged (spectrum, enstrophy) of the FVM flows."""
  import jax_cfd_gb300.base as cfd
  from jax_cfd_gb300 import diagnostics
  from oracle import fvm as ofvm
  from oracle import initial_conditions as oic
  n, steps, burn, every = (int(x) for x in golden['config'])
  og = ofvm.Grid.make((n, n), domain=((0, TWO_PI), (0, TWO_PI)))
  grid = cfd.grids.Grid((n, n), domain=((0, TWO_PI), (0, TWO_PI)))
  dt = cfd.equations.stable_time_step(float(golden['fvm_dt_speed']), 0.5, 1e-3, grid)
  step = cfd.equations.semi_implicit_navier_stokes(
      1.0, 1e-3, dt, grid, forcing=cfd.forcings.simple_turbulence_forcing(grid, 1, 4, -0.1))
  bc = cfd.boundaries.periodic_boundary_conditions(2)
  specs, enss = [], []
  for seed in golden['fvm_seeds']:
    v0 = oic.filtered_velocity_field(int(seed), og, 2.0, 4)
    v = tuple(cfd.grids.GridVariable(cfd.grids.GridArray(torch.from_numpy(a).to(dev), o, grid), bc)
              for a, o in zip(v0, grid.cell_faces))
    v = cfd.funcutils.repeated(step, burn)(v)
    ens, spec, count = 0.0, 0.0, 0
    for _ in range((steps - burn) // every):
      v = cfd.funcutils.repeated(step, every)(v)
      ens += diagnostics.enstrophy(v[0].data, v[1].data, grid)
      spec = spec + diagnostics.isotropic_energy_spectrum(v[0].data, v[1].data, grid)[1]
      count += 1
    specs.append((spec / count).cpu().numpy())
    enss.append(ens / count)
  return np.array(specs), np.array(enss)


def _gpu_spectral_statistics(dev, golden):
  """Per-seed time-averaged (spectrum, enstrophy) of the spectral flows."""
  import jax_cfd_gb300.base as cfd
  from jax_cfd_gb300 import diagnostics
  from jax_cfd_gb300.spectral import equations as seq
  from jax_cfd_gb300.spectral import time_stepping as sts
  from jax_cfd_gb300.spectral import utils as su
  from oracle import fvm as ofvm
  from oracle import initial_conditions as oic
  n, steps, burn, every = (int(x) for x in golden['config'])
  og = ofvm.Grid.make((n, n), domain=((0, TWO_PI), (0, TWO_PI)))
  grid = cfd.grids.Grid((n, n), domain=((0, TWO_PI), (0, TWO_PI)))
  step = sts.crank_nicolson_rk4(seq.ForcedNavierStokes2D(1e-3, grid, smooth=True), 1e-3)
  to_velocity = su.vorticity_to_velocity(grid)
  specs, enss = [], []
  for seed in golden['spectral_seeds']:
    v0 = oic.filtered_velocity_field(int(seed), og, 2.0, 4)
    w = su.rfft2(torch.from_numpy(ofvm.curl_2d(v0, og.step)).to(dev), grid)
    w = cfd.funcutils.repeated(step, burn)(w)
    ens, spec, count = 0.0, 0.0, 0
    for _ in range((steps - burn) // every):
      w = cfd.funcutils.repeated(step, every)(w)
      vx, vy = (su.irfft2(a.to(torch.complex64), grid) for a in to_velocity(w))
      vort = su.irfft2(w, grid).double()
      ens += float((vort ** 2 / 2).mean())
      spec = spec + diagnostics.isotropic_energy_spectrum(vx, vy, grid)[1]
      count += 1
    specs.append((spec / count).cpu().numpy())
    enss.append(ens / count)
  return np.array(specs), np.array(enss)


@pytest.mark.parametrize('kind', ['fvm', 'spectral'])
def test_long_horizon_statistics_match_float64(cuda_device, kind):
  golden = np.load(GOLDEN)
  if kind == 'fvm':
    specs, enss = _gpu_fvm_statistics(cuda_device, golden)
  else:
    specs, enss = _gpu_spectral_statistics(cuda_device, golden)
  spec, ens = specs.mean(0), float(enss.mean())
  s64, s32 = golden[kind + '_spectrum_64'].mean(0), golden[kind + '_spectrum_32'].mean(0)
  e64, e32 = float(golden[kind + '_enstrophy_64'].mean()), float(golden[kind + '_enstrophy_32'].mean())
  err = {'gpu': (_weighted_l1(spec, s64), abs(ens - e64) / e64),
         'oracle_f32': (_weighted_l1(s32, s64), abs(e32 - e64) / e64)}
  vs_f32 = (_weighted_l1(spec, s32), abs(ens - e32) / e32)
  print(kind, 'spectrum / enstrophy error vs float64:', err, 'gpu vs float32 oracle:', vs_f32)
  assert vs_f32[0] <= 0.02 and vs_f32[1] <= 0.02
  assert err['gpu'][0] <= max(0.02, 1.5 * err['oracle_f32'][0])
  assert err['gpu'][1] <= max(0.02, 1.5 * err['oracle_f32'][1])
