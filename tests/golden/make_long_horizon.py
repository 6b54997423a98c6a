"""Generates tests/golden/long_horizon_64.npz: long-horizon flow statistics of
the oracle (float32 and float64 runs) for the long-horizon check.

Chaotic trajectories of different precisions separate after about a
thousand steps, so the check compares statistics, not states: the energy
spectrum (binsum isotropization) and the mean enstrophy, averaged every
SAMPLE_EVERY steps after BURN_IN steps up to STEPS steps, per seed, for 64^2
Kolmogorov flows.  Single-seed statistics scatter by several per cent between
seeds (long-lived large-scale states), so the check averages over many seeds:
FVM_SEEDS for the FVM flow, SPECTRAL_SEEDS for the spectral one.

* FVM: semi_implicit_navier_stokes, nu = 1e-3, simple_turbulence_forcing(1,
  4, -0.1), initial max speed 2, dt = stable_time_step(4, 0.5, nu): half the
  500-step case's dt, because that one's flow occasionally exceeds twice its
  initial speed over tens of thousands of steps and leaves the explicit
  scheme's stability region;
* spectral: ForcedNavierStokes2D(1e-3, smooth=True) with crank_nicolson_rk4,
  dt = 1e-3, from rfft2(curl_2d(v0)).

Run from the repository root:  python tests/golden/make_long_horizon.py
(about ten minutes on eight cores).
"""
import multiprocessing
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import diagnostics as od  # noqa: E402
from oracle import fvm as ofvm  # noqa: E402
from oracle import initial_conditions as oic  # noqa: E402
from oracle import spectral as ospec  # noqa: E402

N = 64
FVM_SEEDS = tuple(range(64))
SPECTRAL_SEEDS = tuple(range(16))
STEPS = 20000
BURN_IN = 2000
SAMPLE_EVERY = 100
FVM_DT_SPEED = 4.0
SPECTRAL_DT = 1e-3


def grid():
  return ofvm.Grid.make((N, N), domain=((0, 2 * np.pi), (0, 2 * np.pi)))


def fvm_statistics(dtype, seed):
  og = grid()
  v0 = oic.filtered_velocity_field(seed, og, 2.0, 4)
  dt = ofvm.stable_time_step(FVM_DT_SPEED, 0.5, 1e-3, og)
  step = ofvm.semi_implicit_navier_stokes(
      1.0, 1e-3, dt, og, forcing=ofvm.simple_turbulence_forcing(og, 1, 4, -0.1),
      diag=ofvm.pinv_diagonal(og, dtype))
  v = tuple(a.astype(dtype) for a in v0)
  ens, spec, count = 0.0, 0.0, 0
  for k in range(1, STEPS + 1):
    v = step(v)
    if k > BURN_IN and k % SAMPLE_EVERY == 0:
      u64, v64 = (a.astype(np.float64) for a in v)
      ens += float(od.enstrophy_2d(u64, v64, og.step).mean())
      spec = spec + od.isotropic_energy_spectrum(u64, v64, og.step)[1]
      count += 1
  return spec / count, ens / count


def spectral_statistics(dtype, seed):
  og = grid()
  v0 = oic.filtered_velocity_field(seed, og, 2.0, 4)
  cdtype = np.complex64 if dtype == np.float32 else np.complex128
  w = np.fft.rfftn(ofvm.curl_2d(v0, og.step)).astype(cdtype)
  eq = ospec.forced_navier_stokes_2d(1e-3, og, smooth=True, dtype=dtype)
  step = ospec.crank_nicolson_rk4(eq, SPECTRAL_DT)
  to_velocity = ospec.vorticity_to_velocity(og, dtype)
  ens, spec, count = 0.0, 0.0, 0
  for k in range(1, STEPS + 1):
    w = step(w)
    if k > BURN_IN and k % SAMPLE_EVERY == 0:
      vx, vy = (np.fft.irfftn(a, s=(N, N), axes=(0, 1)).astype(np.float64)
                for a in to_velocity(w))
      vort = np.fft.irfftn(w, s=(N, N), axes=(0, 1)).astype(np.float64)
      ens += float((vort ** 2 / 2).mean())
      spec = spec + od.isotropic_energy_spectrum(vx, vy, og.step)[1]
      count += 1
  return spec / count, ens / count


def _run(job):
  kind, name, seed = job
  fn = fvm_statistics if kind == 'fvm' else spectral_statistics
  return job, fn(np.float32 if name == '32' else np.float64, seed)


def main():
  jobs = [(kind, name, seed)
          for kind, seeds in (('fvm', FVM_SEEDS), ('spectral', SPECTRAL_SEEDS))
          for name in ('32', '64') for seed in seeds]
  with multiprocessing.get_context('spawn').Pool(os.cpu_count()) as pool:
    results = dict(pool.map(_run, jobs, chunksize=1))
  out = {'labels': od.shell_bins((N, N), grid().step)[1]}
  for kind, seeds in (('fvm', FVM_SEEDS), ('spectral', SPECTRAL_SEEDS)):
    for name in ('32', '64'):
      runs = [results[(kind, name, seed)] for seed in seeds]
      spec = np.array([r[0] for r in runs])
      ens = np.array([r[1] for r in runs])
      if not (np.isfinite(spec).all() and np.isfinite(ens).all()):
        raise RuntimeError(f'{kind} float{name} run left the stability region')
      # per-seed statistics: [seeds, shells] and [seeds]
      out[f'{kind}_spectrum_{name}'] = spec
      out[f'{kind}_enstrophy_{name}'] = ens
      print(kind, name, 'mean enstrophy', ens.mean(), flush=True)
    out[f'{kind}_seeds'] = np.array(seeds)
  out['config'] = np.array([N, STEPS, BURN_IN, SAMPLE_EVERY])
  out['fvm_dt_speed'] = np.array(FVM_DT_SPEED)
  np.savez(os.path.join(os.path.dirname(os.path.abspath(__file__)), 'long_horizon_64.npz'), **out)


if __name__ == '__main__':
  main()
