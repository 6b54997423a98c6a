"""Parity at the two headline sizes: one 2048^2 step of each method.

* FVM: ``semi_implicit_navier_stokes`` (Van Leer, explicit diffusion,
  ``simple_turbulence_forcing(1, 4, -0.1)``, ``solve_fast_diag``,
  ``forward_euler``; equations.py:120-151) at 2048 x 2048, float32, from the
  seeded filtered initial field with max speed 2 and dt =
  ``stable_time_step(2, 0.5, 1e-3)``, under the default launch and under the
  launch the autotuner picks.
* Spectral: ``crank_nicolson_rk4(ForcedNavierStokes2D(1e-3, smooth=True),
  1e-3)`` (spectral/time_stepping.py:186-197) at 2048^2 from
  ``rfftn(curl_2d(v0))``.

Each step is compared with the float32 oracle (per-step relative L2 <= 1e-5,
the parity bar) and, as the stand-in for a ``jax_enable_x64`` run of the
reference, both the GPU result and the float32 oracle are compared with the
float64 oracle; the two errors are printed and the GPU's is held to the same
1e-5 bar (measured: both about 5e-8 for FVM).  The FVM step's projected field
must have divergence at float32 round-off (the bound is in the test).
"""
import numpy as np
import pytest
import torch

from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu

STEP_TOL = 1e-5
TWO_PI = 2 * np.pi
N = 2048


@pytest.fixture(scope='module')
def initial_field():
  from oracle import fvm as ofvm
  from oracle import initial_conditions as oic
  og = ofvm.Grid.make((N, N), domain=((0, TWO_PI), (0, TWO_PI)))
  return og, oic.filtered_velocity_field(0, og, 2.0, 4)


def _to_gpu(v0, grid, dev):
  import jax_cfd_gb300.base as cfd
  bc = cfd.boundaries.periodic_boundary_conditions(2)
  return tuple(cfd.grids.GridVariable(cfd.grids.GridArray(torch.from_numpy(np.ascontiguousarray(a)).to(dev), o, grid), bc)
               for a, o in zip(v0, grid.cell_faces))


def test_fvm_2048_step_default_and_autotuned_launch(cuda_device, initial_field):
  import jax_cfd_gb300.base as cfd
  from oracle import fvm as ofvm
  og, v0 = initial_field
  grid = cfd.grids.Grid((N, N), domain=((0, TWO_PI), (0, TWO_PI)))
  dt = ofvm.stable_time_step(2.0, 0.5, 1e-3, og)
  step = cfd.equations.semi_implicit_navier_stokes(
      1.0, 1e-3, dt, grid, forcing=cfd.forcings.simple_turbulence_forcing(grid, 1, 4, -0.1))
  v = _to_gpu(v0, grid, cuda_device)
  plan = step.plan(cuda_device)
  default_launch = plan.launch
  got_default = [c.data.cpu().numpy() for c in step(v)]

  want = ofvm.semi_implicit_navier_stokes(
      1.0, 1e-3, dt, og, forcing=ofvm.simple_turbulence_forcing(og, 1, 4, -0.1))(v0)
  want64 = ofvm.semi_implicit_navier_stokes(
      1.0, 1e-3, dt, og,
      forcing=ofvm.simple_turbulence_forcing(og, 1, 4, -0.1, dtype=np.float64))(
          tuple(a.astype(np.float64) for a in v0))

  tuned = plan.autotune(v[0].data, v[1].data, 2)
  got_tuned = [c.data.cpu().numpy() for c in step(v)]
  print(f'FVM 2048^2 launch: default {default_launch} '
        f'{plan.describe_launch(default_launch)}, autotuned {tuned} {plan.describe_launch(tuned)}')
  for name, g, w, w64 in zip('uv', got_default, want, want64):
    err, err64, oracle64 = rel_l2(g, w), rel_l2(g, w64), rel_l2(w, w64)
    print(f'FVM 2048^2 {name}: gpu vs float32 oracle {err:.3e}; vs float64: gpu {err64:.3e}, '
          f'float32 oracle {oracle64:.3e}')
    assert err <= STEP_TOL
    assert err64 <= STEP_TOL
  for g, t, w in zip(got_default, got_tuned, want):
    assert rel_l2(t, w) <= STEP_TOL
    # Every launch choice runs the same arithmetic.
    assert np.array_equal(g, t)
  # Divergence at float32 round-off.  pressure_test.py:91-111 bounds it by
  # 1e-4 at 100^2 (h = 0.1); a backward difference of float32 velocities
  # carries about eps * max|u| / h of rounding, which at h = 2 pi / 2048 is
  # 7.6e-5 per difference, and the float32 oracle itself reaches 1.9e-4.  The
  # bound is four such differences, and at least the reference's 1e-4.
  eps = float(np.finfo(np.float32).eps)
  bound = max(1e-4, 4 * eps * max(np.abs(a).max() for a in want) / og.step[0])
  div_oracle = float(np.abs(ofvm.divergence(want, og.step)).max())
  for got in (got_default, got_tuned):
    div = float(np.abs(ofvm.divergence(got, og.step)).max())
    print(f'FVM 2048^2 max |div|: gpu {div:.3e}, float32 oracle {div_oracle:.3e}, bound {bound:.3e}')
    assert div <= bound


def test_spectral_2048_cn_rk4_step(cuda_device, initial_field):
  import jax_cfd_gb300.base as cfd
  from jax_cfd_gb300.spectral import equations as seq
  from jax_cfd_gb300.spectral import time_stepping as sts
  from oracle import fvm as ofvm
  from oracle import spectral as ospec
  og, v0 = initial_field
  grid = cfd.grids.Grid((N, N), domain=((0, TWO_PI), (0, TWO_PI)))
  w0 = np.fft.rfftn(ofvm.curl_2d(v0, og.step)).astype(np.complex64)
  eq = seq.ForcedNavierStokes2D(1e-3, grid, smooth=True)
  got = sts.crank_nicolson_rk4(eq, 1e-3)(torch.from_numpy(w0).to(cuda_device)).cpu().numpy()
  want = ospec.crank_nicolson_rk4(ospec.forced_navier_stokes_2d(1e-3, og), 1e-3)(w0)
  want64 = ospec.crank_nicolson_rk4(
      ospec.forced_navier_stokes_2d(1e-3, og, dtype=np.float64), 1e-3)(w0.astype(np.complex128))
  err, err64, oracle64 = rel_l2(got, want), rel_l2(got, want64), rel_l2(want, want64)
  print(f'spectral 2048^2: gpu vs float32 oracle {err:.3e}; vs float64: gpu {err64:.3e}, '
        f'float32 oracle {oracle64:.3e}')
  assert np.isfinite(got).all()
  assert err <= STEP_TOL
  assert err64 <= STEP_TOL
