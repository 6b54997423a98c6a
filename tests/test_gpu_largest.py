"""The largest grid the path supports, 4096 x 4096: one FVM step under the
default launch and under every launch configuration the grid admits (same
bits), and one CN-RK4 step, each against the float32 oracle at the per-step
bar (relative L2 <= 1e-5).  Rows and columns of 4096 points take the wide
transform blocks (the narrow ones hold at most 2048-point rows and columns),
two-column groups in the persistent column pass and 4096-point spectral
column passes.
"""
import numpy as np
import pytest
import torch

from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu

STEP_TOL = 1e-5
TWO_PI = 2 * np.pi
N = 4096


@pytest.fixture(scope='module')
def initial_field():
  from oracle import fvm as ofvm
  from oracle import initial_conditions as oic
  og = ofvm.Grid.make((N, N), domain=((0, TWO_PI), (0, TWO_PI)))
  return og, oic.filtered_velocity_field(3, og, 2.0, 4)


def _to_gpu(v0, grid, dev):
  import jax_cfd_gb300.base as cfd
  bc = cfd.boundaries.periodic_boundary_conditions(2)
  return tuple(cfd.grids.GridVariable(cfd.grids.GridArray(torch.from_numpy(np.ascontiguousarray(a)).to(dev), o, grid), bc)
               for a, o in zip(v0, grid.cell_faces))


def test_fvm_4096_step_every_launch(cuda_device, initial_field):
  import jax_cfd_gb300.base as cfd
  from oracle import fvm as ofvm
  og, v0 = initial_field
  grid = cfd.grids.Grid((N, N), domain=((0, TWO_PI), (0, TWO_PI)))
  dt = ofvm.stable_time_step(2.0, 0.5, 1e-3, og)
  step = cfd.equations.semi_implicit_navier_stokes(
      1.0, 1e-3, dt, grid, forcing=cfd.forcings.simple_turbulence_forcing(grid, 1, 4, -0.1))
  v = _to_gpu(v0, grid, cuda_device)
  plan = step.plan(cuda_device)
  default = plan.launch
  got = [c.data.cpu().numpy() for c in step(v)]
  want = ofvm.semi_implicit_navier_stokes(
      1.0, 1e-3, dt, og, forcing=ofvm.simple_turbulence_forcing(og, 1, 4, -0.1))(v0)
  for name, g, w in zip('uv', got, want):
    err = rel_l2(g, w)
    print(f'FVM 4096^2 {name}: launch {default} {plan.describe_launch(default)}, vs float32 oracle {err:.3e}')
    assert err <= STEP_TOL
  ref = [torch.from_numpy(g).to(cuda_device) for g in got]
  ran = 0
  try:
    for choice in range(plan.LAUNCH_CHOICES):
      try:
        plan.set_launch(choice)
      except NotImplementedError:
        continue
      out = step(v)
      assert torch.equal(out[0].data, ref[0]) and torch.equal(out[1].data, ref[1]), choice
      ran += 1
  finally:
    plan.set_launch(default)
  print(f'FVM 4096^2: {ran} launch configurations, all bit-identical')
  assert ran >= 8


def test_spectral_4096_cn_rk4_step(cuda_device, initial_field):
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
  err = rel_l2(got, want)
  print(f'spectral 4096^2: gpu vs float32 oracle {err:.3e}')
  assert np.isfinite(got).all()
  assert err <= STEP_TOL
