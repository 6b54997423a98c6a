"""funcutils.trajectory (funcutils.py:95-126) on the GPU against the oracle.

``trajectory(repeated(step, inner), outer, post_process)`` stacks one
post-processed frame per chunk.  For the forward-Euler step with the
identity or ``curl_2d`` as post-processing the whole trajectory is one native
call writing frames into a device buffer; with any other post-processing it
is a host loop of native steps.  Checks: the two give identical bits; every
frame matches the oracle's ``trajectory`` within the per-step bound times
the steps taken (the float32 rounding differences of the two sides add up
step by step); ``start_with_input`` shifts the frames by one chunk.
"""
import numpy as np
import pytest
import torch

from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu

STEP_TOL = 1e-5
TWO_PI = 2 * np.pi


def _setup(shape, dev, seed=2):
  import jax_cfd_gb300.base as cfd
  from oracle import fvm as ofvm
  from oracle import initial_conditions as oic
  dom = ((0, TWO_PI), (0, TWO_PI))
  og = ofvm.Grid.make(shape, domain=dom)
  v0 = oic.filtered_velocity_field(seed, og, 2.0, 4)
  grid = cfd.grids.Grid(shape, domain=dom)
  dt = ofvm.stable_time_step(2.0, 0.5, 1e-3, og)
  step = cfd.equations.semi_implicit_navier_stokes(
      1.0, 1e-3, dt, grid, forcing=cfd.forcings.simple_turbulence_forcing(grid, 1, 4, -0.1))
  ref = ofvm.semi_implicit_navier_stokes(
      1.0, 1e-3, dt, og, forcing=ofvm.simple_turbulence_forcing(og, 1, 4, -0.1))
  bc = cfd.boundaries.periodic_boundary_conditions(2)
  v = tuple(cfd.grids.GridVariable(cfd.grids.GridArray(torch.from_numpy(a).to(dev), o, grid), bc)
            for a, o in zip(v0, grid.cell_faces))
  return og, v0, step, ref, v


@pytest.mark.parametrize('shape', [(64, 64), (128, 256)])
def test_vorticity_frames_match_oracle_and_host_loop(cuda_device, shape):
  import jax_cfd_gb300.base as cfd
  from oracle import fvm as ofvm
  inner, outer = 10, 6
  og, v0, step, ref, v = _setup(shape, cuda_device)
  run = cfd.funcutils.trajectory(cfd.funcutils.repeated(step, inner), outer,
                                 post_process=cfd.finite_differences.curl_2d)
  final, frames = run(v)
  loop_final, loop_frames = cfd.funcutils.trajectory(
      cfd.funcutils.repeated(step, inner), outer,
      post_process=lambda x: cfd.finite_differences.curl_2d(x))(v)
  assert frames.data.shape == (outer,) + shape and frames.offset == (1.0, 1.0)
  assert torch.equal(frames.data, loop_frames.data)
  for a, b in zip(final, loop_final):
    assert torch.equal(a.data, b.data)
  ref_final, ref_frames = ofvm.trajectory(
      ofvm.repeated(ref, inner), outer, post_process=lambda x: ofvm.curl_2d(x, og.step))(v0)
  got = frames.data.cpu().numpy()
  for k in range(outer):
    assert rel_l2(got[k], ref_frames[k]) <= (k + 1) * inner * STEP_TOL, k
  for a, b in zip(final, ref_final):
    assert rel_l2(a.data.cpu().numpy(), b) <= outer * inner * STEP_TOL


@pytest.mark.parametrize('start_with_input', [False, True])
def test_velocity_frames_match_oracle(cuda_device, start_with_input):
  import jax_cfd_gb300.base as cfd
  from oracle import fvm as ofvm
  inner, outer = 7, 4
  og, v0, step, ref, v = _setup((64, 128), cuda_device, seed=3)
  final, frames = cfd.funcutils.trajectory(cfd.funcutils.repeated(step, inner), outer,
                                           start_with_input=start_with_input)(v)
  assert isinstance(frames, tuple) and frames[0].data.shape == (outer, 64, 128)
  assert frames[0].offset == v[0].offset and frames[1].offset == v[1].offset
  _, ref_frames = ofvm.trajectory(ofvm.repeated(ref, inner), outer,
                                  start_with_input=start_with_input)(v0)
  for c in range(2):
    got = frames[c].data.cpu().numpy()
    for k in range(outer):
      taken = (k if start_with_input else k + 1) * inner
      assert rel_l2(got[k], ref_frames[c][k]) <= max(taken, 1) * STEP_TOL, (c, k)
  if start_with_input:
    assert np.array_equal(frames[0].data[0].cpu().numpy(), v0[0])
  # One-step trajectory (no repeated): frames are the states after each step.
  _, single = cfd.funcutils.trajectory(step, 3)(v)
  state = v
  for k in range(3):
    state = step(state)
    assert torch.equal(single[0].data[k], state[0].data)
