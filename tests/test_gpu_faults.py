"""Failure detection on the GPU without a fault, a trap or a hang.

Kernels that wait on asynchronous copies bound every wait (bulk.cuh): when a
wait runs out, the kernel records a code in the device fault word, skips its
work and returns, leaving the context usable.  The self-test entry point
makes such a wait run out on purpose -- its mbarrier never completes because
nothing is copied and nothing arrives -- with a short poll limit, and the
checks are: the C call returns CFD_ERR_DEVICE_FAULT, ``cfd_device_fault``
reports code 1 (bulk-copy wait) and clears, and a step launched afterwards
still matches the oracle.  The reference's own failure checks are NaN checks
(spectral/equations_test.py:137,166,233); those are the health flags' tests.
"""
import ctypes

import numpy as np
import pytest
import torch

from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu


def test_bounded_wait_gives_up_reports_and_leaves_context_usable(cuda_device):
  import jax_cfd_gb300.base as cfd
  from jax_cfd_gb300 import _native, plans
  from oracle import fvm as ofvm
  from oracle import initial_conditions as oic
  lib = _native.load()
  assert _native.device_fault(clear=True) in (0, 1)
  assert _native.device_fault() == 0
  rc = lib.cfd_bounded_wait_selftest(ctypes.c_void_p(plans.current_stream_ptr(cuda_device)), 1000)
  assert rc == _native.CFD_ERR_DEVICE_FAULT
  assert 'bounded wait ran out' in _native.last_error()
  with pytest.raises(_native.DeviceFaultError):
    _native.check(rc, 'cfd_bounded_wait_selftest')
  assert _native.device_fault() == 1
  assert _native.device_fault(clear=True) == 1
  assert _native.device_fault() == 0

  # The context still runs work correctly after the give-up.
  shape = (64, 64)
  dom = ((0, 2 * np.pi), (0, 2 * np.pi))
  og = ofvm.Grid.make(shape, domain=dom)
  v0 = oic.filtered_velocity_field(0, og, 2.0, 4)
  grid = cfd.grids.Grid(shape, domain=dom)
  dt = ofvm.stable_time_step(2.0, 0.5, 1e-3, og)
  step = cfd.equations.semi_implicit_navier_stokes(
      1.0, 1e-3, dt, grid, forcing=cfd.forcings.simple_turbulence_forcing(grid, 1, 4, -0.1))
  bc = cfd.boundaries.periodic_boundary_conditions(2)
  v = tuple(cfd.grids.GridVariable(cfd.grids.GridArray(torch.from_numpy(a).to(cuda_device), o, grid), bc)
            for a, o in zip(v0, grid.cell_faces))
  got = [c.data.cpu().numpy() for c in step(v)]
  want = ofvm.semi_implicit_navier_stokes(
      1.0, 1e-3, dt, og, forcing=ofvm.simple_turbulence_forcing(og, 1, 4, -0.1))(v0)
  for g, w in zip(got, want):
    assert rel_l2(g, w) <= 1e-5
  assert _native.device_fault() == 0
