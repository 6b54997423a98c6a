"""The allocation-free projection entry point agrees with the plan-based one.

``cfd_fvm_projection_noalloc`` serves callers that cannot call cudaMalloc
(graph capture into a pool they do not own, allocators that forbid allocation
after start-up, plugin hosts that pass only pre-allocated buffers).  It keeps
its scratch in a fixed device array of at most 512 x 512 cells.  This test
calls it through the C ABI twice in a row, on different grids and data, and
compares each result with ``cfd_fvm_projection`` (a plan with its own
workspace) and with the oracle's projection, within the per-step tolerance
the other parity tests use, and checks the projected field's divergence.  The
shapes cover every row-transform path the array serves: the shared-memory
Stockham rows, the one-warp 1024-point rows (ny = 2048) and very elongated
grids.  The file name sorts last so that a run stopping at the first failure
has already run every other test.
"""
import ctypes

import numpy as np
import pytest
import torch

from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _noalloc_projection(u, v, hx, hy):
  from jax_cfd_gb300 import _native, plans
  uo, vo = torch.empty_like(u), torch.empty_like(v)
  nx, ny = u.shape
  rc = _native.load().cfd_fvm_projection_noalloc(
      plans.current_stream_ptr(u.device), nx, ny, ctypes.c_double(hx), ctypes.c_double(hy),
      u.data_ptr(), v.data_ptr(), uo.data_ptr(), vo.data_ptr())
  _native.check(rc, 'cfd_fvm_projection_noalloc')
  return uo, vo


def _divergence(u, v, h):
  """Backward-difference divergence (finite_differences.py:136-143)."""
  return (u - np.roll(u, 1, axis=0)) / h + (v - np.roll(v, 1, axis=1)) / h


@pytest.mark.parametrize('calls', [((128, 256), 0.05, 11), ((512, 512), 0.1, 12),
                                   ((128, 2048), 0.1, 13), ((2048, 128), 0.1, 14),
                                   ((4096, 64), 0.1, 15)])
def test_noalloc_projection_two_calls_match_plan(cuda_device, calls):
  from jax_cfd_gb300 import plans
  from oracle import fvm as ofvm
  # Two calls in a row on one device: the second call reuses the array the
  # first one left behind (a different grid, so every table is rewritten).
  cases = [((64, 64), 0.2, 1), calls]
  for shape, h, seed in cases:
    rng = np.random.default_rng(seed)
    u0 = (1 + 0.3 * rng.standard_normal(shape)).astype(np.float32)
    v0 = (1 + 0.3 * rng.standard_normal(shape)).astype(np.float32)
    u = torch.from_numpy(u0).to(cuda_device)
    v = torch.from_numpy(v0).to(cuda_device)
    got = _noalloc_projection(u, v, h, h)
    want = plans.FvmPlan(shape, (h, h), device=cuda_device).projection(u, v)
    torch.cuda.synchronize(cuda_device)
    oracle = ofvm.projection((u0, v0), ofvm.Grid.make(shape, step=(h, h)))
    got_np = [g.cpu().numpy() for g in got]
    for g, w, o in zip(got_np, want, oracle):
      assert rel_l2(g, w.cpu().numpy()) <= TOL
      assert rel_l2(g, o) <= TOL
    # pressure_test.py:91-111 holds the projected field's divergence to 1e-4.
    assert np.abs(_divergence(got_np[0], got_np[1], h)).max() <= 1e-4


def test_noalloc_projection_rejects_oversize_grid(cuda_device):
  u = torch.zeros((1024, 512), dtype=torch.float32, device=cuda_device)
  with pytest.raises(ValueError, match='static scratch limit'):
    _noalloc_projection(u, u.clone(), 0.1, 0.1)
