"""The continuous-batching server: results are independent of the mix, equal
to the drop-in path, and admission respects the memory budget."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _requests(count, seed=5, sizes=(64, 128)):
  from jax_cfd_gb300 import serving
  reqs = serving.poisson_requests(rate=1000.0, duration=count / 1000.0 * 3, seed=seed,
                                  sizes=sizes, min_steps=20, max_steps=250)
  return reqs[:count]


def _fresh(req):
  from jax_cfd_gb300 import serving
  return serving.Request(rid=req.rid, kind=req.kind, n=req.n, steps=req.steps,
                         viscosity=req.viscosity, k=req.k, vmax=req.vmax, seed=req.seed,
                         arrival=0.0)


def _same(a, b):
  return all(np.array_equal(x.view(np.uint32), y.view(np.uint32)) for x, y in zip(a, b))


def test_result_alone_equals_result_in_the_mix(cuda_device):
  from jax_cfd_gb300 import serving
  mix = _requests(40)
  kinds = {r.kind for r in mix}
  assert kinds == {'fvm', 'spectral'}
  done = serving.Server(device=cuda_device, chunk=50).serve(mix, realtime=False, timeout=120)
  assert len(done) == len(mix)
  by_id = {r.rid: r for r in done}
  picks = [next(r for r in mix if r.kind == 'fvm'), next(r for r in mix if r.kind == 'spectral'),
           max(mix, key=lambda r: r.steps)]
  for p in picks:
    alone = serving.Server(device=cuda_device, chunk=50).serve([_fresh(p)], realtime=False,
                                                              timeout=60)
    assert _same(alone[0].result, by_id[p.rid].result), (p.kind, p.n, p.steps)


def test_served_results_equal_the_dropin_path(cuda_device):
  import jax_cfd_gb300.base as cfd
  from jax_cfd_gb300 import serving
  from jax_cfd_gb300.base import forcings
  from jax_cfd_gb300.spectral import equations as seq
  from jax_cfd_gb300.spectral import time_stepping as sts
  from jax_cfd_gb300.spectral import utils as su
  mix = _requests(12, seed=9)
  done = serving.Server(device=cuda_device, chunk=64).serve(mix, realtime=False, timeout=120)
  for r in done:
    grid = cfd.grids.Grid((r.n, r.n), domain=((0, 2 * np.pi), (0, 2 * np.pi)))
    v0 = cfd.initial_conditions.filtered_velocity_field(r.seed, grid, r.vmax, 4,
                                                        device=cuda_device)
    if r.kind == 'fvm':
      step = cfd.equations.semi_implicit_navier_stokes(
          1.0, r.viscosity, r.dt, grid,
          forcing=cfd.forcings.simple_turbulence_forcing(grid, 1, r.k, -0.1))
      want = cfd.funcutils.repeated(step, r.steps)(v0)
      want = tuple(w.data.cpu().numpy() for w in want)
    else:
      eq = seq.NavierStokes2D(r.viscosity, grid, drag=0.1, smooth=True,
                              forcing_fn=lambda g, k=r.k: forcings.kolmogorov_forcing(
                                  g, k=k, offsets=((0, 0), (0, 0))))
      w0 = su.rfft2(cfd.finite_differences.curl_2d(v0).data, grid)
      want = (cfd.funcutils.repeated(sts.crank_nicolson_rk4(eq, r.dt), r.steps)(w0)
              .cpu().numpy(),)
    assert _same(r.result, want), (r.kind, r.n, r.steps)


def test_admission_waits_for_memory_budget(cuda_device):
  from jax_cfd_gb300 import serving
  mix = _requests(16, seed=3, sizes=(64,))
  # Room for one two-slot pool of each kind, not for a second one.
  budget = 2 * (serving.Server.slot_bytes('fvm', 64) + serving.Server.slot_bytes('spectral', 64))
  budget += 64 << 10
  server = serving.Server(device=cuda_device, chunk=40, budget_bytes=budget,
                          capacity=lambda kind, n: 2)
  done = server.serve(mix, realtime=False, timeout=120)
  assert len(done) == len(mix)
  assert server.bytes_in_use <= budget
  assert sum(len(p) for p in server.pools.values()) <= 2
  # realtime=False submits everything at t = 0, so only the order of the
  # server's own timestamps is meaningful here.
  assert all(r.finished >= r.admitted for r in done)
