"""Host-side logic of the serving layer (CPU only): the request stream and
the dt policy."""
import math

import numpy as np


def test_poisson_stream_rate_mix_and_determinism():
  from jax_cfd_gb300 import serving
  a = serving.poisson_requests(200.0, 20.0, seed=1)
  b = serving.poisson_requests(200.0, 20.0, seed=1)
  assert [(r.kind, r.n, r.steps, r.arrival) for r in a] == [(r.kind, r.n, r.steps, r.arrival) for r in b]
  assert abs(len(a) - 4000) < 4 * math.sqrt(4000)
  arr = np.array([r.arrival for r in a])
  assert np.all(np.diff(arr) > 0) and arr[-1] < 20.0
  frac_fvm = np.mean([r.kind == 'fvm' for r in a])
  assert abs(frac_fvm - 0.5) < 0.03
  steps = np.array([r.steps for r in a])
  assert steps.min() >= 100 and steps.max() <= 5000
  # log-uniform horizon: the median is near sqrt(100 * 5000)
  assert abs(np.median(steps) - math.sqrt(100 * 5000)) < 80
  w = serving.size_weights()
  cells = np.array(serving.SIZES, dtype=float) ** 2
  np.testing.assert_allclose(w * cells, (w * cells)[0])
  assert {r.k for r in a} == {2, 4, 8}
  nu = np.array([r.viscosity for r in a])
  assert nu.min() >= 1e-4 and nu.max() <= 1e-2


def test_dt_policy_matches_reference_where_it_accepts():
  from jax_cfd_gb300 import serving
  from jax_cfd_gb300.base import equations, grids
  for n, nu, vmax in ((64, 1e-3, 2.0), (256, 1e-4, 3.5), (1024, 1e-2, 1.0)):
    r = serving.Request(rid=0, kind='fvm', n=n, steps=1, viscosity=nu, k=4, vmax=vmax, seed=0)
    grid = grids.Grid((n, n), domain=((0, 2 * np.pi), (0, 2 * np.pi)))
    try:
      want = equations.stable_time_step(vmax, 0.5, nu, grid)
      assert abs(r.dt - want) <= 1e-12 * want
    except ValueError:
      h = 2 * np.pi / n
      assert r.dt == h * h / (4 * nu)
    s = serving.Request(rid=0, kind='spectral', n=n, steps=1, viscosity=nu, k=4, vmax=vmax, seed=0)
    assert s.dt == 0.5 * (2 * np.pi / n) / vmax


def test_pool_capacity_and_slot_bytes():
  from jax_cfd_gb300 import serving
  assert serving.default_capacity('fvm', 64) == 16
  assert serving.default_capacity('spectral', 2048) == 2
  assert serving.Server.slot_bytes('fvm', 64) == 7 * 64 * 64 * 4 + 8 * 64
  assert serving.Server.slot_bytes('spectral', 64) == 7 * 64 * 33 * 8


def test_health_records_decode_and_failure_policy():
  from jax_cfd_gb300 import batching, serving
  raw = np.array([[0, np.float32(1.5).view(np.int32)], [1, 0],
                  [0, np.float32(300.0).view(np.int32)]], dtype=np.int32)
  rec = batching.decode_health(raw)
  assert list(rec['flags']) == [0, 1, 0]
  assert rec['max_abs'][0] == np.float32(1.5) and rec['max_abs'][2] == np.float32(300.0)
  server = serving.Server.__new__(serving.Server)
  server.max_speed_factor = 100.0
  fvm = serving.Request(rid=0, kind='fvm', n=64, steps=1, viscosity=1e-3, k=4, vmax=2.0, seed=0)
  spec = serving.Request(rid=1, kind='spectral', n=64, steps=1, viscosity=1e-3, k=4, vmax=2.0,
                         seed=0)
  assert server._unhealthy(fvm, rec[0]) is None
  assert server._unhealthy(fvm, rec[1])[0] == 'nonfinite'
  assert server._unhealthy(fvm, rec[2])[0] == 'diverged'
  assert server._unhealthy(spec, rec[2]) is None  # spectral magnitudes are not speeds
  assert server._unhealthy(spec, rec[1])[0] == 'nonfinite'
  fvm.dt_override = 0.25
  assert fvm.dt == 0.25
