"""Per-trajectory health flags of batches, ensembles and the server.

The reference's failure checks are NaN checks on the state
(spectral/equations_test.py:137,166,233).  Here every batched chunk ends with
a per-slot reduction on the device (cfd_health: a non-finite flag and the
largest finite magnitude).  Faults are injected from the host: a NaN written
into one member's state, or a request given a time step far beyond the
stable one.  The checks: the poisoned member is flagged, the others are not,
their records match their states, and their results are bit-identical to a
run without the poisoned member.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

TWO_PI = 2 * np.pi


def _member(shape, seed, nu, k, vmax):
  from jax_cfd_gb300 import batching
  from jax_cfd_gb300.base import equations, grids
  from oracle import fvm as ofvm
  from oracle import initial_conditions as oic
  og = ofvm.Grid.make(shape, domain=((0, TWO_PI), (0, TWO_PI)))
  v0 = oic.filtered_velocity_field(seed, og, vmax, 4)
  grid = grids.Grid(shape, domain=((0, TWO_PI), (0, TWO_PI)))
  dt = equations.stable_time_step(vmax, 0.5, nu, grid)
  return batching.kolmogorov_member(shape, nu, dt, k), v0


def _fvm_batch(pairs, dev, poison=None):
  from jax_cfd_gb300 import batching
  m0 = pairs[0][0]
  b = batching.FvmBatch(m0['shape'], m0['step'], len(pairs), device=dev)
  for i, (m, v0) in enumerate(pairs):
    kw = dict(m)
    kw.pop('shape'), kw.pop('step')
    b.set_slot(i, **kw)
    u = np.array(v0[0], copy=True)
    if i == poison:
      u[3, 5] = np.nan
    b.set_state(i, torch.from_numpy(u).to(dev), torch.from_numpy(np.ascontiguousarray(v0[1])).to(dev))
    b.set_steps(i, 6)
  return b


@pytest.mark.parametrize('graph', [False, True])
def test_fvm_batch_flags_the_poisoned_slot_only(cuda_device, graph):
  from jax_cfd_gb300 import _native as nat
  shape = (64, 64)
  pairs = [_member(shape, 31 + i, 1e-3, 4, 2.0) for i in range(3)]
  clean = _fvm_batch(pairs, cuda_device)
  clean.run(6, graph=graph)
  poisoned = _fvm_batch(pairs, cuda_device, poison=1)
  # The pinned-host mirror receives the same records from the device.
  mirror = torch.full((3, 2), -1, dtype=torch.int32, pin_memory=True)
  poisoned.set_health_mirror(mirror)
  poisoned.run(6, graph=graph)
  torch.cuda.synchronize(cuda_device)
  hc, hp = clean.health(), poisoned.health()
  assert np.array_equal(mirror.numpy(), poisoned.health_device().cpu().numpy())
  assert (hc['flags'] == 0).all()
  assert hp['flags'][1] & nat.HEALTH_NONFINITE
  assert hp['flags'][0] == 0 and hp['flags'][2] == 0
  for i in (0, 2):
    for a, b in zip(clean.state(i), poisoned.state(i)):
      assert torch.equal(a, b)
    u, v = poisoned.state(i)
    assert hp['max_abs'][i] == max(float(u.abs().max()), float(v.abs().max()))
  assert not torch.isfinite(poisoned.state(1)[0]).all()


def test_spectral_batch_flags_the_poisoned_slot_only(cuda_device):
  from jax_cfd_gb300 import _native as nat
  from jax_cfd_gb300 import batching
  from jax_cfd_gb300.base import grids
  from jax_cfd_gb300.spectral import equations as seq
  from jax_cfd_gb300.spectral import time_stepping as sts
  from oracle import fvm as ofvm
  from oracle import initial_conditions as oic
  shape = (64, 64)
  grid = grids.Grid(shape, domain=((0, TWO_PI), (0, TWO_PI)))
  og = ofvm.Grid.make(shape, domain=((0, TWO_PI), (0, TWO_PI)))
  step = sts.crank_nicolson_rk4(seq.ForcedNavierStokes2D(1e-3, grid, smooth=True), 1e-3)
  w0 = [np.fft.rfftn(ofvm.curl_2d(oic.filtered_velocity_field(41 + i, og, 2.0, 4), og.step))
        .astype(np.complex64) for i in range(3)]

  def run(poison):
    b = batching.SpecBatch(shape, grid.step, 3, device=cuda_device)
    for i in range(3):
      b.set_slot_from_step(i, step)
      w = w0[i].copy()
      if i == poison:
        w[2, 3] = np.nan
      b.set_state(i, torch.from_numpy(w).to(cuda_device))
      b.set_steps(i, 4)
    b.run(4)
    torch.cuda.synchronize(cuda_device)
    return b

  clean, poisoned = run(None), run(2)
  assert (clean.health()['flags'] == 0).all()
  h = poisoned.health()
  assert h['flags'][2] & nat.HEALTH_NONFINITE and h['flags'][0] == 0 and h['flags'][1] == 0
  for i in (0, 1):
    assert torch.equal(clean.state(i), poisoned.state(i))
    assert h['max_abs'][i] == float(torch.view_as_real(poisoned.state(i)).abs().max())


def test_ensemble_health_per_member(cuda_device):
  from jax_cfd_gb300 import batching
  draws = [((64, 64), 51, 1e-3, 4, 2.0), ((128, 128), 52, 1e-3, 2, 2.0),
           ((64, 64), 53, 1e-3, 8, 3.0)]
  pairs = [_member(*d) for d in draws]

  def run(poison):
    ens = batching.FvmEnsemble([m for m, _ in pairs], device=cuda_device)
    for i, (_, v0) in enumerate(pairs):
      u = np.array(v0[0], copy=True)
      if i == poison:
        u[0, 0] = np.inf
      ens.set_state(i, torch.from_numpy(u).to(cuda_device),
                    torch.from_numpy(np.ascontiguousarray(v0[1])).to(cuda_device))
    ens.step(5)
    torch.cuda.synchronize(cuda_device)
    return ens

  clean, poisoned = run(None), run(1)
  assert (clean.health()['flags'] == 0).all()
  h = poisoned.health()
  assert list(h['flags'] != 0) == [False, True, False]
  for i in (0, 2):
    for a, b in zip(clean.state(i), poisoned.state(i)):
      assert torch.equal(a, b)


def test_server_retires_a_diverging_request_with_an_error_status(cuda_device):
  from jax_cfd_gb300 import serving

  def reqs():
    out = [serving.Request(rid=i, kind=kind, n=64, steps=150, viscosity=1e-3, k=4, vmax=2.0,
                           seed=60 + i) for i, kind in enumerate(('fvm', 'fvm', 'spectral'))]
    # Fifty times the stable time step: leaves the explicit scheme's
    # stability region within the first chunk.
    out.append(serving.Request(rid=3, kind='fvm', n=64, steps=150, viscosity=1e-3, k=4,
                               vmax=2.0, seed=63))
    out[3].dt_override = 50 * out[3].dt
    return out

  done = serving.Server(device=cuda_device, chunk=50).serve(reqs(), realtime=False, timeout=120)
  by_id = {r.rid: r for r in done}
  assert len(by_id) == 4
  bad = by_id[3]
  assert bad.status in ('nonfinite', 'diverged') and bad.result is None and bad.error
  assert bad.finished is not None
  for rid in (0, 1, 2):
    assert by_id[rid].status == 'ok'
    assert all(np.isfinite(a).all() for a in by_id[rid].result)
  # The others' results do not depend on the failed request.
  clean = [r for r in reqs() if r.rid != 3]
  alone = {r.rid: r for r in serving.Server(device=cuda_device, chunk=50).serve(
      clean, realtime=False, timeout=120)}
  for rid in (0, 1, 2):
    for a, b in zip(alone[rid].result, by_id[rid].result):
      assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
  st = serving.Server.stats(done, 1.0)
  assert st['completed_ok'] == 3 and st['nonfinite'] + st['diverged'] == 1
