"""Batched and ragged FVM execution against the single-trajectory path.

The batched kernels run the same per-tile and per-row code as the
single-trajectory kernels, with the member index as a grid axis, so a member's
result must equal the single-trajectory result bit for bit (the single path is
pinned to the oracle in test_gpu_fvm.py; one member is also checked against
the oracle directly here).  "Alone" and "in the mix" must agree bit for bit as
well: no kernel reads another member's buffers.
"""
import numpy as np
import pytest
import torch

from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu

TWO_PI = 2 * np.pi
STEP_TOL = 1e-5


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


def _single(member, v0, steps, dev):
  from jax_cfd_gb300 import plans
  kw = dict(member)
  shape, step = kw.pop('shape'), kw.pop('step')
  plan = plans.FvmPlan(shape, step, device=dev, **kw)
  u = torch.from_numpy(np.ascontiguousarray(v0[0])).to(dev)
  v = torch.from_numpy(np.ascontiguousarray(v0[1])).to(dev)
  return plan.step(u, v, steps)


def _batch(members, dev):
  from jax_cfd_gb300 import batching
  m0 = members[0]
  b = batching.FvmBatch(m0['shape'], m0['step'], len(members), device=dev)
  for i, m in enumerate(members):
    kw = dict(m)
    kw.pop('shape'), kw.pop('step')
    b.set_slot(i, **kw)
  return b


def _load(b, i, v0, dev):
  b.set_state(i, torch.from_numpy(np.ascontiguousarray(v0[0])).to(dev),
              torch.from_numpy(np.ascontiguousarray(v0[1])).to(dev))


@pytest.mark.parametrize('graph', [False, True])
@pytest.mark.parametrize('shape', [(64, 64), (64, 2048), (2048, 64)])
def test_batch_slots_equal_single_trajectories(cuda_device, graph, shape):
  """Rows of 2048 take the one-warp row transforms.  (The third draw's
  diffusion number is only stable on square cells.)"""
  draws = [(shape, 11, 1e-3, 4, 2.0), (shape, 12, 1e-4, 2, 1.0)]
  if shape[0] == shape[1]:
    draws.append((shape, 13, 1e-2, 8, 4.0))
  pairs = [_member(*d) for d in draws]
  b = _batch([m for m, _ in pairs], cuda_device)
  for i, (_, v0) in enumerate(pairs):
    _load(b, i, v0, cuda_device)
    b.set_steps(i, 7)
  b.run(7, graph=graph)
  torch.cuda.synchronize(cuda_device)
  for i, (m, v0) in enumerate(pairs):
    want = _single(m, v0, 7, cuda_device)
    for got, w in zip(b.state(i), want):
      assert torch.isfinite(w).all()
      assert torch.equal(got, w)


@pytest.mark.parametrize('shape', [(256, 256), (1024, 128)])
def test_every_batch_launch_configuration_gives_the_same_bits(cuda_device, shape):
  """Tiles vs warp-streaming stencil, wide vs narrow row blocks, per-block,
  cluster and persistent pipelined column passes (staged by cp.async or by
  TMA tensor loads), rows fed through registers or by bulk copies, over a
  batch with an idle slot: identical results, equal to the single
  trajectories."""
  draws = [(shape, 21, 1e-3, 4, 2.0), (shape, 22, 1e-4, 2, 1.0), (shape, 23, 1e-3, 8, 3.0)]
  pairs = [_member(*d) for d in draws]
  b = _batch([m for m, _ in pairs], cuda_device)
  results = {}
  for choice in range(b.LAUNCH_CHOICES):
    try:
      b.set_launch(choice)
    except NotImplementedError:
      continue
    for i, (_, v0) in enumerate(pairs):
      _load(b, i, v0, cuda_device)
      b.set_steps(i, [5, 0, 3][i])
    b.run(5, graph=choice % 2 == 0)
    torch.cuda.synchronize(cuda_device)
    results[choice] = [tuple(t.clone() for t in b.state(i)) for i in range(len(pairs))]
  # blocks, pipelined, TMA x 2 stencils; the same with bulk-copy row feed
  assert all(c in results for c in (0, 6, 8, 16, 18, 21, 29, 39))
  for i, (m, v0) in enumerate(pairs):
    want = _single(m, v0, [5, 0, 3][i], cuda_device)
    for choice, states in results.items():
      for got, w in zip(states[i], want):
        assert torch.equal(got, w), (choice, i)


@pytest.mark.parametrize('shape', [(64, 64), (128, 64), (64, 128)])
def test_resident_chunk_gives_the_per_step_bits(cuda_device, shape):
  """Launch configuration 20 runs each member's whole chunk in one block with
  the fields in shared memory; with ragged steps and an idle slot it must
  give the per-step launches' bits (and so the single trajectories')."""
  draws = [(shape, 31, 1e-3, 4, 2.0), (shape, 32, 1e-4, 2, 1.0), (shape, 33, 1e-3, 8, 3.0)]
  pairs = [_member(*d) for d in draws]
  b = _batch([m for m, _ in pairs], cuda_device)
  results = {}
  for choice in (0, 20):
    b.set_launch(choice)
    for graph in (False, True):
      for i, (_, v0) in enumerate(pairs):
        _load(b, i, v0, cuda_device)
        b.set_steps(i, [12, 0, 7][i])
      b.run(12, graph=graph)
      torch.cuda.synchronize(cuda_device)
      results[(choice, graph)] = [tuple(t.clone() for t in b.state(i)) for i in range(3)]
  for key, states in results.items():
    for i in range(3):
      for got, want in zip(states[i], results[(0, False)][i]):
        assert torch.equal(got, want), (key, i)
  for i, (m, v0) in enumerate(pairs):
    want = _single(m, v0, [12, 0, 7][i], cuda_device)
    for got, w in zip(results[(20, True)][i], want):
      assert torch.equal(got, w)
  # Health records are written after the resident chunk too.
  h = b.health()
  assert h['flags'][0] == 0 and h['max_abs'][0] > 0


def test_ragged_steps_and_idle_slots(cuda_device):
  draws = [((128, 64), 21, 1e-3, 4, 2.0), ((128, 64), 22, 3e-3, 2, 3.0),
           ((128, 64), 23, 1e-3, 8, 1.5)]
  pairs = [_member(*d) for d in draws]
  b = _batch([m for m, _ in pairs], cuda_device)
  steps = [5, 2, 0]
  for i, (_, v0) in enumerate(pairs):
    _load(b, i, v0, cuda_device)
    b.set_steps(i, steps[i])
  b.run(5)
  torch.cuda.synchronize(cuda_device)
  for i, (m, v0) in enumerate(pairs):
    want = _single(m, v0, steps[i], cuda_device)
    for got, w in zip(b.state(i), want):
      assert torch.equal(got, w)


def test_member_alone_equals_member_in_the_mix(cuda_device):
  draws = [((128, 128), 31, 1e-3, 4, 2.0), ((128, 128), 32, 2e-4, 8, 4.0),
           ((128, 128), 33, 5e-3, 2, 1.0), ((128, 128), 34, 1e-3, 4, 3.0)]
  pairs = [_member(*d) for d in draws]
  mix = _batch([m for m, _ in pairs], cuda_device)
  for i, (_, v0) in enumerate(pairs):
    _load(mix, i, v0, cuda_device)
    mix.set_steps(i, 12)
  mix.run(12)
  alone = _batch([m for m, _ in pairs], cuda_device)
  _load(alone, 1, pairs[1][1], cuda_device)
  alone.set_steps(1, 12)
  alone.run(12)
  torch.cuda.synchronize(cuda_device)
  for a, b in zip(alone.state(1), mix.state(1)):
    assert torch.equal(a, b)


def test_ragged_ensemble_graph_matches_single_and_oracle(cuda_device):
  from jax_cfd_gb300 import batching
  from oracle import fvm as ofvm
  draws = [((64, 64), 41, 1e-3, 4, 2.0), ((256, 256), 42, 1e-4, 2, 1.0),
           ((128, 128), 43, 1e-2, 8, 4.0), ((64, 64), 44, 3e-3, 2, 3.0),
           ((256, 256), 45, 1e-3, 4, 2.5)]
  pairs = [_member(*d) for d in draws]
  ens = batching.FvmEnsemble([m for m, _ in pairs], device=cuda_device)
  assert ens.num_batches == 3
  for i, (_, v0) in enumerate(pairs):
    ens.set_state(i, torch.from_numpy(v0[0]).to(cuda_device),
                  torch.from_numpy(v0[1]).to(cuda_device))
  ens.autotune(2)
  ens.step(4, graph=True)
  ens.step(4, graph=True)  # graph replay
  torch.cuda.synchronize(cuda_device)
  for i, (m, v0) in enumerate(pairs):
    want = _single(m, v0, 8, cuda_device)
    for got, w in zip(ens.state(i), want):
      assert torch.equal(got, w)
  # Member 0 against the oracle (8 steps).
  m, v0 = pairs[0]
  og = ofvm.Grid.make(m['shape'], domain=((0, TWO_PI), (0, TWO_PI)))
  step = ofvm.semi_implicit_navier_stokes(
      1.0, m['viscosity'], m['dt'], og, forcing=ofvm.simple_turbulence_forcing(og, 1, 4, -0.1))
  ref = ofvm.repeated(step, 8)([a.copy() for a in v0])
  for got, w in zip(ens.state(0), ref):
    assert rel_l2(got.cpu().numpy(), w) <= 8 * STEP_TOL


def test_dropin_ensemble_over_step_functions(cuda_device):
  import jax_cfd_gb300.base as cfd
  from jax_cfd_gb300 import batching
  from oracle import fvm as ofvm
  from oracle import initial_conditions as oic
  fns, states = [], []
  for n, seed, k in ((64, 51, 4), (128, 52, 2)):
    grid = cfd.grids.Grid((n, n), domain=((0, TWO_PI), (0, TWO_PI)))
    dt = cfd.equations.stable_time_step(2.0, 0.5, 1e-3, grid)
    fns.append(cfd.equations.semi_implicit_navier_stokes(
        1.0, 1e-3, dt, grid, forcing=cfd.forcings.simple_turbulence_forcing(grid, 1, k, -0.1)))
    og = ofvm.Grid.make((n, n), domain=((0, TWO_PI), (0, TWO_PI)))
    v0 = oic.filtered_velocity_field(seed, og, 2.0, 4)
    bc = cfd.boundaries.periodic_boundary_conditions(2)
    states.append(tuple(cfd.grids.GridVariable(
        cfd.grids.GridArray(torch.from_numpy(a).to(cuda_device), o, grid), bc)
        for a, o in zip(v0, grid.cell_faces)))
  ens = batching.Ensemble(fns, device=cuda_device)
  for i, v in enumerate(states):
    ens.set_velocity(i, v)
  ens.advance(6)
  for i, v in enumerate(states):
    want = cfd.funcutils.repeated(fns[i], 6)(v)
    got = ens.velocity(i)
    for g, w in zip(got, want):
      assert g.offset == w.offset
      assert torch.equal(g.data, w.data)


def test_batch_rejects_mismatched_slot(cuda_device):
  from jax_cfd_gb300 import batching
  m, _ = _member((64, 64), 1, 1e-3, 4, 2.0)
  b = batching.FvmBatch((64, 64), m['step'], 2, device=cuda_device)
  with pytest.raises(ValueError):
    b2 = batching.FvmBatch((128, 128), (TWO_PI / 128, TWO_PI / 128), 1, device=cuda_device)
    kw = dict(m)
    kw.pop('shape'), kw.pop('step')
    b2.set_slot(0, **kw)  # member built for 64^2 tables: forcing length mismatch is caught
  with pytest.raises(IndexError):
    b.set_steps(5, 1)


# ---- spectral batches --------------------------------------------------

def _spec_step(n, nu, k, dt):
  from jax_cfd_gb300.base import forcings, grids
  from jax_cfd_gb300.spectral import equations as seq
  from jax_cfd_gb300.spectral import time_stepping as sts
  grid = grids.Grid((n, n), domain=((0, TWO_PI), (0, TWO_PI)))
  eq = seq.NavierStokes2D(nu, grid, drag=0.1, smooth=True,
                          forcing_fn=lambda g: forcings.kolmogorov_forcing(
                              g, k=k, offsets=((0, 0), (0, 0))))
  return sts.crank_nicolson_rk4(eq, dt)


def _vorticity_hat(n, seed, vmax, dev):
  import jax_cfd_gb300.base as cfd
  from jax_cfd_gb300.spectral import utils as su
  grid = cfd.grids.Grid((n, n), domain=((0, TWO_PI), (0, TWO_PI)))
  v0 = cfd.initial_conditions.filtered_velocity_field(seed, grid, vmax, 4, device=dev)
  return su.rfft2(cfd.finite_differences.curl_2d(v0).data, grid)


@pytest.mark.parametrize('graph', [False, True])
@pytest.mark.parametrize('n', [64, 2048])
def test_spectral_batch_slots_equal_single_steps(cuda_device, graph, n):
  """Slots of a batch equal the single-trajectory step bit for bit."""
  from jax_cfd_gb300 import batching
  draws = [(1e-3, 4, 1e-2, 61, 2.0), (1e-4, 2, 5e-3, 62, 1.0), (1e-2, 8, 2e-2, 63, 3.0)]
  # dt chosen for 64^2; scaled with the grid step to keep the Courant number.
  steps = [_spec_step(n, nu, k, dt * 64 / n) for nu, k, dt, _, _ in draws]
  w0 = [_vorticity_hat(n, seed, vmax, cuda_device) for _, _, _, seed, vmax in draws]
  grid_step = steps[0].equation.grid.step
  b = batching.SpecBatch((n, n), grid_step, len(draws), device=cuda_device)
  for i, (st, w) in enumerate(zip(steps, w0)):
    b.set_slot_from_step(i, st)
    b.set_state(i, w)
    b.set_steps(i, [5, 3, 0][i])
  b.run(5, graph=graph)
  torch.cuda.synchronize(cuda_device)
  for i, (st, w) in enumerate(zip(steps, w0)):
    want = st.gb300_repeat(w, [5, 3, 0][i])
    assert torch.isfinite(torch.view_as_real(want)).all()
    assert torch.equal(torch.view_as_real(b.state(i)), torch.view_as_real(want))


def test_spectral_member_alone_equals_in_the_mix(cuda_device):
  from jax_cfd_gb300 import batching
  n = 128
  draws = [(1e-3, 4, 1e-2, 71, 2.0), (3e-4, 8, 5e-3, 72, 4.0), (5e-3, 2, 1e-2, 73, 1.5)]
  steps = [_spec_step(n, nu, k, dt) for nu, k, dt, _, _ in draws]
  w0 = [_vorticity_hat(n, seed, vmax, cuda_device) for _, _, _, seed, vmax in draws]
  grid_step = steps[0].equation.grid.step
  mix = batching.SpecBatch((n, n), grid_step, 3, device=cuda_device)
  alone = batching.SpecBatch((n, n), grid_step, 3, device=cuda_device)
  for i in range(3):
    mix.set_slot_from_step(i, steps[i])
    mix.set_state(i, w0[i])
    mix.set_steps(i, 6)
  alone.set_slot_from_step(2, steps[2])
  alone.set_state(2, w0[2])
  alone.set_steps(2, 6)
  mix.run(6)
  alone.run(6)
  torch.cuda.synchronize(cuda_device)
  assert torch.equal(torch.view_as_real(mix.state(2)), torch.view_as_real(alone.state(2)))
