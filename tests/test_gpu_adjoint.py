"""The hand-written adjoint of the FVM step against float64 autograd of the
restatement (the jax.grad stand-in) and against central finite differences.

Tolerances: the GPU adjoint runs in float32 and is compared with float64
gradients, so relative L2 errors of a few 1e-5 per step are float32 rounding;
the bounds below leave room for the accumulation over a rollout.  Finite
differences use eps = 1e-3 along unit-norm random directions with the float64
forward, so they are accurate to O(eps^2) away from limiter kinks.
"""
import numpy as np
import pytest
import torch

from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu

TWO_PI = 2 * np.pi


def _case(n, seed, nu=1e-3, vmax=2.0, k=4):
  import jax_cfd_gb300.base as cfd
  from jax_cfd_gb300 import adjoint
  from oracle import fvm as ofvm
  from oracle import initial_conditions as oic
  og = ofvm.Grid.make((n, n), domain=((0, TWO_PI), (0, TWO_PI)))
  v0 = oic.filtered_velocity_field(seed, og, vmax, 4)
  grid = cfd.grids.Grid((n, n), domain=((0, TWO_PI), (0, TWO_PI)))
  dt = cfd.equations.stable_time_step(vmax, 0.5, nu, grid)
  step = cfd.equations.semi_implicit_navier_stokes(
      1.0, nu, dt, grid, forcing=cfd.forcings.simple_turbulence_forcing(grid, 1, k, -0.1))
  const_u = ofvm.kolmogorov_forcing(og, 1, k)(None)[0].astype(np.float64)
  return og, v0, step, dt, const_u, adjoint


def _torch_step(og, nu, dt, const_u, convect='van_leer'):
  from oracle import fvm_torch as otorch
  return otorch.step_fn(1.0, nu, dt, og, convect=convect, linear_coefficient=-0.1,
                        const_u=torch.from_numpy(const_u))


@pytest.mark.parametrize('convect', ['van_leer', 'linear'])
def test_adjoint_step_matches_float64_autograd(cuda_device, convect):
  import jax_cfd_gb300.base as cfd
  from jax_cfd_gb300 import plans
  og, v0, step, dt, const_u, _ = _case(64, seed=3)
  conv = None if convect == 'van_leer' else cfd.advection.convect_linear
  grid = step.grid
  step = cfd.equations.semi_implicit_navier_stokes(
      1.0, 1e-3, dt, grid, convect=conv,
      forcing=cfd.forcings.simple_turbulence_forcing(grid, 1, 4, -0.1))
  rng = np.random.default_rng(11)
  g = [rng.standard_normal(og.shape) for _ in range(2)]
  # float64 autograd of one step (viscosity as a differentiable tensor)
  nu = torch.tensor(1e-3, dtype=torch.float64, requires_grad=True)
  x = [torch.from_numpy(a.astype(np.float64)).requires_grad_() for a in v0]
  out = _torch_step(og, nu, dt, const_u, convect)(tuple(x))
  sum((o * torch.from_numpy(gi)).sum() for o, gi in zip(out, g)).backward()
  # GPU adjoint
  plan = step.plan(cuda_device)
  dev = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).to(cuda_device)
  gu, gv, nu_dot = plan.adjoint_step(dev(v0[0]), dev(v0[1]), dev(g[0]), dev(g[1]))
  assert rel_l2(gu.cpu().numpy(), x[0].grad.numpy()) <= 2e-5
  assert rel_l2(gv.cpu().numpy(), x[1].grad.numpy()) <= 2e-5
  nu_grad = float(nu_dot.double().sum()) * dt
  assert abs(nu_grad - float(nu.grad)) <= 1e-4 * abs(float(nu.grad))


@pytest.mark.parametrize('n', [64, 256])
def test_adjoint_segment_matches_the_step_loop(cuda_device, n):
  """cfd_fvm_adjoint_segment (one native call per checkpoint segment) gives
  the bits of recomputing the segment with single steps and running
  cfd_fvm_adjoint_step newest first; its viscosity sum (double, fixed order)
  agrees with the float64 sum of the per-step products."""
  og, v0, step, dt, const_u, _ = _case(n, seed=8)
  plan = step.plan(cuda_device)
  dev = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).to(cuda_device)
  rng = np.random.default_rng(4)
  g0 = [dev(rng.standard_normal(og.shape)) for _ in range(2)]
  u0, w0 = dev(v0[0]), dev(v0[1])
  steps = 5
  states = [(u0, w0)]
  for _ in range(steps - 1):
    states.append(plan.step(*states[-1], 1))
  gu, gv = g0[0].clone(), g0[1].clone()
  want_nu = 0.0
  for t in reversed(range(steps)):
    gu, gv, nu_dot = plan.adjoint_step(states[t][0], states[t][1], gu, gv)
    want_nu += float(nu_dot.double().sum())
  su, sv = g0[0].clone(), g0[1].clone()
  acc = torch.zeros((), dtype=torch.float64, device=cuda_device)
  plan.adjoint_segment(u0, w0, steps, su, sv, acc)
  assert torch.equal(su, gu) and torch.equal(sv, gv)
  assert abs(float(acc) - want_nu) <= 1e-12 * abs(want_nu)
  # One step: no recomputed states.
  su1, sv1 = g0[0].clone(), g0[1].clone()
  plan.adjoint_segment(u0, w0, 1, su1, sv1)
  gu1, gv1, _ = plan.adjoint_step(u0, w0, g0[0], g0[1])
  assert torch.equal(su1, gu1) and torch.equal(sv1, gv1)


def _vorticity64(v, og):
  from oracle import fvm_torch as otorch
  return otorch.curl_2d(v, og.step)


def test_rollout_gradient_matches_float64_autograd_and_checkpoints(cuda_device):
  from jax_cfd_gb300 import adjoint
  og, v0, step, dt, const_u, _ = _case(64, seed=5)
  _, target_v, _, _, _, _ = _case(64, seed=105)
  steps = 24
  target = _vorticity64(tuple(torch.from_numpy(a.astype(np.float64)) for a in target_v), og)
  # float64 reference gradient
  nu = torch.tensor(1e-3, dtype=torch.float64, requires_grad=True)
  x = [torch.from_numpy(a.astype(np.float64)).requires_grad_() for a in v0]
  from oracle import fvm_torch as otorch
  out = otorch.rollout(_torch_step(og, nu, dt, const_u), tuple(x), steps)
  ((_vorticity64(out, og) - target) ** 2).mean().backward()
  # GPU: hand-written adjoint at several checkpoint intervals
  grads = []
  for every in (1, 8, 24):
    spec = adjoint.spec_for(step, steps, checkpoint_every=every)
    u0 = torch.from_numpy(v0[0]).to(cuda_device).requires_grad_()
    w0 = torch.from_numpy(v0[1]).to(cuda_device).requires_grad_()
    nug = torch.tensor(1e-3, device=cuda_device, requires_grad=True)
    u, v = adjoint.rollout(u0, w0, nug, spec)
    loss = ((adjoint.vorticity(u, v, og.step) - target.float().to(cuda_device)) ** 2).mean()
    loss.backward()
    grads.append((u0.grad.clone(), w0.grad.clone(), nug.grad.clone()))
  for a, b in zip(grads[0], grads[1]):
    assert torch.equal(a, b)
  for a, b in zip(grads[0], grads[2]):
    assert torch.equal(a, b)
  gu, gv, gn = grads[0]
  assert rel_l2(gu.cpu().numpy(), x[0].grad.numpy()) <= 1e-3
  assert rel_l2(gv.cpu().numpy(), x[1].grad.numpy()) <= 1e-3
  assert abs(float(gn) - float(nu.grad)) <= 1e-3 * abs(float(nu.grad))


def test_rollout_gradient_matches_central_differences(cuda_device):
  from jax_cfd_gb300 import adjoint
  from oracle import fvm_torch as otorch
  og, v0, step, dt, const_u, _ = _case(32, seed=7)
  steps = 16
  rng = np.random.default_rng(3)
  target = torch.from_numpy(rng.standard_normal(og.shape))
  spec = adjoint.spec_for(step, steps, checkpoint_every=4)
  u0 = torch.from_numpy(v0[0]).to(cuda_device).requires_grad_()
  w0 = torch.from_numpy(v0[1]).to(cuda_device).requires_grad_()
  nug = torch.tensor(1e-3, device=cuda_device, requires_grad=True)
  u, v = adjoint.rollout(u0, w0, nug, spec)
  ((adjoint.vorticity(u, v, og.step) - target.float().to(cuda_device)) ** 2).mean().backward()
  gx = np.concatenate([u0.grad.cpu().numpy().ravel(), w0.grad.cpu().numpy().ravel()])

  def loss64(xvec, nu):
    n = og.shape[0] * og.shape[1]
    v = (torch.from_numpy(xvec[:n].reshape(og.shape)), torch.from_numpy(xvec[n:].reshape(og.shape)))
    out = otorch.rollout(_torch_step(og, nu, dt, const_u), v, steps)
    return float(((_vorticity64(out, og) - target) ** 2).mean())
  x0 = np.concatenate([v0[0].ravel(), v0[1].ravel()]).astype(np.float64)
  eps = 1e-3
  worst = 0.0
  for _ in range(32):
    d = rng.standard_normal(x0.shape)
    d /= np.linalg.norm(d)
    fd = (loss64(x0 + eps * d, 1e-3) - loss64(x0 - eps * d, 1e-3)) / (2 * eps)
    worst = max(worst, abs(fd - gx @ d) / (abs(fd) + 1e-12))
  assert worst <= 5e-3
  fd_nu = (loss64(x0, 1e-3 + 1e-6) - loss64(x0, 1e-3 - 1e-6)) / 2e-6
  assert abs(float(nug.grad) - fd_nu) <= 5e-3 * abs(fd_nu)


def test_config3_gradient_at_512(cuda_device):
  """The differentiation workload at its own scale, one trajectory: 512^2,
  64 steps, a checkpoint every 8, loss = mean squared vorticity error against
  a target produced by the float64 restatement from another seed (the
  reference stand-in).  The GPU gradient (initial velocity and viscosity) is
  compared with float64 autograd of the restatement (the jax.grad stand-in,
  run on the GPU in float64) and with 32 central differences of the float64
  forward along unit-norm random directions, eps 1e-3 (advection_test.py:298-314
  differentiates the same kind of rollout with jax.grad through jax.remat).
  A batch of two trajectories (run concurrently) gives the single
  trajectories' bits."""
  from jax_cfd_gb300 import adjoint
  from oracle import fvm_torch as otorch
  n, steps, every, nu0 = 512, 64, 8, 1e-3
  og, v0, step, dt, const_u, _ = _case(n, seed=0)
  _, vt, _, _, _, _ = _case(n, seed=100)
  dev64 = lambda a: torch.from_numpy(np.asarray(a, dtype=np.float64)).to(cuda_device)
  f64 = otorch.step_fn(1.0, nu0, dt, og, linear_coefficient=-0.1, const_u=dev64(const_u))
  with torch.no_grad():
    target = otorch.curl_2d(otorch.rollout(f64, tuple(dev64(a) for a in vt), steps), og.step)
  # float64 autograd (viscosity differentiable)
  nu = torch.tensor(nu0, dtype=torch.float64, device=cuda_device, requires_grad=True)
  x = [dev64(a).requires_grad_() for a in v0]
  fn = otorch.step_fn(1.0, nu, dt, og, linear_coefficient=-0.1, const_u=dev64(const_u))
  out = otorch.rollout(fn, tuple(x), steps)
  ((otorch.curl_2d(out, og.step) - target) ** 2).mean().backward()
  # GPU hand-written adjoint
  spec = adjoint.spec_for(step, steps, checkpoint_every=every)
  u0 = torch.from_numpy(v0[0]).to(cuda_device).requires_grad_()
  w0 = torch.from_numpy(v0[1]).to(cuda_device).requires_grad_()
  nug = torch.tensor(nu0, device=cuda_device, requires_grad=True)
  u, v = adjoint.rollout(u0, w0, nug, spec)
  ((adjoint.vorticity(u, v, og.step) - target.float()) ** 2).mean().backward()
  eu = rel_l2(u0.grad.cpu().numpy(), x[0].grad.cpu().numpy())
  ev = rel_l2(w0.grad.cpu().numpy(), x[1].grad.cpu().numpy())
  en = abs(float(nug.grad) - float(nu.grad)) / abs(float(nu.grad))
  print(f'512^2 x 64 steps: gradient vs float64 autograd: u {eu:.2e}, v {ev:.2e}, nu {en:.2e}')
  assert eu <= 1e-2 and ev <= 1e-2 and en <= 1e-2
  # 32 central differences of the float64 forward.
  gx = torch.cat([u0.grad.double().ravel(), w0.grad.double().ravel()])
  rng = np.random.default_rng(21)
  x0 = torch.cat([dev64(v0[0]).ravel(), dev64(v0[1]).ravel()])
  cells = n * n

  def loss64(xvec):
    with torch.no_grad():
      vv = (xvec[:cells].reshape(og.shape), xvec[cells:].reshape(og.shape))
      return float(((otorch.curl_2d(otorch.rollout(f64, vv, steps), og.step) - target) ** 2).mean())
  eps, worst = 1e-3, 0.0
  for _ in range(32):
    d = torch.from_numpy(rng.standard_normal(2 * cells)).to(cuda_device)
    d /= torch.linalg.norm(d)
    fd = (loss64(x0 + eps * d) - loss64(x0 - eps * d)) / (2 * eps)
    worst = max(worst, abs(fd - float(gx @ d)) / (abs(fd) + 1e-30))
  print(f'512^2 x 64 steps: worst relative error over 32 central differences {worst:.2e}')
  assert worst <= 1e-2
  # A batch of two runs concurrently and gives the single trajectories' bits.
  _, v1, _, _, _, _ = _case(n, seed=1)
  ub = torch.stack([torch.from_numpy(v0[0]), torch.from_numpy(v1[0])]).to(cuda_device).requires_grad_()
  wb = torch.stack([torch.from_numpy(v0[1]), torch.from_numpy(v1[1])]).to(cuda_device).requires_grad_()
  nub = torch.tensor(nu0, device=cuda_device, requires_grad=True)
  a, b = adjoint.rollout(ub, wb, nub, spec)
  assert torch.equal(a[0], u) and torch.equal(b[0], v)
  ((adjoint.vorticity(a[0], b[0], og.step) - target.float()) ** 2).mean().backward()
  assert torch.equal(ub.grad[0], u0.grad) and torch.equal(wb.grad[0], w0.grad)
  assert torch.equal(nub.grad, nug.grad)
  assert float(ub.grad[1].abs().max()) == 0.0
