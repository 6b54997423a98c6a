"""The float64 torch restatement used as the jax.grad stand-in (CPU only):
pinned to the NumPy oracle's forward step, and its autograd gradients to
central finite differences."""
import numpy as np
import pytest
import torch

from oracle import fvm as ofvm
from oracle import fvm_torch as otorch
from oracle import initial_conditions as oic

TWO_PI = 2 * np.pi


def _setup(n, seed=0, vmax=2.0):
  og = ofvm.Grid.make((n, n), domain=((0, TWO_PI), (0, TWO_PI)))
  v0 = oic.filtered_velocity_field(seed, og, vmax, 4)
  return og, tuple(a.astype(np.float64) for a in v0)


def test_restatement_forward_matches_numpy_oracle_in_float64():
  og, v0 = _setup(32, seed=1)
  dt = ofvm.stable_time_step(2.0, 0.5, 1e-3, og)
  forcing = ofvm.simple_turbulence_forcing(og, 1, 4, -0.1)
  ref = ofvm.repeated(ofvm.semi_implicit_navier_stokes(
      1.0, 1e-3, dt, og, forcing=forcing, diag=ofvm.pinv_diagonal(og, np.float64)), 3)(v0)
  const_u = ofvm.kolmogorov_forcing(og, 1, 4)(None)[0].astype(np.float64)
  f = otorch.step_fn(1.0, 1e-3, dt, og, linear_coefficient=-0.1,
                     const_u=torch.from_numpy(const_u))
  got = otorch.rollout(f, tuple(torch.from_numpy(a) for a in v0), 3)
  for g, r in zip(got, ref):
    np.testing.assert_allclose(g.numpy(), r, rtol=0, atol=1e-12)


def test_restatement_autograd_matches_central_differences():
  og, v0 = _setup(16, seed=2)
  dt = ofvm.stable_time_step(2.0, 0.5, 1e-3, og)
  f = otorch.step_fn(1.0, 1e-3, dt, og, linear_coefficient=-0.1)
  x = [torch.from_numpy(a.copy()).requires_grad_() for a in v0]
  rng = np.random.default_rng(0)
  w = [torch.from_numpy(rng.standard_normal(a.shape)) for a in v0]

  def loss(v):
    out = otorch.rollout(f, v, 2)
    return sum((o * wi).sum() for o, wi in zip(out, w))
  loss(x).backward()
  for _ in range(3):
    d = [torch.from_numpy(rng.standard_normal(a.shape)) for a in v0]
    eps = 1e-6
    with torch.no_grad():
      lp = loss([a + eps * di for a, di in zip(x, d)])
      lm = loss([a - eps * di for a, di in zip(x, d)])
    fd = (lp - lm) / (2 * eps)
    ad = sum((xi.grad * di).sum() for xi, di in zip(x, d))
    assert abs(float(fd - ad)) <= 1e-6 * abs(float(ad)) + 1e-9


# --- advection_test.py:298-351 (gradients through Van Leer advection) -------
def _unit_velocity(shape, sign=1.):
  nd = len(shape)
  offs = tuple(tuple((np.eye(nd) + np.ones((nd, nd)))[ax] / 2.) for ax in range(nd))
  v = tuple(torch.full(shape, sign, dtype=torch.float64) if ax == 0
            else torch.zeros(shape, dtype=torch.float64) for ax in range(nd))
  return v, offs


def _advected_gradient(c0, shape, sign):
  """Gradient of 0.5 |c_T|^2 after 10 forward-Euler Van Leer (limiter)
  advection steps at CFL 0.5 in a unit velocity, h = 1 / n."""
  step = tuple(1. / s for s in shape)
  v, offs = _unit_velocity(shape, sign)
  dt = 0.5 * min(step)
  c0 = c0.clone().requires_grad_(True)
  c = c0
  for _ in range(10):
    c = c + dt * otorch.advect(c, (0.5,) * len(shape), v, offs, dt, step)
  (0.5 * (c ** 2).sum()).backward()
  return c0.grad


@pytest.mark.parametrize('shape,sign', [((101,), 1.), ((101,), -1.), ((101, 101), 1.)])
def test_van_leer_advection_gradient_is_the_concentration(shape, sign):
  """Advection at unit speed nearly conserves 0.5 |c|^2, so its gradient is
  c (atol and rtol 1e-2), for a Gaussian centred in the box."""
  step = tuple(1. / s for s in shape)
  axes = [(np.arange(s) - int(np.ceil(s / 2.))) * h for s, h in zip(shape, step)]
  c0 = torch.tensor(np.exp(-sum(m ** 2 * 30. for m in np.meshgrid(*axes, indexing='ij'))))
  g = _advected_gradient(c0, shape, sign)
  torch.testing.assert_close(g, c0, atol=1e-2, rtol=1e-2)


@pytest.mark.parametrize('sign', [1., -1.])
def test_van_leer_advection_gradient_of_a_constant_is_finite(sign):
  """A constant field makes every limiter ratio 0/0: the gradient must still
  be the field (safe_div's where-branches carry no NaN)."""
  c0 = torch.ones((101,), dtype=torch.float64)
  g = _advected_gradient(c0, (101,), sign)
  assert torch.isfinite(g).all()
  torch.testing.assert_close(g, c0, atol=1e-2, rtol=1e-2)

