"""Differentiable FVM rollouts through a hand-written adjoint.

The reference differentiates a rollout with ``jax.grad`` through
``funcutils.repeated(semi_implicit_navier_stokes(...), steps)``
(funcutils.py:82-88, equations.py:120-151).  Here ``rollout`` is a
``torch.autograd.Function`` whose backward pass runs the native adjoint of one
step (``cfd_fvm_adjoint_step``: projection of the cotangent, transposed Van
Leer / linear advection, diffusion and forcing) once per step, newest first.
The forward pass keeps the state every ``checkpoint_every`` steps; the
backward pass recomputes the states of one segment from its checkpoint before
running that segment's adjoint steps, so memory is one segment plus the
checkpoints.  Gradients flow to the initial velocity and to the viscosity.
"""
from __future__ import annotations

import dataclasses
from typing import Optional, Tuple

import torch

from jax_cfd_gb300 import _native as nat
from jax_cfd_gb300 import plans


@dataclasses.dataclass(frozen=True)
class RolloutSpec:
  """Everything about a rollout except the differentiable inputs."""
  shape: Tuple[int, int]
  step: Tuple[float, float]
  dt: float
  steps: int
  density: float = 1.0
  convect: int = nat.CONVECT_VAN_LEER
  linear_coefficient: Optional[float] = None
  const_forcing: int = nat.FORCE_NONE
  force_u: Optional[tuple] = None
  force_v: Optional[tuple] = None
  checkpoint_every: int = 8

  def plan(self, viscosity: float, device) -> plans.FvmPlan:
    import numpy as np  # pylint: disable=import-outside-toplevel
    arr = lambda t: None if t is None else np.asarray(t, dtype=np.float32)
    key = (device, self.shape, self.step, self.dt, self.density, self.convect,
           self.linear_coefficient, self.const_forcing, self.force_u, self.force_v,
           float(viscosity))
    return plans.cached('adjoint', key, lambda: plans.FvmPlan(
        self.shape, self.step, density=self.density, viscosity=float(viscosity), dt=self.dt,
        convect=self.convect, linear_coefficient=self.linear_coefficient,
        const_forcing=self.const_forcing, force_u=arr(self.force_u),
        force_v=arr(self.force_v), device=device))


class _Rollout(torch.autograd.Function):
  """(u0, v0, viscosity) -> state after spec.steps steps."""

  @staticmethod
  def forward(ctx, u0, v0, viscosity, spec: RolloutSpec):  # pylint: disable=arguments-differ
    plan = spec.plan(float(viscosity), u0.device)
    k = max(1, int(spec.checkpoint_every))
    checkpoints = []
    u, v = u0.contiguous(), v0.contiguous()
    for s0 in range(0, spec.steps, k):
      checkpoints.append((u, v))
      u, v = plan.step(u, v, min(k, spec.steps - s0))
    ctx.spec, ctx.plan, ctx.checkpoints = spec, plan, checkpoints
    ctx.nu_shape = viscosity.shape
    return u, v

  @staticmethod
  def backward(ctx, gu, gv):  # pylint: disable=arguments-differ
    spec, plan = ctx.spec, ctx.plan
    u_last = ctx.checkpoints[0][0]
    gu = torch.zeros_like(u_last) if gu is None else gu.contiguous().float()
    gv = torch.zeros_like(u_last) if gv is None else gv.contiguous().float()
    k = max(1, int(spec.checkpoint_every))
    nu_grad = torch.zeros((), dtype=torch.float64, device=u_last.device)
    for seg in reversed(range(len(ctx.checkpoints))):
      n = min(k, spec.steps - seg * k)
      states = [ctx.checkpoints[seg]]
      for _ in range(n - 1):
        states.append(plan.step(*states[-1], 1))
      for t in reversed(range(n)):
        gu, gv, nu_dot = plan.adjoint_step(states[t][0], states[t][1], gu, gv)
        nu_grad = nu_grad + nu_dot.double().sum()
    grad_nu = (nu_grad * (spec.dt / spec.density)).to(torch.float32).reshape(ctx.nu_shape)
    return gu, gv, grad_nu, None


def rollout(u0: torch.Tensor, v0: torch.Tensor, viscosity, spec: RolloutSpec):
  """Differentiable ``funcutils.repeated(step, spec.steps)`` of the FVM step
  on (u0, v0); ``viscosity`` is a float or a scalar tensor (gradients flow to
  every tensor argument that requires them).  A leading batch axis runs each
  trajectory in turn."""
  nu = viscosity if isinstance(viscosity, torch.Tensor) else torch.tensor(
      float(viscosity), dtype=torch.float32, device=u0.device)
  if u0.dim() == 3:
    outs = [_Rollout.apply(u0[b], v0[b], nu, spec) for b in range(u0.shape[0])]
    return torch.stack([o[0] for o in outs]), torch.stack([o[1] for o in outs])
  return _Rollout.apply(u0, v0, nu, spec)


def spec_for(step_fn, steps: int, checkpoint_every: int = 8) -> RolloutSpec:
  """RolloutSpec of a drop-in step from ``equations.semi_implicit_navier_stokes``."""
  from jax_cfd_gb300.base import equations  # pylint: disable=import-outside-toplevel
  if not isinstance(step_fn, equations.FvmStep):
    raise NotImplementedError('rollouts differentiate semi_implicit_navier_stokes steps')
  kw = dict(step_fn._plan_kwargs)  # pylint: disable=protected-access
  tup = lambda a: None if a is None else tuple(float(x) for x in a.ravel())
  return RolloutSpec(shape=tuple(step_fn.grid.shape), step=tuple(step_fn.grid.step),
                     dt=float(kw['dt']), steps=int(steps), density=float(kw['density']),
                     convect=int(kw['convect']), linear_coefficient=kw['linear_coefficient'],
                     const_forcing=int(kw['const_forcing']), force_u=tup(kw['force_u']),
                     force_v=tup(kw['force_v']), checkpoint_every=int(checkpoint_every))


def vorticity(u: torch.Tensor, v: torch.Tensor, step) -> torch.Tensor:
  """curl_2d (finite_differences.py:186-193) with torch ops (differentiable)."""
  hx, hy = step
  return ((torch.roll(v, -1, dims=-2) - v) / hx) - ((torch.roll(u, -1, dims=-1) - u) / hy)
