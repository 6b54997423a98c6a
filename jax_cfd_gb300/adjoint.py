"""Differentiable FVM rollouts through a hand-written adjoint.

The reference differentiates a rollout with ``jax.grad`` through
``funcutils.repeated(semi_implicit_navier_stokes(...), steps)``
(funcutils.py:82-88, equations.py:120-151).  Here ``rollout`` is a
``torch.autograd.Function`` whose backward pass runs the native adjoint of one
step (``cfd_fvm_adjoint_step``: projection of the cotangent, transposed Van
Leer / linear advection, diffusion and forcing) once per step, newest first.
The forward pass keeps the state every ``checkpoint_every`` steps; the
backward pass recomputes the states of one segment from its checkpoint before
running that segment's adjoint steps (``cfd_fvm_adjoint_segment``: one native
call per segment, the viscosity products summed on the device), so memory is
one segment plus the checkpoints.  Gradients flow to the initial velocity and
to the viscosity.

A batch of trajectories (a leading axis) runs concurrently: each trajectory
has its own plan (workspace) and CUDA stream, forward and backward, and the
caller's stream waits for all of them.
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

  def plan(self, viscosity: float, device, index: int = 0) -> plans.FvmPlan:
    """The step's plan; `index` selects one of several plans of the same
    configuration (separate workspaces for trajectories run concurrently)."""
    import numpy as np  # pylint: disable=import-outside-toplevel
    arr = lambda t: None if t is None else np.asarray(t, dtype=np.float32)
    key = (device, self.shape, self.step, self.dt, self.density, self.convect,
           self.linear_coefficient, self.const_forcing, self.force_u, self.force_v,
           float(viscosity), int(index))
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
    gu = _owned_cotangent(gu, u_last)
    gv = _owned_cotangent(gv, u_last)
    k = max(1, int(spec.checkpoint_every))
    nu_grad = torch.zeros((), dtype=torch.float64, device=u_last.device)
    for seg in reversed(range(len(ctx.checkpoints))):
      n = min(k, spec.steps - seg * k)
      _segment_adjoint(plan, ctx.checkpoints[seg], n, gu, gv, nu_grad)
    grad_nu = (nu_grad * (spec.dt / spec.density)).to(torch.float32).reshape(ctx.nu_shape)
    return gu, gv, grad_nu, None


_STREAMS = {}


def _side_streams(device, count: int):
  """`count` CUDA streams of `device`, created once and reused."""
  key = torch.device(device)
  have = _STREAMS.setdefault(key, [])
  while len(have) < count:
    have.append(torch.cuda.Stream(key))
  return have[:count]


def _owned_cotangent(g, like):
  """A contiguous float32 copy of the incoming cotangent (zeros for None) that
  the segment adjoints may update in place."""
  if g is None:
    return torch.zeros_like(like)
  return g.detach().to(torch.float32).contiguous().clone()


def _segment_adjoint(plan, checkpoint, n: int, gu, gv, nu_acc):
  """Adjoint of `n` steps from `checkpoint` in one native call: recomputes the
  segment's states, runs its adjoint steps newest first with (gu, gv) updated
  in place, and adds the sum of the per-cell viscosity products (float64) to
  the device scalar nu_acc."""
  plan.adjoint_segment(checkpoint[0], checkpoint[1], n, gu, gv, nu_acc)


class _BatchRollout(torch.autograd.Function):
  """(u0, v0, viscosity) with a leading batch axis -> final states; each
  trajectory on its own plan and stream."""

  @staticmethod
  def forward(ctx, u0, v0, viscosity, spec: RolloutSpec):  # pylint: disable=arguments-differ
    dev = u0.device
    count = u0.shape[0]
    k = max(1, int(spec.checkpoint_every))
    nu = float(viscosity)
    plans_b = [spec.plan(nu, dev, index=b) for b in range(count)]
    main = torch.cuda.current_stream(dev)
    u0, v0 = u0.contiguous(), v0.contiguous()
    uo, vo = torch.empty_like(u0), torch.empty_like(v0)
    start = torch.cuda.Event()
    start.record(main)
    checkpoints = []
    streams = _side_streams(dev, count)
    for b, (plan, st) in enumerate(zip(plans_b, streams)):
      st.wait_event(start)
      with torch.cuda.stream(st):
        cps = []
        u, v = u0[b], v0[b]
        for s0 in range(0, spec.steps, k):
          cps.append((u, v))
          n = min(k, spec.steps - s0)
          if s0 + n >= spec.steps:
            plan.step(u, v, n, uo[b], vo[b])
          else:
            u, v = plan.step(u, v, n)
        if spec.steps == 0:
          uo[b].copy_(u)
          vo[b].copy_(v)
        checkpoints.append(cps)
      done = torch.cuda.Event()
      done.record(st)
      main.wait_event(done)
    ctx.spec, ctx.plans, ctx.checkpoints, ctx.streams = spec, plans_b, checkpoints, streams
    ctx.nu_shape = viscosity.shape
    ctx.save_for_backward(u0, v0)
    return uo, vo

  @staticmethod
  def backward(ctx, gu, gv):  # pylint: disable=arguments-differ
    spec = ctx.spec
    u0, _ = ctx.saved_tensors
    dev = u0.device
    # Owned copies, made on the caller's stream before the side streams start.
    gu_out = _owned_cotangent(gu, u0)
    gv_out = _owned_cotangent(gv, u0)
    k = max(1, int(spec.checkpoint_every))
    main = torch.cuda.current_stream(dev)
    nu_parts = torch.zeros(len(ctx.plans), dtype=torch.float64, device=dev)
    start = torch.cuda.Event()
    start.record(main)
    for b, (plan, st) in enumerate(zip(ctx.plans, ctx.streams)):
      st.wait_event(start)
      with torch.cuda.stream(st):
        cps = ctx.checkpoints[b]
        for seg in reversed(range(len(cps))):
          n = min(k, spec.steps - seg * k)
          _segment_adjoint(plan, cps[seg], n, gu_out[b], gv_out[b], nu_parts[b])
      done = torch.cuda.Event()
      done.record(st)
      main.wait_event(done)
    grad_nu = (nu_parts.sum() * (spec.dt / spec.density)).to(torch.float32).reshape(ctx.nu_shape)
    ctx.checkpoints = None
    return gu_out, gv_out, grad_nu, None


def rollout(u0: torch.Tensor, v0: torch.Tensor, viscosity, spec: RolloutSpec):
  """Differentiable ``funcutils.repeated(step, spec.steps)`` of the FVM step
  on (u0, v0); ``viscosity`` is a float or a scalar tensor (gradients flow to
  every tensor argument that requires them).  With a leading batch axis the
  trajectories run concurrently, one plan and one stream each (same results
  as one at a time)."""
  nu = viscosity if isinstance(viscosity, torch.Tensor) else torch.tensor(
      float(viscosity), dtype=torch.float32, device=u0.device)
  if u0.dim() == 3:
    return _BatchRollout.apply(u0, v0, nu, spec)
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
