"""Drivers, mirroring ``jax_cfd/base/funcutils.py:65-126``.

``repeated`` hands a fused step to its native multi-step entry point (one
enqueue of all ``steps``), which is where the reference's ``lax.scan`` loop
lives on GB300.  Other callables are applied in a host loop.
"""
from __future__ import annotations

import contextlib
from typing import Any, Callable, Sequence

import torch

from jax_cfd_gb300.base import grids

PyTree = Any

_INITIALIZING = 0


@contextlib.contextmanager
def init_context():
  global _INITIALIZING
  _INITIALIZING += 1
  try:
    yield
  finally:
    _INITIALIZING -= 1


def _tree_stack(trees: Sequence[PyTree]) -> PyTree:
  """Stacks a list of identically structured pytrees along a new axis 0."""
  if not trees:
    return trees
  first = trees[0]
  if isinstance(first, grids.GridVariable):
    arr = _tree_stack([t.array for t in trees])
    return grids.GridVariable(arr, first.bc)
  if isinstance(first, grids.GridArray):
    return grids.GridArray(torch.stack([t.data for t in trees]), first.offset, first.grid)
  if isinstance(first, (tuple, list)):
    return type(first)(_tree_stack([t[i] for t in trees]) for i in range(len(first)))
  if isinstance(first, dict):
    return {k: _tree_stack([t[k] for t in trees]) for k in first}
  return torch.stack([torch.as_tensor(t) for t in trees])


def scan(f, init, xs, length=None):
  """funcutils.py:65-79 as a host loop over f(carry, x) -> (carry, y)."""
  if xs is None:
    xs = [None] * length
  carry, ys = init, []
  for x in xs:
    carry, y = f(carry, x)
    ys.append(y)
    if _INITIALIZING:
      ys = ys * len(xs)
      break
  if ys and ys[0] is None:
    return carry, None
  return carry, _tree_stack(ys)


def repeated(f: Callable, steps: int) -> Callable:
  """funcutils.py:82-88."""
  multistep = getattr(f, 'gb300_repeat', None)

  def f_repeated(x_initial):
    if multistep is not None:
      return multistep(x_initial, steps)
    x = x_initial
    for _ in range(steps):
      x = f(x)
    return x
  f_repeated.gb300_inner = f
  f_repeated.gb300_steps = steps
  return f_repeated


def _identity(x):
  return x


def _native_trajectory(step_fn: Callable, post_process: Callable):
  """(FvmStep, inner steps, frame kind) when the trajectory maps onto
  cfd_fvm_trajectory: a forward-Euler FvmStep, alone or under repeated(), with
  post_process the identity or finite_differences.curl_2d; else None."""
  from jax_cfd_gb300 import _native  # pylint: disable=import-outside-toplevel
  from jax_cfd_gb300.base import equations, finite_differences  # pylint: disable=import-outside-toplevel
  inner, f = 1, step_fn
  if getattr(step_fn, 'gb300_inner', None) is not None:
    inner, f = step_fn.gb300_steps, step_fn.gb300_inner
  if not isinstance(f, equations.FvmStep) or f.tableau is not None or (
      f.implicit_viscosity is not None):
    return None
  if post_process is _identity:
    return f, inner, _native.FRAME_VELOCITY
  if post_process is finite_differences.curl_2d:
    return f, inner, _native.FRAME_VORTICITY
  return None


def trajectory(step_fn: Callable, steps: int, post_process: Callable = _identity,
               *, start_with_input: bool = False) -> Callable:
  """funcutils.py:95-126: (final state, stacked post-processed frames).

  For the forward-Euler step (alone or under ``repeated``) with
  ``post_process`` the identity or ``finite_differences.curl_2d``, the whole
  trajectory is one native call that writes each frame into a device buffer
  (``cfd_fvm_trajectory``); other steps and post-processing run frame by
  frame on the device from a host loop.  Both give the same bits.
  """
  def multistep(values):
    native = _native_trajectory(step_fn, post_process)
    if native is not None and steps > 0:
      return _run_native(native, values)
    frames = []
    x = values
    for _ in range(steps):
      y = step_fn(x)
      frames.append(post_process(x if start_with_input else y))
      x = y
    return x, _tree_stack(frames)

  def _run_native(native, v):
    from jax_cfd_gb300 import _native  # pylint: disable=import-outside-toplevel
    from jax_cfd_gb300.base import equations  # pylint: disable=import-outside-toplevel
    f, inner, kind = native
    equations._check_state(v, f.grid)  # pylint: disable=protected-access
    plan = f.plan(v[0].data.device)
    uo, vo, out = plan.trajectory(v[0].data, v[1].data, inner, steps, kind, start_with_input)
    final = (grids.GridVariable(grids.GridArray(uo, v[0].offset, f.grid), v[0].bc),
             grids.GridVariable(grids.GridArray(vo, v[1].offset, f.grid), v[1].bc))
    if kind == _native.FRAME_VELOCITY:
      stacked = (grids.GridVariable(grids.GridArray(out[:, 0], v[0].offset, f.grid), v[0].bc),
                 grids.GridVariable(grids.GridArray(out[:, 1], v[1].offset, f.grid), v[1].bc))
    else:
      stacked = grids.GridArray(out, (1.0, 1.0), f.grid)
    return final, stacked
  return multistep
