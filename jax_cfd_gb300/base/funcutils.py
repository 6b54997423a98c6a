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


def trajectory(step_fn: Callable, steps: int, post_process: Callable = _identity,
               *, start_with_input: bool = False) -> Callable:
  """funcutils.py:95-126: (final state, stacked post-processed frames)."""
  def multistep(values):
    frames = []
    x = values
    for _ in range(steps):
      y = step_fn(x)
      frames.append(post_process(x if start_with_input else y))
      x = y
    return x, _tree_stack(frames)
  return multistep
