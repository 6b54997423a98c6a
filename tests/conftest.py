"""Test configuration: the `gpu` marker and shared helpers."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
  sys.path.insert(0, ROOT)


def pytest_configure(config):
  config.addinivalue_line('markers', 'gpu: needs a CUDA GPU (GB300) and the native library')


def rel_l2(a, b) -> float:
  a = np.asarray(a)
  b = np.asarray(b)
  dt = np.complex128 if (np.iscomplexobj(a) or np.iscomplexobj(b)) else np.float64
  a = a.astype(dt)
  b = b.astype(dt)
  return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture(scope='session')
def cuda_device():
  import torch  # pylint: disable=import-outside-toplevel
  if not torch.cuda.is_available():
    pytest.fail('gpu tests need a CUDA device')
  from jax_cfd_gb300 import _native  # pylint: disable=import-outside-toplevel
  _native.load()
  return torch.device('cuda', 0)
