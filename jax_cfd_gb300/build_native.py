"""Builds the native library ``libcfd_gb300.so`` from ``csrc/*.cu`` with nvcc.

Each translation unit is compiled for sm_103a in parallel, then linked into a
shared library that the ctypes layer (``_native.py``) loads.  Objects go to
``_build/`` beside this file; both are git-ignored build products.
"""
from __future__ import annotations

import concurrent.futures
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / 'csrc'
BUILD = PKG / '_build'
LIB = PKG / 'libcfd_gb300.so'
INCLUDE = PKG.parent / 'include'

ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
# -fmad=false: no implicit multiply-add contraction; kernels spell out each
# fma they want, so results do not depend on how a body is inlined.
NVCC_FLAGS = ['-O3', '-lineinfo', '-std=c++17', '-fmad=false', '-Xcompiler', '-fPIC',
              '--expt-relaxed-constexpr', '-I', str(INCLUDE)]


def _nvcc() -> str:
  cand = shutil.which('nvcc') or '/usr/local/cuda/bin/nvcc'
  if not os.path.exists(cand):
    raise RuntimeError('nvcc not found; the CUDA toolkit is required to build')
  return cand


def sources():
  return sorted(CSRC.glob('*.cu'))


def _stale() -> bool:
  if not LIB.exists():
    return True
  t = LIB.stat().st_mtime
  deps = list(CSRC.glob('*')) + list(INCLUDE.glob('*.h'))
  return any(d.stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False, extra_flags=()) -> Path:
  """Compiles and links the library; returns its path."""
  if not force and not _stale():
    return LIB
  nvcc = _nvcc()
  BUILD.mkdir(exist_ok=True)
  srcs = sources()

  def compile_one(src: Path) -> Path:
    obj = BUILD / (src.stem + '.o')
    cmd = [nvcc, *ARCH, *NVCC_FLAGS, *extra_flags, '-c', str(src), '-o', str(obj)]
    if verbose:
      print(' '.join(cmd), file=sys.stderr)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
      raise RuntimeError(f'nvcc failed on {src.name}:\n{r.stdout}\n{r.stderr}')
    if verbose and (r.stdout or r.stderr):
      print(r.stdout + r.stderr, file=sys.stderr)
    return obj

  with concurrent.futures.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
    objs = list(ex.map(compile_one, srcs))
  tmp = LIB.with_suffix('.so.tmp')
  cmd = [nvcc, *ARCH, '-shared', '-o', str(tmp), *map(str, objs)]
  r = subprocess.run(cmd, capture_output=True, text=True)
  if r.returncode != 0:
    raise RuntimeError(f'nvcc link failed:\n{r.stdout}\n{r.stderr}')
  os.replace(tmp, LIB)
  return LIB


if __name__ == '__main__':
  build(force='--force' in sys.argv, verbose='-v' in sys.argv)
  print(LIB)
