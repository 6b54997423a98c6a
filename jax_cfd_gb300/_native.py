"""ctypes binding of ``libcfd_gb300.so`` (declared in ``include/cfd_gb300.h``).

The library is the only compute path: if it is missing or cannot load, every
operation raises instead of falling back to anything else.
"""
from __future__ import annotations

import ctypes
import threading
from pathlib import Path

LIB_PATH = Path(__file__).resolve().with_name('libcfd_gb300.so')

CFD_OK = 0
CFD_ERR_INVALID_ARGUMENT = 1
CFD_ERR_UNSUPPORTED = 2
CFD_ERR_CUDA = 3
CFD_ERR_OUT_OF_MEMORY = 4
CFD_ERR_DEVICE_FAULT = 5

CONVECT_VAN_LEER = 0
CONVECT_LINEAR = 1

HEALTH_NONFINITE = 1

FRAME_VELOCITY = 0
FRAME_VORTICITY = 1

FORCE_NONE = 0
FORCE_U_OF_Y = 1
FORCE_V_OF_X = 2
FORCE_FULL = 3



class DeviceFaultError(RuntimeError):
  """A kernel's bounded wait ran out: it skipped its work and recorded a code
  in the device fault word (read it with ``device_fault``)."""


_f32p = ctypes.POINTER(ctypes.c_float)
_f64p = ctypes.POINTER(ctypes.c_double)
_vp = ctypes.c_void_p


class FvmConfig(ctypes.Structure):
  _fields_ = [
      ('nx', ctypes.c_int), ('ny', ctypes.c_int),
      ('hx', ctypes.c_double), ('hy', ctypes.c_double),
      ('density', ctypes.c_double),
      ('has_viscosity', ctypes.c_int),
      ('viscosity', ctypes.c_double),
      ('dt', ctypes.c_double),
      ('convect', ctypes.c_int),
      ('has_linear_forcing', ctypes.c_int),
      ('linear_coefficient', ctypes.c_double),
      ('const_forcing', ctypes.c_int),
      ('force_u', _f32p), ('force_v', _f32p),
  ]


class SpecConfig(ctypes.Structure):
  _fields_ = [
      ('nx', ctypes.c_int), ('ny', ctypes.c_int),
      ('hx', ctypes.c_double), ('hy', ctypes.c_double),
      ('viscosity', ctypes.c_double),
      ('drag', ctypes.c_double),
      ('dt', ctypes.c_double),
      ('smooth', ctypes.c_int),
      ('num_stages', ctypes.c_int),
      ('alphas', _f64p), ('betas', _f64p), ('gammas', _f64p),
  ]


# name -> (restype, argtypes)
_SIGNATURES = {
    'cfd_last_error': (ctypes.c_char_p, []),
    'cfd_version': (ctypes.c_int, []),
    'cfd_fvm_plan_create': (ctypes.c_int, [ctypes.POINTER(FvmConfig), ctypes.POINTER(_vp)]),
    'cfd_fvm_plan_destroy': (ctypes.c_int, [_vp]),
    'cfd_fvm_plan_bytes': (ctypes.c_longlong, [_vp]),
    'cfd_fvm_step': (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, ctypes.c_int]),
    'cfd_fvm_plan_autotune': (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, ctypes.c_int, _vp]),
    'cfd_fvm_profile': (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, ctypes.c_int, _vp]),
    'cfd_fvm_explicit_terms': (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, _vp]),
    'cfd_fvm_projection': (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, _vp]),
    'cfd_fvm_pressure_solve': (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp]),
    'cfd_fvm_divergence': (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp]),
    'cfd_fvm_curl_2d': (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp]),
    'cfd_fvm_trajectory': (ctypes.c_int, [_vp, _vp, _vp, _vp, ctypes.c_int, ctypes.c_int,
                                           ctypes.c_int, ctypes.c_int, _vp, _vp, _vp]),
    'cfd_fvm_projection_noalloc': (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                                   ctypes.c_double, _vp, _vp, _vp, _vp]),
    'cfd_device_fault': (ctypes.c_int, [ctypes.POINTER(ctypes.c_uint), ctypes.c_int]),
    'cfd_bounded_wait_selftest': (ctypes.c_int, [_vp, ctypes.c_int]),
    'cfd_fvm_plan_set_launch': (ctypes.c_int, [_vp, ctypes.c_int]),
    'cfd_fvm_plan_get_launch': (ctypes.c_int, [_vp]),
    'cfd_fvm_step_rk': (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, ctypes.c_int, ctypes.c_int,
                                        _vp, _vp]),
    'cfd_fvm_adjoint_step': (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    'cfd_fvm_adjoint_segment': (ctypes.c_int, [_vp, _vp, _vp, _vp, ctypes.c_int, _vp, _vp, _vp,
                                               _vp, _vp]),
    'cfd_fvm_diffusion_solve': (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, ctypes.c_double,
                                                ctypes.c_double]),
    'cfd_fvm_step_implicit': (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, ctypes.c_int,
                                              ctypes.c_double]),
    'cfd_fvm_batch_create': (ctypes.c_int, [ctypes.POINTER(FvmConfig), ctypes.c_int,
                                             ctypes.POINTER(_vp)]),
    'cfd_fvm_batch_destroy': (ctypes.c_int, [_vp]),
    'cfd_fvm_batch_set_launch': (ctypes.c_int, [_vp, ctypes.c_int]),
    'cfd_fvm_batch_size': (ctypes.c_int, [_vp]),
    'cfd_fvm_batch_bytes': (ctypes.c_longlong, [_vp]),
    'cfd_fvm_batch_state': (ctypes.c_int, [_vp, ctypes.c_int, ctypes.POINTER(_vp),
                                            ctypes.POINTER(_vp)]),
    'cfd_fvm_batch_set_slot': (ctypes.c_int, [_vp, _vp, ctypes.c_int, ctypes.POINTER(FvmConfig)]),
    'cfd_fvm_batch_set_steps': (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int]),
    'cfd_fvm_batch_run': (ctypes.c_int, [_vp, _vp, ctypes.c_int, ctypes.c_int]),
    'cfd_fvm_batch_autotune': (ctypes.c_int, [_vp, _vp, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]),
    'cfd_fvm_ensemble_create': (ctypes.c_int, [ctypes.POINTER(FvmConfig), ctypes.c_int,
                                                ctypes.POINTER(_vp)]),
    'cfd_fvm_ensemble_destroy': (ctypes.c_int, [_vp]),
    'cfd_fvm_ensemble_size': (ctypes.c_int, [_vp]),
    'cfd_fvm_ensemble_batches': (ctypes.c_int, [_vp]),
    'cfd_fvm_ensemble_state': (ctypes.c_int, [_vp, ctypes.c_int, ctypes.POINTER(_vp),
                                               ctypes.POINTER(_vp)]),
    'cfd_fvm_ensemble_autotune': (ctypes.c_int, [_vp, _vp, ctypes.c_int]),
    'cfd_fvm_batch_health': (ctypes.c_int, [_vp, ctypes.POINTER(_vp)]),
    'cfd_fvm_ensemble_health': (ctypes.c_int, [_vp, ctypes.c_int, ctypes.POINTER(_vp)]),
    'cfd_spec_batch_health': (ctypes.c_int, [_vp, ctypes.POINTER(_vp)]),
    'cfd_fvm_batch_set_health_mirror': (ctypes.c_int, [_vp, _vp]),
    'cfd_spec_batch_set_health_mirror': (ctypes.c_int, [_vp, _vp]),
    'cfd_fvm_ensemble_step': (ctypes.c_int, [_vp, _vp, ctypes.c_int, ctypes.c_int]),
    'cfd_energy_spectrum_shells': (ctypes.c_int, [_vp, _vp, _vp, _vp, ctypes.c_double,
                                                   ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                                   _vp]),
    'cfd_enstrophy_sum': (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                         ctypes.c_double, _vp, _vp, _vp]),
    'cfd_spec_batch_create': (ctypes.c_int, [ctypes.POINTER(SpecConfig), ctypes.c_int,
                                              ctypes.POINTER(_vp)]),
    'cfd_spec_batch_destroy': (ctypes.c_int, [_vp]),
    'cfd_spec_batch_size': (ctypes.c_int, [_vp]),
    'cfd_spec_batch_bytes': (ctypes.c_longlong, [_vp]),
    'cfd_spec_batch_state': (ctypes.c_int, [_vp, ctypes.c_int, ctypes.POINTER(_vp)]),
    'cfd_spec_batch_set_slot': (ctypes.c_int, [_vp, ctypes.c_int, ctypes.POINTER(SpecConfig), _vp]),
    'cfd_spec_batch_set_steps': (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int]),
    'cfd_spec_batch_run': (ctypes.c_int, [_vp, _vp, ctypes.c_int, ctypes.c_int]),
    'cfd_max_speed': (ctypes.c_int, [_vp, ctypes.c_int, _vp, _vp, _vp]),
    'cfd_scale_to_max_speed': (ctypes.c_int, [_vp, ctypes.c_int, _vp, _vp, _vp, ctypes.c_double]),
    'cfd_spec_plan_create': (ctypes.c_int, [ctypes.POINTER(SpecConfig), ctypes.POINTER(_vp)]),
    'cfd_spec_plan_destroy': (ctypes.c_int, [_vp]),
    'cfd_spec_plan_bytes': (ctypes.c_longlong, [_vp]),
    'cfd_spec_plan_set_launch': (ctypes.c_int, [_vp, ctypes.c_int]),
    'cfd_spec_plan_get_launch': (ctypes.c_int, [_vp]),
    'cfd_spec_set_forcing': (ctypes.c_int, [_vp, _vp, _vp, _vp]),
    'cfd_spec_step': (ctypes.c_int, [_vp, _vp, _vp, _vp, ctypes.c_int]),
    'cfd_spec_profile': (ctypes.c_int, [_vp, _vp, _vp, _vp, ctypes.c_int, _vp]),
    'cfd_spec_explicit_terms': (ctypes.c_int, [_vp, _vp, _vp, _vp]),
    'cfd_rfft2': (ctypes.c_int, [_vp, _vp, _vp, _vp]),
    'cfd_irfft2': (ctypes.c_int, [_vp, _vp, _vp, _vp]),
    'cfd_spectral_filter': (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp]),
}

_lib = None
_lock = threading.Lock()


def exported_symbols():
  """Names of every C entry point this binding declares."""
  return tuple(_SIGNATURES)


def load(path: Path | str | None = None):
  """Loads the native library (once) and declares its signatures."""
  global _lib
  with _lock:
    if _lib is not None and path is None:
      return _lib
    p = Path(path) if path is not None else LIB_PATH
    if not p.exists():
      raise RuntimeError(
          f'native library {p} is missing: build it with '
          '`python -c "import __graft_entry__ as g; g.build()"` '
          '(there is no non-native fallback)')
    lib = ctypes.CDLL(str(p))
    for name, (res, args) in _SIGNATURES.items():
      fn = getattr(lib, name)
      fn.restype = res
      fn.argtypes = args
    if path is None:
      _lib = lib
    return lib


def last_error() -> str:
  msg = load().cfd_last_error()
  return msg.decode() if msg else ''


def check(rc: int, what: str = '') -> None:
  """Maps a cfd_status to the reference's Python exception types."""
  if rc == CFD_OK:
    return
  msg = f'{what}: {last_error()}' if what else last_error()
  if rc == CFD_ERR_INVALID_ARGUMENT:
    raise ValueError(msg)
  if rc == CFD_ERR_UNSUPPORTED:
    raise NotImplementedError(msg)
  if rc == CFD_ERR_OUT_OF_MEMORY:
    raise MemoryError(msg)
  if rc == CFD_ERR_DEVICE_FAULT:
    raise DeviceFaultError(msg)
  raise RuntimeError(msg)


def device_fault(clear: bool = False) -> int:
  """The device fault word (0: no bounded wait has run out); synchronous."""
  code = ctypes.c_uint(0)
  check(load().cfd_device_fault(ctypes.byref(code), int(bool(clear))), 'cfd_device_fault')
  return int(code.value)


def call(name: str, *args) -> None:
  check(getattr(load(), name)(*args), name)
