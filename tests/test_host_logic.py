"""Host-side logic of the drop-in API and the C ABI (CPU only, no GPU work).

* the native library loads and exports every entry point the public header
  declares (no compute calls: there is no GPU here);
* argument pattern-matching of semi_implicit_navier_stokes onto the fused
  kernels, with the reference's exception types for unsupported options;
* forcing descriptors, grid geometry and driver semantics.
"""
import re
from pathlib import Path

import numpy as np
import pytest
import torch

ROOT = Path(__file__).resolve().parents[1]


def _header_functions():
  text = (ROOT / 'include' / 'cfd_gb300.h').read_text()
  text = re.sub(r'/\*.*?\*/', '', text, flags=re.S)
  return sorted(set(re.findall(r'\b(cfd_[a-z0-9_]+)\s*\(', text)))


@pytest.fixture(scope='module')
def lib():
  from jax_cfd_gb300 import _native, build_native
  build_native.build()
  return _native.load()


def test_library_exports_every_declared_symbol(lib):
  declared = _header_functions()
  assert 'cfd_fvm_step' in declared and 'cfd_spec_step' in declared
  for name in declared:
    assert hasattr(lib, name), name


def test_binding_declares_exactly_the_header(lib):
  from jax_cfd_gb300 import _native
  assert sorted(_native.exported_symbols()) == _header_functions()


def test_status_codes_map_to_reference_exceptions(lib):
  from jax_cfd_gb300 import _native
  _native.check(_native.CFD_OK)
  for code, exc in ((_native.CFD_ERR_INVALID_ARGUMENT, ValueError),
                    (_native.CFD_ERR_UNSUPPORTED, NotImplementedError),
                    (_native.CFD_ERR_OUT_OF_MEMORY, MemoryError),
                    (_native.CFD_ERR_CUDA, RuntimeError),
                    (_native.CFD_ERR_DEVICE_FAULT, _native.DeviceFaultError)):
    with pytest.raises(exc):
      _native.check(code)


def test_bounded_wait_selftest_validates_before_launching(lib):
  from jax_cfd_gb300 import _native
  for polls in (0, -3, (1 << 22) + 1):
    assert lib.cfd_bounded_wait_selftest(None, polls) == _native.CFD_ERR_INVALID_ARGUMENT
    assert 'polls' in _native.last_error()


def test_adjoint_segment_validates_before_launching(lib):
  from jax_cfd_gb300 import _native
  fake = 0x1000  # never dereferenced: validation fails first
  # no plan; zero steps; missing state buffer for steps > 1; one of the two
  # viscosity pointers without the other
  cases = [(None, fake, fake, 2, fake, fake, fake, None, None),
           (fake, fake, fake, 0, fake, fake, fake, None, None),
           (fake, fake, fake, 3, None, fake, fake, None, None),
           (fake, fake, fake, 1, None, fake, fake, fake, None)]
  for plan, u, v, steps, states, gu, gv, scratch, acc in cases:
    rc = lib.cfd_fvm_adjoint_segment(plan, None, u, v, steps, states, gu, gv, scratch, acc)
    assert rc == _native.CFD_ERR_INVALID_ARGUMENT
    assert 'cfd_fvm_adjoint_segment' in _native.last_error()


def test_plan_rejects_non_power_of_two_before_touching_the_gpu(lib):
  import ctypes
  from jax_cfd_gb300 import _native
  cfg = _native.FvmConfig()
  cfg.nx, cfg.ny, cfg.hx, cfg.hy, cfg.density, cfg.dt = 100, 100, 0.1, 0.1, 1.0, 1e-3
  handle = ctypes.c_void_p()
  rc = lib.cfd_fvm_plan_create(ctypes.byref(cfg), ctypes.byref(handle))
  assert rc == _native.CFD_ERR_UNSUPPORTED
  assert 'powers of two' in _native.last_error()


def _grid(n=64):
  import jax_cfd_gb300.base as cfd
  return cfd.grids.Grid((n, n), domain=((0, 2 * np.pi), (0, 2 * np.pi)))


def test_grid_geometry_matches_reference_conventions():
  from oracle import fvm
  g = _grid()
  og = fvm.Grid.make((64, 64), domain=((0, 2 * np.pi), (0, 2 * np.pi)))
  assert g.step == og.step
  assert g.cell_faces == ((1.0, 0.5), (0.5, 1.0))
  for a, b in zip(g.mesh_numpy(g.cell_faces[0]), og.mesh(og.cell_faces[0])):
    np.testing.assert_array_equal(a, b)
  for a, b in zip(g.rfft_axes_numpy(), (fvm.fftfreq(64, g.step[0]), fvm.rfftfreq(64, g.step[1]))):
    np.testing.assert_array_equal(a, b)


def test_kolmogorov_descriptor_matches_oracle_field():
  import jax_cfd_gb300.base as cfd
  from jax_cfd_gb300 import _native
  from oracle import fvm
  g = _grid()
  og = fvm.Grid.make((64, 64), domain=((0, 2 * np.pi), (0, 2 * np.pi)))
  f = cfd.forcings.simple_turbulence_forcing(g, 1, 4, -0.1)
  assert f.linear == -0.1 and f.const_kind == _native.FORCE_U_OF_Y
  want_u = fvm.kolmogorov_forcing(og, 1, 4)(None)[0]
  np.testing.assert_array_equal(np.broadcast_to(f.const_u[None, :], (64, 64)), want_u)
  spec = cfd.forcings.kolmogorov_forcing(g, k=4, offsets=((0, 0), (0, 0)))
  fu, fv = spec.constant_fields()
  np.testing.assert_array_equal(fu, fvm.kolmogorov_forcing(og, k=4, offsets=((0, 0), (0, 0)))(None)[0])
  assert fv is None


def test_unsupported_options_raise_not_implemented():
  import jax_cfd_gb300.base as cfd
  g = _grid()
  with pytest.raises(NotImplementedError):
    cfd.equations.semi_implicit_navier_stokes(1.0, 1e-3, 1e-3, g, convect=lambda v: v)
  with pytest.raises(NotImplementedError):
    cfd.equations.semi_implicit_navier_stokes(1.0, 1e-3, 1e-3, g,
                                              pressure_solve=cfd.pressure.solve_cg)
  five = cfd.time_stepping.ButcherTableau(a=[[1], [0, 1], [0, 0, 1], [0, 0, 0, 1]],
                                          b=[0.2] * 5)
  with pytest.raises(NotImplementedError):
    cfd.equations.semi_implicit_navier_stokes(
        1.0, 1e-3, 1e-3, g,
        time_stepper=lambda eq, dt: cfd.time_stepping.navier_stokes_rk(five, eq, dt))
  with pytest.raises(NotImplementedError):
    cfd.equations.semi_implicit_navier_stokes(1.0, 1e-3, 1e-3, g, diffuse=lambda c, nu: c)
  three = cfd.forcings.sum_forcings(cfd.forcings.linear_forcing(g, 1.0),
                                    cfd.forcings.linear_forcing(g, 2.0),
                                    cfd.forcings.kolmogorov_forcing(g))
  with pytest.raises(NotImplementedError):
    cfd.equations.semi_implicit_navier_stokes(1.0, 1e-3, 1e-3, g, forcing=three)


def test_step_function_is_built_without_gpu_work():
  import jax_cfd_gb300.base as cfd
  g = _grid()
  step = cfd.equations.semi_implicit_navier_stokes(
      1.0, 1e-3, 1e-3, g, forcing=cfd.forcings.simple_turbulence_forcing(g, 1, 4, -0.1))
  assert isinstance(step, cfd.equations.FvmStep)
  assert cfd.funcutils.repeated(step, 3).gb300_steps == 3


def test_stable_time_step_raises_like_reference():
  import jax_cfd_gb300.base as cfd
  g = _grid(2048)
  assert abs(cfd.equations.stable_time_step(2.0, 0.5, 1e-3, g) - 7.66990e-4) < 1e-9
  with pytest.raises(ValueError):
    cfd.equations.stable_time_step(2.0, 0.5, 1.0, g)


def test_repeated_and_trajectory_host_semantics():
  import jax_cfd_gb300.base as cfd
  f = lambda x: x + 1
  assert cfd.funcutils.repeated(f, 5)(torch.zeros(2)).tolist() == [5.0, 5.0]
  final, frames = cfd.funcutils.trajectory(f, 3)(torch.zeros(2))
  assert final.tolist() == [3.0, 3.0]
  assert frames[:, 0].tolist() == [1.0, 2.0, 3.0]
  _, frames = cfd.funcutils.trajectory(f, 3, start_with_input=True)(torch.zeros(2))
  assert frames[:, 0].tolist() == [0.0, 1.0, 2.0]


def test_brick_wall_filter_mirror():
  from jax_cfd_gb300.base import grids
  from jax_cfd_gb300.spectral import utils as su
  from oracle import fvm
  from oracle import spectral as ospec
  for n in (64, 128):
    g = grids.Grid((n, n))
    got = su.brick_wall_filter_2d(g, device='cpu').numpy()
    np.testing.assert_array_equal(got, ospec.brick_wall_filter_2d(fvm.Grid.make((n, n))))


def test_other_tableaux_build_rk_steps():
  import jax_cfd_gb300.base as cfd
  g = _grid()
  for stepper, stages in ((cfd.time_stepping.midpoint_rk2, 2), (cfd.time_stepping.heun_rk2, 2),
                          (cfd.time_stepping.classic_rk4, 4)):
    step = cfd.equations.semi_implicit_navier_stokes(1.0, 1e-3, 1e-3, g, time_stepper=stepper)
    assert isinstance(step, cfd.equations.FvmStep)
    assert len(step.tableau[1]) == stages
  euler = cfd.equations.semi_implicit_navier_stokes(1.0, 1e-3, 1e-3, g)
  assert euler.tableau is None


def test_launch_choice_names_follow_the_abi_encoding():
  """FvmPlan.describe_launch decodes the index cfd_fvm_plan_autotune reports
  (row shape + 2 * column scheme + 12 * stencil + 24 * row feed + 48 * rows
  per stencil warp)."""
  from jax_cfd_gb300 import plans
  P = plans.FvmPlan
  seen = set()
  for c in range(P.LAUNCH_CHOICES):
    d = P.describe_launch(c)
    key = (P.ROW_BLOCKS.index(d['row_blocks']), P.COLUMN_PASSES.index(d['column_pass']),
           P.STENCILS.index(d['stencil']), P.ROW_FEEDS.index(d['row_feed']),
           P.STREAM_ROWS.index(d['stream_rows']))
    assert key[0] + 2 * key[1] + 12 * key[2] + 24 * key[3] + 48 * key[4] == c
    seen.add(key)
  assert len(seen) == P.LAUNCH_CHOICES
  assert P.describe_launch(19) == {'row_blocks': 'narrow', 'column_pass': 'pipelined4',
                                   'stencil': 'warp_streams', 'row_feed': 'registers',
                                   'stream_rows': 16}
  assert P.describe_launch(23)['column_pass'] == 'pipelined4_tma'
  assert P.describe_launch(23 + 96)['stream_rows'] == 32
  with pytest.raises(ValueError):
    P.describe_launch(P.LAUNCH_CHOICES)
  header = (ROOT / 'include' / 'cfd_gb300.h').read_text()
  assert f'{P.LAUNCH_CHOICES} choices' in header


def _zero_velocity(grid):
  from jax_cfd_gb300.base import boundaries, grids
  offsets = (np.eye(2) + np.ones((2, 2))) / 2.
  bc = boundaries.periodic_boundary_conditions(2)
  return tuple(grids.GridVariable(grids.GridArray(torch.zeros(grid.shape), tuple(o), grid), bc)
               for o in offsets)


@pytest.mark.parametrize('name,kwargs', [
    ('taylor_green_forcing', dict(scale=1.0, k=2)),
    ('kolmogorov_forcing', dict(scale=1.0, k=2)),
    ('linear_forcing', dict(coefficient=2.0)),
    ('no_forcing', {}),
    ('simple_turbulence_forcing', dict(constant_magnitude=0.0, constant_wavenumber=2,
                                       linear_coefficient=0.0, forcing_type='kolmogorov')),
])
def test_forcing_offsets_and_grid_match_velocity(name, kwargs):
  """forcings_test.py:39-79 (2-D): each forcing's components carry the
  offset and grid of the velocity component they act on."""
  from jax_cfd_gb300.base import forcings, grids
  g = grids.Grid((16, 16))
  v = _zero_velocity(g)
  force = getattr(forcings, name)(g, **kwargs)(v)
  for f, u in zip(force, v):
    assert tuple(float(o) for o in f.offset) == tuple(float(o) for o in u.offset)
    assert f.grid == u.grid
    assert tuple(f.data.shape) == tuple(u.data.shape)
    assert torch.equal(0 * f.data, u.data)


def test_sum_forcings_with_no_forcing_is_exact():
  """forcings_test.py:81-91."""
  from jax_cfd_gb300.base import forcings, grids
  g = grids.Grid((16, 16))
  v = _zero_velocity(g)
  f1 = forcings.kolmogorov_forcing(g, scale=1.0, k=2)
  total = forcings.sum_forcings(f1, forcings.no_forcing(g))(v)
  for a, b in zip(total, f1(v)):
    assert torch.equal(a.data, b.data)
