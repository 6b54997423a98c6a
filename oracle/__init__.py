"""CPU oracle for the jax-cfd time-stepping hot path (TEST INFRASTRUCTURE ONLY).

This package restates, op for op in NumPy, the arithmetic of the reference
jax-cfd 0.2.1 functions on the hot path:

* ``oracle.fvm``       -- staggered MAC-grid ``semi_implicit_navier_stokes``
  (Van Leer advection via ``advect_van_leer_using_limiters``, explicit
  diffusion, Kolmogorov + linear forcing, ``forward_euler`` and the real-FFT
  ``solve_fast_diag`` projection), plus the interpolation operators the
  reference tests pin.
* ``oracle.spectral``  -- ``spectral.equations.NavierStokes2D`` /
  ``ForcedNavierStokes2D`` with ``crank_nicolson_rk4``.
* ``oracle.initial_conditions`` -- ``filtered_velocity_field`` with a NumPy
  PCG64 noise source (JAX's PRNG bit stream cannot be reproduced here).
* ``oracle.diagnostics`` -- energy spectrum and enstrophy definitions from
  ``jax_cfd/data/xarray_utils.py``.

JAX is not importable where this repository is built or tested, so the oracle
cannot be checked against a live run of the reference.  It is pinned instead
against every known-answer and property test the reference ships for this path
(interpolation 10x10 exact cases, fast-diagonalisation Poisson solves, the
projection's divergence, Taylor-Green analytic decay, the spectral ODE closed
forms); see ``tests/test_oracle_pins.py``.

Dtype semantics follow JAX with ``jax_enable_x64`` off: Python scalars are weakly
typed and are rounded once to the array dtype (NumPy 2's NEP 50 rules give the
same result), so passing float32 arrays reproduces the reference's float32 run
and passing float64 arrays stands in for a ``jax_enable_x64`` run.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg
may import this package; the product library never does.
"""
