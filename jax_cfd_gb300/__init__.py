"""GB300-native drop-in for the time-stepping hot path of jax-cfd 0.2.1.

``jax_cfd_gb300.base`` mirrors ``jax_cfd.base`` (grids, boundaries, equations,
pressure, funcutils, forcings, ...) and ``jax_cfd_gb300.spectral`` mirrors
``jax_cfd.spectral`` for the two hot-path steps: the staggered-grid
``semi_implicit_navier_stokes`` step and the pseudospectral ``NavierStokes2D``
step with ``crank_nicolson_rk4``.  Arrays are torch CUDA tensors; the compute
is hand-written sm_103a CUDA in ``libcfd_gb300.so`` behind the C ABI of
``include/cfd_gb300.h``.
"""
__version__ = '0.1.0'

from jax_cfd_gb300 import base  # noqa: E402,F401
from jax_cfd_gb300 import spectral  # noqa: E402,F401
