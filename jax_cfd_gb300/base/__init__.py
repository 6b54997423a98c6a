"""Mirror of ``jax_cfd.base`` for the GB300 hot path."""
from jax_cfd_gb300.base import grids  # noqa: F401
from jax_cfd_gb300.base import boundaries  # noqa: F401
from jax_cfd_gb300.base import finite_differences  # noqa: F401
from jax_cfd_gb300.base import advection  # noqa: F401
from jax_cfd_gb300.base import diffusion  # noqa: F401
from jax_cfd_gb300.base import pressure  # noqa: F401
from jax_cfd_gb300.base import time_stepping  # noqa: F401
from jax_cfd_gb300.base import forcings  # noqa: F401
from jax_cfd_gb300.base import equations  # noqa: F401
from jax_cfd_gb300.base import funcutils  # noqa: F401
from jax_cfd_gb300.base import initial_conditions  # noqa: F401
