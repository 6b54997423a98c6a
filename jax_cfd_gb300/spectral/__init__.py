"""Mirror of ``jax_cfd.spectral`` for the GB300 hot path."""
from jax_cfd_gb300.spectral import utils  # noqa: F401
from jax_cfd_gb300.spectral import equations  # noqa: F401
from jax_cfd_gb300.spectral import time_stepping  # noqa: F401
