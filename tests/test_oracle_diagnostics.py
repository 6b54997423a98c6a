"""The NumPy restatement of the reference's diagnostics (CPU): shell
assignment, Parseval, enstrophy of a known field."""
import numpy as np

from oracle import diagnostics as od

TWO_PI = 2 * np.pi


def _mesh(n):
  h = TWO_PI / n
  x = (np.arange(n) + 1.0) * h
  return np.meshgrid(x, x, indexing='ij'), (h, h)


def test_bins_follow_the_reference_rule():
  bounds, labels = od.shell_bins((64, 64), (TWO_PI / 64,) * 2)
  # k_max = 31 - 0.5 = 30.5 -> round(30.5) = 30 shells labelled 1..30
  np.testing.assert_allclose(labels, np.arange(1, 31))
  np.testing.assert_allclose(bounds, np.arange(1, 32) - 0.5)


def test_single_modes_and_parseval():
  n = 64
  (x, y), step = _mesh(n)
  u = np.cos(3 * x) + 0.5 * np.sin(5 * y)
  v = np.sin(4 * y + 2 * x)
  labels, spec = od.isotropic_energy_spectrum(u, v, step)
  one = 0.5 * 2 * (n * n / 2) ** 2
  np.testing.assert_allclose(spec[2], one)             # |k| = 3
  np.testing.assert_allclose(spec[4], 0.25 * one)      # |k| = 5
  np.testing.assert_allclose(spec[3], one)             # |k| = sqrt(20)
  # Parseval: all energy sits in shells, sum = 0.5 n^2 sum(u^2 + v^2)
  np.testing.assert_allclose(spec.sum(), 0.5 * n * n * (u ** 2 + v ** 2).sum(), rtol=1e-12)


def test_enstrophy_of_a_shear_mode():
  n = 32
  (x, y), step = _mesh(n)
  u = np.sin(y)
  v = np.zeros_like(u)
  w = od.vorticity_2d(u, v, step)
  # forward difference of sin along y: -(sin(y + h) - sin(y)) / h
  np.testing.assert_allclose(w, -(np.roll(u, -1, axis=1) - u) / step[1])
  np.testing.assert_allclose(od.enstrophy_2d(u, v, step), w ** 2 / 2)
