"""The device generator's collision draws against the reference's samplers.

Free-running steps draw, per cell, a Gamma(3(N_c-1)/2, 1) variate for the
Maxwell-Boltzmann-scaling thermostat (Marsaglia-Tsang, the method of rgamma,
src/libcilia/mpcd.cpp:13-43) and a uniformly random rotation axis
(generate_collision_matrix, src/libcilia/mpcd.cpp:269-284).  The device
draws them from Philox counters in float arithmetic (24-bit uniforms), the
reference from MT19937 in double, so they are compared as distributions:

  * Gamma: a two-sample Kolmogorov-Smirnov test against the 500 rgamma(N_c)
    samples the reference itself produced (tests/golden/mt.npz, N_c = 2, 5,
    10, 30), p > 1e-3; and the first two moments of 200,000 device draws
    against the Gamma law's (mean = variance = 3(N_c-1)/2) within 5 standard
    errors.
  * Axis: unit length to float64 rounding, cos(theta) and phi uniform
    (one-sample KS against the uniform law, p > 1e-3), mean of the axis
    within 5 standard errors of zero.

The draws are deterministic for a fixed seed, so the test is too.
"""
import numpy as np
import pytest

import cilia_gpu as cg
from conftest import golden

pytestmark = pytest.mark.gpu

stats = pytest.importorskip("scipy.stats")


@pytest.mark.parametrize("nc", [2, 5, 10, 30])
def test_gamma_draws_match_reference_rgamma(nc):
    ref = golden("mt")[f"gamma42_{nc}"]
    g, _ = cg.collision_draws(nc, 200000, seed=12345, step=7, axis=False)
    k = 1.5 * (nc - 1)
    assert np.all(g > 0)
    ks = stats.ks_2samp(g, ref)
    assert ks.pvalue > 1e-3, (nc, ks)
    n = g.size
    assert abs(g.mean() - k) < 5 * np.sqrt(k / n), (nc, g.mean(), k)
    # variance of the sample variance of a Gamma(k): (2k^2 + 6k) / n approximately (mu4 - sigma^4)
    assert abs(g.var() - k) < 5 * np.sqrt((2 * k * k + 6 * k) / n), (nc, g.var(), k)
    # the reference's own samples agree with the same law
    assert abs(ref.mean() - k) < 5 * np.sqrt(k / ref.size)


def test_gamma_draws_differ_by_step_and_cell():
    a, _ = cg.collision_draws(10, 4096, seed=3, step=1, axis=False)
    b, _ = cg.collision_draws(10, 4096, seed=3, step=2, axis=False)
    c, _ = cg.collision_draws(10, 4096, seed=3, step=1, axis=False)
    assert np.array_equal(a, c)
    assert np.mean(a == b) < 0.01
    assert np.unique(a).size > 4000


def test_rotation_axis_uniform_on_the_sphere():
    _, ax = cg.collision_draws(10, 200000, seed=99, step=5, gamma=False)
    r = np.linalg.norm(ax, axis=1)
    assert np.abs(r - 1.0).max() < 1e-15
    ct = ax[:, 2]
    phi = np.arctan2(ax[:, 1], ax[:, 0])
    assert stats.kstest(ct, "uniform", args=(-1.0, 2.0)).pvalue > 1e-3
    assert stats.kstest(phi, "uniform", args=(-np.pi, 2 * np.pi)).pvalue > 1e-3
    # E[r] = 0, Var[r_i] = 1/3
    assert np.abs(ax.mean(axis=0)).max() < 5 * np.sqrt(1.0 / 3.0 / ax.shape[0])
