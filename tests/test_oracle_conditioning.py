"""Conditioning of the reference's Kobayashi step at zero gradient.

The reference takes theta = atan2(phi_y, phi_x) (snowflake/function.h:32).  On
a mirror-symmetric seed the gradient is exactly zero at the centre, where
atan2 is discontinuous: a one-ulp change of one neighbouring value turns
theta from 0 into an arbitrary angle and eps(theta)^2 * lap(phi) changes by
O(delta).  Two correct implementations whose libm differ by one ulp
therefore differ by ~1e-4 there.  This test pins that sensitivity on the
oracle itself; the GPU parity tests use it to set their bar on symmetric seeds.
"""
import numpy as np

import oracle_bind as ob


def test_one_ulp_at_zero_gradient_moves_the_reference_step_by_1e_4():
    n = 64
    phi0, T0 = ob.kob_init_disc(n, n, 32, 32, 30.0)
    q = ob.kob_params(n, n)
    a = ob.kob_run(q, phi0, T0, 10)
    b = a[0].copy()
    b[32, 33] = np.nextafter(b[32, 33], 2.0)
    x = ob.kob_run(q, a[0], a[1], 10)
    y = ob.kob_run(q, b, a[1], 10)
    d = np.abs(x[0] - y[0]).max()
    assert 1e-6 < d < 1e-2, d


def test_noise_breaks_the_symmetry_and_conditioning_recovers():
    n = 64
    phi0, T0 = ob.kob_init_disc(n, n, 32, 32, 30.0)
    q = ob.kob_params(n, n, noise=0.01, seed=5)
    a = ob.kob_run(q, phi0, T0, 10)
    b = a[0].copy()
    b[32, 33] = np.nextafter(b[32, 33], 2.0)
    x = ob.kob_run(q, a[0], a[1], 10, step0=10)
    y = ob.kob_run(q, b, a[1], 10, step0=10)
    assert np.abs(x[0] - y[0]).max() < 1e-13
