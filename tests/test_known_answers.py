"""Known answers the reference itself checks, and analytic pins of the terms it
lacks, on the oracle (CPU).  The same cases run through the CUDA path in
tests/test_gpu_rk4.py."""
import numpy as np

import mpaso
from mpaso.testcases import del2_mode, sw_case1, sw_case1_error
from oracle import Oracle


def test_sw_case1_error_within_reference_tolerance():
    """Williamson case 1 on a 240 km sphere (level 5), 5 steps of dt = 40 s: the
    reference's ctest and its 0.0015 bound (apps/sw/finalize.cc:24-25)."""
    S = Oracle("restatement")
    m = mpaso.Mesh.icosa(5)
    h, u = sw_case1(m)
    assert sw_case1_error(m, h, 0.0) == 0.0
    h5, u5, _ = S.sw_run(m, S.static(m), S.config(1, 0, pin_u=True), 40.0, 5, h, u, np.zeros((m.nCells, 1, 0)))
    assert np.array_equal(u5, u)  # the wind stays pinned
    assert sw_case1_error(m, h5, 200.0) <= 0.0015


def test_del2_momentum_decays_a_fourier_mode_at_nu_k2():
    """u = curl(sin(k x)) at 1e-6 m/s on an f = 0 plane with uniform h decays as
    exp(-nu k^2 t): the discrete rate is within 1% of nu k^2 and h stays uniform."""
    S = Oracle("restatement")
    m = mpaso.Mesh.hex(32, 32, 10e3, 0.0)
    h, u, pattern, k2 = del2_mode(m)
    nu, dt, n = 1e5, 30.0, 100
    hn, un, _ = S.sw_run(m, S.static(m), S.config(1, 0, nu=nu), dt, n, h, u, np.zeros((m.nCells, 1, 0)))
    a = float((un[:, 0] * pattern).sum() / (pattern * pattern).sum()) / 1e-6
    assert abs(-np.log(a) / (nu * dt * n) / k2 - 1) < 0.01
    assert np.abs(hn - h).max() < 1e-9
    # dissipative: with nu = 0 the mode keeps its amplitude
    _, u0, _ = S.sw_run(m, S.static(m), S.config(1, 0, nu=0.0), dt, n, h, u, np.zeros((m.nCells, 1, 0)))
    assert abs(float((u0[:, 0] * pattern).sum() / (pattern * pattern).sum()) / 1e-6 - 1) < 1e-6
