"""Known answers the reference itself checks, and analytic pins of the terms it
lacks, on the oracle (CPU).  The same cases run through the CUDA path in
tests/test_gpu_rk4.py."""
import numpy as np

import mpaso
from mpaso.setup import fct_statics
from mpaso.testcases import (del2_mode, ocean_case, ocean_case_error, sw_case1, sw_case1_error, sw_case5, sw_case6,
                             sw_invariants)
from oracle import Oracle

# ocean test cases (apps/ocean/tasks/testcase.cc): (dt, days) per icosahedral level
OCEAN_RUN = {1: {3: (1800.0, 1), 4: (900.0, 1)}, 2: {4: (900.0, 1)}, 3: {4: (3600.0, 10), 5: (1800.0, 10)}}


def ocean_run(level, case):
    """The ocean app (apps/ocean/run.cc:10-50) on test case `case` with the oracle;
    FCT advection for the rotating cases, del2 mixing (kappa = 1e7, as
    apps/ocean/initialize.cc:79 sets) for the diffusing one."""
    S = Oracle("restatement")
    m = mpaso.Mesh.icosa(level)
    h, u, tr = ocean_case(m, case)
    dt, days = OCEAN_RUN[case][level]
    n = int(round(days * 86400.0 / dt))
    cfg = S.config(1, 1, fct=True) if case in (1, 2) else S.config(1, 1, hmix=True, kappa=1e7)
    out = S.ocean_run(m, S.static(m, fct_statics(m, 1)), cfg, dt, n, h, np.ones((m.nEdges, 1)), u, tr)
    return m, tr, out, n * dt


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


def test_ocean_case3_diffusion_decays_at_6_kappa_over_a2():
    """Ocean case 3: a degree-2 spherical harmonic under del2 mixing decays as
    exp(-6 kappa t / a^2); after 10 days the pointwise relative error is 3e-4
    at level 4 and falls ~4x per level (second order), the l2 norm ~8x."""
    m4, _, out4, t4 = ocean_run(4, 3)
    l2_4, mx4 = ocean_case_error(m4, 3, out4, t4)
    m5, _, out5, t5 = ocean_run(5, 3)
    l2_5, mx5 = ocean_case_error(m5, 3, out5, t5)
    assert l2_4 < 4e-6 and mx4 < 4e-4
    assert mx5 < 0.3 * mx4 and l2_5 < 0.2 * l2_4


def test_ocean_case1_gaussian_hill_one_rotation():
    """Ocean case 1: a Gaussian hill carried once round the sphere by FCT advection
    comes back with a relative l2 error that shrinks with resolution, no overshoot
    of its initial maximum and an undershoot of the background below 0.05%."""
    errs = {}
    for level in (3, 4):
        m, tr0, out, t = ocean_run(level, 1)
        errs[level] = ocean_case_error(m, 1, out, t)[0]
        assert out.max() <= tr0.max() and out.min() > 50.0 * (1 - 2e-3)
    assert errs[4] < 5e-4 and errs[4] < 0.5 * errs[3]


def test_ocean_case2_slotted_cylinder_stays_in_range():
    """Ocean case 2: the slotted cylinder (values 50 and 100) after one rotation:
    the FCT limiter keeps it inside [50, 100] up to a 0.2% undershoot of the
    background (the prescribed unit thickness is not the provisional thickness
    the limiter bounds against), and the l2 error stays below 2.5e-3."""
    m, tr0, out, t = ocean_run(4, 2)
    assert out.max() <= 100.0 and out.min() > 50.0 * (1 - 2e-3)
    assert ocean_case_error(m, 2, out, t)[0] < 2.5e-3


def sw_case_run(case, level=4, dt=600.0, n=144):
    """One day of sw case 5 (with its two cone tracers, FCT) or 6 on the oracle."""
    S = Oracle("restatement")
    m = mpaso.Mesh.icosa(level)
    if case == 6:
        h, u = sw_case6(m)
        hs, tr, T, st, opts = None, np.zeros((m.nCells, 1, 0)), 0, S.static(m), {}
    else:
        h, u, hs, tr = sw_case5(m)
        T, st, opts = 2, S.static(m, fct_statics(m, 1), bottomDepth=hs), {"fct": True}
    out = S.sw_run(m, st, S.config(1, T, **opts), dt, n, h, u, tr)
    return m, (h, u, tr, hs), out


def test_sw_case6_rossby_haurwitz_conserves_mass_and_energy():
    """Case 6 for a day at level 4: mass to roundoff, total energy to 1e-6 (TRiSK
    conserves energy in space; RK4 in time loses 6.5e-8 here)."""
    m, (h, u, _, _), (hn, un, _) = sw_case_run(6)
    i0, i1 = sw_invariants(m, h, u), sw_invariants(m, hn, un)
    assert abs(i1["mass"] / i0["mass"] - 1) < 1e-14
    assert abs(i1["energy"] / i0["energy"] - 1) < 1e-6


def test_sw_case5_mountain_conserves_mass_tracers_and_bounds():
    """Case 5 for a day at level 4 with its two cone tracers under FCT: mass and
    tracer mass to roundoff, energy to 1e-7, tracers inside their initial range
    up to 1e-6 (the limiter bounds against the full-dt provisional thickness, the
    RK substeps use fractions of dt)."""
    m, (h, u, tr, hs), (hn, un, trn) = sw_case_run(5)
    i0, i1 = sw_invariants(m, h, u, tr, hs), sw_invariants(m, hn, un, trn, hs)
    assert abs(i1["mass"] / i0["mass"] - 1) < 1e-14
    assert np.all(np.abs(i1["tracer_mass"] / i0["tracer_mass"] - 1) < 1e-13)
    assert abs(i1["energy"] / i0["energy"] - 1) < 1e-7
    assert trn.min() > -1e-6 and trn.max() <= tr.max()
