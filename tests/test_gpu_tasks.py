"""Per-task entries of the CUDA path against the oracle (GPU).

Every per-task entry mirrors one reference task (apps/sw/tasks/solve.cc,
apps/ocean/tasks/solve.cc).  Its kernels keep the reference's operation
order and rounding, so the comparison is bit for bit (np.array_equal)."""
import numpy as np
import pytest

from helpers import Golden
from oracle import Oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", params=["ocean_icosa3_L3T2", "sw_fct_icosa3_L1T1", "sw_hex16_L1T1"])
def case(request):
    import mpaso.gpu as G
    g = Golden(request.param)
    L, T = g.L, g.T
    dm = G.DeviceMesh(g.mesh, fct=g.fct, reorder=True)
    S = Oracle("restatement")
    rng = np.random.default_rng(5)
    nC, nE, nV = g.mesh.nCells, g.mesh.nEdges, g.mesh.nVertices
    data = dict(
        h=1000.0 + 50 * rng.random((nC, L)), u=rng.standard_normal((nE, L)) * 10,
        tr=rng.random((nC, L, T)), hE=900.0 + 50 * rng.random((nE, L)))
    yield g, dm, S, data
    dm.close()


def test_permutation_roundtrip(case):
    g, dm, S, data = case
    for ent, n in ((0, g.mesh.nCells), (1, g.mesh.nEdges), (2, g.mesh.nVertices)):
        p = dm.permutation(ent)
        assert np.array_equal(np.sort(p), np.arange(n))
        inv = np.empty_like(p)
        inv[p] = np.arange(n, dtype=p.dtype)
        assert np.array_equal(p[inv], np.arange(n))


def test_sw_diagnostics_bit_exact(case):
    g, dm, S, data = case
    L = g.L
    out = dm.sw_compute_solve_diagnostics(L, data["h"], data["u"])
    om, st, cfg = S.mesh(g.mesh), S.static(g.mesh, g.fct), S.config(L, g.T)
    ref = {k: np.zeros_like(v) for k, v in out.items()}
    S.call("sw_compute_solve_diagnostics", om, st, cfg, data["h"], data["u"], ref["h_edge"],
           ref["h_vertex"], ref["circulation"], ref["vorticity"], ref["ke"], ref["pv_edge"], ref["pv_vertex"])
    for k in out:
        assert np.array_equal(out[k], ref[k]), k


def test_sw_tend_bit_exact(case):
    g, dm, S, data = case
    L, rng = g.L, np.random.default_rng(7)
    nC, nE = g.mesh.nCells, g.mesh.nEdges
    he, ke, pve = rng.random((nE, L)) * 1000, rng.random((nC, L)), rng.standard_normal((nE, L)) * 1e-5
    th, tu = dm.sw_compute_tend(L, he, data["h"], data["u"], ke, pve)
    om, st, cfg = S.mesh(g.mesh), S.static(g.mesh, g.fct), S.config(L, g.T)
    rth, rtu = np.zeros_like(th), np.zeros_like(tu)
    S.call("sw_compute_tend", om, st, cfg, he, data["h"], data["u"], ke, pve, rth, rtu)
    assert np.array_equal(th, rth)
    assert np.array_equal(tu, rtu)


def test_sw_scalar_tend_and_elementwise_bit_exact(case):
    g, dm, S, data = case
    L, T = g.L, g.T
    om, st, cfg = S.mesh(g.mesh), S.static(g.mesh, g.fct), S.config(L, T)
    got = dm.sw_compute_scalar_tend(L, T, data["hE"], data["u"], data["tr"])
    ref = np.zeros_like(got)
    S.call("sw_compute_scalar_tend", om, st, cfg, data["hE"], data["u"], data["tr"], ref)
    assert np.array_equal(got, ref)
    rng = np.random.default_rng(3)
    ut, ht, tt = (rng.standard_normal(data["u"].shape), rng.standard_normal(data["h"].shape),
                  rng.standard_normal(data["tr"].shape))
    for pin in (0, 1):
        a = [np.zeros_like(data["u"]), np.zeros_like(data["h"]), np.zeros_like(data["tr"])]
        b = [x.copy() for x in a]
        dm.call("sw_compute_substep", L, T, a[0], data["u"], ut, a[1], data["h"], ht, a[2], data["tr"], tt,
                37.5, pin)
        S.call("sw_compute_substep", om, S.config(L, T, pin_u=bool(pin)), b[0], data["u"], ut, b[1],
               data["h"], ht, b[2], data["tr"], tt, 37.5)
        for x, y in zip(a, b):
            assert np.array_equal(x, y)


def test_ocean_fct_sequence_bit_exact(case):
    g, dm, S, data = case
    if g.fct is None:
        pytest.skip("planar fixture has no FCT statics")
    L, T, dt = g.L, g.T, 600.0
    om, st, cfg = S.mesh(g.mesh), S.static(g.mesh, g.fct), S.config(L, T)
    nC, nE = g.mesh.nCells, g.mesh.nEdges
    z = lambda *s: np.zeros(s)  # noqa: E731
    # GPU sequence
    ntf = z(nE, L)
    dm.call("oc_calc_normal_thickness_flux", L, data["hE"], data["u"], ntf)
    hp, hpi, hni = z(nC, L), z(nC, L), z(nC, L)
    dm.call("oc_calc_provisional_layer_thicknesses", L, data["h"], ntf, hp, hpi, hni, dt)
    lo, ho = z(nE, L, T), z(nE, L, T)
    dm.call("oc_calc_horiz_tracer_advection_flux_mono_low_order", L, T, ntf, data["tr"], lo)
    dm.call("oc_calc_horiz_tracer_advection_flux_mono_high_order", L, T, ntf, data["tr"], ho)
    fi, fo, tend, tmx, tmn = z(nC, L, T), z(nC, L, T), z(nC, L, T), z(nC, L, T), z(nC, L, T)
    dm.call("oc_correct_and_rescale_high_order_mono_horiz_flux", L, T, hpi, data["h"], ntf, lo, data["tr"],
            ho, fi, fo, tend, tmx, tmn, dt)
    tp = z(nC, L, T)
    dm.call("oc_accumulate_horiz_tracer_advection_tend_mono_FCT", L, T, hpi, data["h"], ho, data["tr"], tp,
            tend, dt)
    dm.call("oc_tracer_hmix_del2_tend", L, T, data["hE"], data["tr"], tend, 1e4)
    # oracle sequence
    r = {k: np.zeros_like(v) for k, v in dict(ntf=ntf, hp=hp, hpi=hpi, hni=hni, lo=lo, ho=ho, fi=fi, fo=fo,
                                              tend=tend, tmx=tmx, tmn=tmn, tp=tp).items()}
    S.call("oc_normal_thickness_flux", om, cfg, data["hE"], data["u"], r["ntf"])
    S.call("oc_provisional_layer_thicknesses", om, st, cfg, data["h"], r["ntf"], r["hp"], r["hp"], r["hpi"],
           r["hni"], dt)
    S.call("oc_low_order", om, st, cfg, r["ntf"], data["tr"], r["lo"])
    S.call("oc_high_order", om, st, cfg, r["ntf"], data["tr"], r["ho"])
    S.call("oc_correct_and_rescale", om, st, cfg, r["hpi"], data["h"], r["ntf"], r["lo"], data["tr"], r["ho"],
           r["fi"], r["fo"], r["tend"], r["tmx"], r["tmn"], dt)
    S.call("oc_accumulate_fct", om, st, cfg, r["hpi"], data["h"], r["ho"], data["tr"], r["tp"], r["tend"], dt)
    S.call("oc_hmix_del2", om, st, cfg, data["hE"], data["tr"], r["tend"], 1e4)
    for k, v in dict(ntf=ntf, hp=hp, hpi=hpi, hni=hni, lo=lo, ho=ho, fi=fi, fo=fo, tend=tend, tmx=tmx,
                     tmn=tmn, tp=tp).items():
        assert np.array_equal(v, r[k]), k
    # FCT keeps the provisional tracer inside its local bounds
    span = tmx - tmn
    assert np.all(tp <= tmx + 1e-12 * (1 + span)) and np.all(tp >= tmn - 1e-12 * (1 + span))


def test_sw_accumulate_and_finalize_bit_exact(case):
    """accumulate_update (apps/sw/tasks/solve.cc:317-341) and finalize_timestep
    (solve.cc:344-367) through the C ABI, with and without the pinned wind of
    test case 1."""
    g, dm, S, data = case
    L, T = g.L, g.T
    om = S.mesh(g.mesh)
    rng = np.random.default_rng(11)
    ut, ht, tt = (rng.standard_normal(data["u"].shape), rng.standard_normal(data["h"].shape),
                  rng.standard_normal(data["tr"].shape))
    a = [data["u"].copy(), data["h"].copy(), data["h"][..., None] * data["tr"]]
    b = [x.copy() for x in a]
    dm.call("sw_accumulate_update", L, T, a[0], ut, a[1], ht, a[2], tt, 12.5)
    S.call("sw_accumulate_update", om, S.config(L, T), b[0], ut, b[1], ht, b[2], tt, 12.5)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    u_old = rng.standard_normal(data["u"].shape)
    for pin in (0, 1):
        ga, gb = [x.copy() for x in a], [x.copy() for x in a]
        dm.call("sw_finalize_timestep", L, T, u_old, ga[0], ga[1], ga[2], pin)
        S.call("sw_finalize_timestep", om, S.config(L, T, pin_u=bool(pin)), u_old, gb[0], gb[1], gb[2])
        for x, y in zip(ga, gb):
            assert np.array_equal(x, y), pin
        assert np.array_equal(ga[0], u_old if pin else a[0])


def test_ocean_step_tracers_forward_bit_exact(case):
    """step_tracers_forward (apps/ocean/tasks/solve.cc:368-399) through the C
    ABI: tracersNew += w tend; tracersPrev = tracers + w_sub tend."""
    g, dm, S, data = case
    L, T = g.L, g.T
    om = S.mesh(g.mesh)
    rng = np.random.default_rng(13)
    tend = rng.standard_normal(data["tr"].shape) * 1e-4
    for w, wsub in ((100.0, 300.0), (50.0, 0.0)):
        new_a, prev_a = rng.random(data["tr"].shape), np.zeros_like(data["tr"])
        new_b, prev_b = new_a.copy(), prev_a.copy()
        dm.call("oc_step_tracers_forward", L, T, tend, data["tr"], new_a, prev_a, w, wsub)
        S.call("oc_step_tracers_forward", om, S.config(L, T), tend, data["tr"], new_b, prev_b, w, wsub)
        assert np.array_equal(new_a, new_b)
        assert np.array_equal(prev_a, prev_b)


def test_device_pointers_match_host(case):
    torch = pytest.importorskip("torch")
    g, dm, S, data = case
    L = g.L
    host = dm.sw_compute_solve_diagnostics(L, data["h"], data["u"])
    dev = {k: torch.zeros(v.shape, dtype=torch.float64, device="cuda") for k, v in host.items()}
    h, u = torch.from_numpy(data["h"]).cuda(), torch.from_numpy(data["u"]).cuda()
    torch.cuda.synchronize()  # torch fills on its own stream; the context uses another
    dm.sw_compute_solve_diagnostics(L, h, u, out=dev)
    torch.cuda.synchronize()
    for k in host:
        assert np.array_equal(dev[k].cpu().numpy(), host[k]), k
