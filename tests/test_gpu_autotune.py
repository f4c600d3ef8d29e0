"""Launch-configuration variants and the per-mesh autotuner (GPU).

Every launch variant of the stage kernels (stencil unrolled at compile time or
not; 64/128/256 threads per block) must reproduce the reference goldens at the
one-step parity bar of the fused path (relative max-norm 1e-12).  Block size
does not change any thread's arithmetic, so two configurations differing only
in threads per block agree bit for bit.  The autotuner restores the state it
timed on, bit for bit."""
import numpy as np
import pytest

from helpers import Golden, golden_names, rel_max
from test_gpu_rk4 import make_state

pytestmark = pytest.mark.gpu
TOL1 = 1e-12

CONFIGS = [([1, 1, 1], [256, 256, 256], [0, 0, 0], 0, 1, 0), ([0, 0, 0], [256, 256, 256], [1, 1, 1], 1, 0, 1),
           ([1, 1, 1], [64, 128, 64], [1, 0, 1], 2, 1, 1), ([0, 1, 0], [128, 64, 256], [0, 1, 0], 1, 0, 0),
           ([1, 1, 1], [128, 128, 128], [0, 0, 0], 0, 0, 1)]


def _fields(st, app):
    import mpaso.gpu as G
    out = [st.get(G.FIELD_TRACERS)]
    if app == "sw":
        out += [st.get(G.FIELD_H), st.get(G.FIELD_U)]
    return out


@pytest.mark.parametrize("name", golden_names())
@pytest.mark.parametrize("cfg", range(len(CONFIGS)))
def test_every_launch_variant_matches_goldens(name, cfg):
    g = Golden(name)
    dm, st = make_state(g)
    st.set_launch_config(*CONFIGS[cfg])
    got_cfg = st.launch_config()
    assert {k: got_cfg[k] for k in ("unroll", "threads", "capped")} == {
        "unroll": CONFIGS[cfg][0], "threads": CONFIGS[cfg][1], "capped": CONFIGS[cfg][2]}
    assert got_cfg["l2"] in (0, CONFIGS[cfg][3])  # 0 where the state has no such array
    assert got_cfg["overlap"] == CONFIGS[cfg][4]
    assert got_cfg["split"] == (CONFIGS[cfg][5] if g.app == "sw" and g.T > 0 else 0)
    st.step_graph(g.dt, 1)
    got = _fields(st, g.app)
    want = [g["tr_1"]] + ([g["h_1"], g["u_1"]] if g.app == "sw" else [])
    for a, b in zip(got, want):
        assert rel_max(a, b) < TOL1
    st.close()
    dm.close()


@pytest.mark.parametrize("name", golden_names())
@pytest.mark.parametrize("lanes", [2, 4])
def test_lanes_per_edge_match_goldens(name, lanes):
    """2 or 4 threads per edge-level in the TRiSK loop (sw app, at most one
    tracer) keep the one-step parity bar; elsewhere the choice is refused."""
    from mpaso._lib import MpasoError
    g = Golden(name)
    dm, st = make_state(g)
    if g.app != "sw" or g.T > 1:
        with pytest.raises(MpasoError):
            st.set_launch_config([1, 1, 1], [256, 256, 256], lanes=lanes)
        return
    st.set_launch_config([1, 1, 1], [128, 128, 128], lanes=lanes)
    assert st.launch_config()["lanes"] == lanes
    st.step_graph(g.dt, 1)
    for a, b in zip(_fields(st, g.app), [g["tr_1"], g["h_1"], g["u_1"]]):
        assert rel_max(a, b) < TOL1
    st.close()
    dm.close()


@pytest.mark.parametrize("name", golden_names())
def test_block_size_is_bitwise_neutral(name):
    g = Golden(name)
    res = []
    for threads in ([256, 256, 256], [64, 128, 64]):
        dm, st = make_state(g)
        st.set_launch_config([1, 1, 1], threads)
        st.step(g.dt, 3)
        res.append(_fields(st, g.app))
        st.close()
        dm.close()
    for a, b in zip(*res):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("name", ["sw_fct_icosa3_L1T1", "ocean_icosa3_L3T2"])
def test_autotune_restores_state_and_keeps_parity(name):
    g = Golden(name)
    dm, st = make_state(g)
    before = _fields(st, g.app)
    st.step_graph(g.dt, 0)  # captures a step graph with the default launch shapes
    cfg = st.autotune(g.dt, 2)
    assert all(b in (64, 128, 256) for b in cfg["threads"]) and all(u in (0, 1) for u in cfg["unroll"])
    assert all(o in (0, 1) for o in cfg["capped"]) and cfg["l2"] in (0, 1, 2) and cfg["overlap"] in (0, 1)
    assert cfg["split"] in (0, 1)
    assert st.launch_config() == cfg
    for a, b in zip(_fields(st, g.app), before):
        assert np.array_equal(a, b)
    st.step_graph(g.dt, 1)
    want = [g["tr_1"]] + ([g["h_1"], g["u_1"]] if g.app == "sw" else [])
    for a, b in zip(_fields(st, g.app), want):
        assert rel_max(a, b) < TOL1
    st.close()
    dm.close()


def test_bad_launch_config_is_rejected():
    import mpaso
    g = Golden("sw_hex16_L1T1")
    dm, st = make_state(g)
    with pytest.raises(mpaso.MpasoError) as e:
        st.set_launch_config([1, 1, 1], [256, 512, 256])
    assert e.value.code == 1
    with pytest.raises(mpaso.MpasoError):
        st.set_launch_config([2, 1, 1], [256, 256, 256])
    with pytest.raises(mpaso.MpasoError):
        st.set_launch_config([1, 1, 1], [256, 256, 256], [0, 3, 0])
    with pytest.raises(mpaso.MpasoError):
        st.set_launch_config([1, 1, 1], [256, 256, 256], [0, 0, 0], 5)
    assert st.launch_config()["threads"] == [256, 256, 256]
    st.close()
    dm.close()


@pytest.mark.parametrize("mode", [0, 1, 2, 3])
def test_every_ordering_matches_goldens(mode):
    """Each numbering of the device mesh (file order, Hilbert cells with edges and
    vertices after them, Hilbert curve per entity, Morton cells) reproduces the
    reference goldens at the one-step bar and keeps the permutation a bijection."""
    import mpaso.gpu as G
    g = Golden("sw_fct_icosa3_L1T1")
    dm = G.DeviceMesh(g.mesh, fct=g.fct, reorder=mode)
    for ent, n in ((0, g.mesh.nCells), (1, g.mesh.nEdges), (2, g.mesh.nVertices)):
        assert np.array_equal(np.sort(dm.permutation(ent)), np.arange(n))
    o = g.opts
    st = G.State(dm, nlev=g.L, ntr=g.T, fct=o.get("fct", False), hmix=o.get("hmix", False),
                 kappa=o.get("kappa", 0.0), nu=o.get("nu", 0.0))
    st.set(G.FIELD_H, g["h0"])
    st.set(G.FIELD_U, g["u0"])
    st.set(G.FIELD_TRACERS, g["tr0"])
    st.step_graph(g.dt, 1)
    for f, k in ((G.FIELD_H, "h_1"), (G.FIELD_U, "u_1"), (G.FIELD_TRACERS, "tr_1")):
        assert rel_max(st.get(f), g[k]) < TOL1


def test_ordering_tuner_picks_a_timed_mode():
    import mpaso.gpu as G
    g = Golden("sw_fct_icosa3_L1T1")
    o = g.opts
    fields = {G.FIELD_H: g["h0"], G.FIELD_U: g["u0"], G.FIELD_TRACERS: g["tr0"]}
    mode, ms, (dm, st), cfg = G.tune_ordering(
        g.mesh, fields, g.dt, fct=g.fct, state_kwargs=dict(nlev=g.L, ntr=g.T, fct=o.get("fct", False),
                                                             hmix=o.get("hmix", False), kappa=o.get("kappa", 0.0),
                                                             nu=o.get("nu", 0.0)), nsteps=5)
    assert set(ms) == {0, 1, 2, 3} and ms[mode] == min(ms.values())
    st.step_graph(g.dt, 1)
    assert rel_max(st.get(G.FIELD_H), g["h_1"]) < TOL1
