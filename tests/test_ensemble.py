"""Ensemble unions (CPU): stepping the disjoint union of uneven meshes gives,
member by member, exactly what stepping each member alone gives."""
import numpy as np

import mpaso
from mpaso.ensemble import build
from mpaso.initial import sw_state
from oracle import Oracle


def test_union_steps_like_its_members():
    specs = [("hex", 8, 6, 20e3, 1e-4), ("icosa", 2), ("hex", 6, 8, 15e3, 1e-4)]
    u, fct, offs, members = build(specs, nlev=1)
    S = Oracle("restatement")
    opts = dict(fct=True, hmix=True, kappa=1e3, nu=1e3)
    states = [sw_state(m, 10 + i, 1, 1) for i, m in enumerate(members)]
    hu, uu, tu = (np.concatenate([s[k] for s in states]) for k in range(3))
    H, U, TR = S.sw_run(u, S.static(u, fct), S.config(1, 1, **opts), 30.0, 3, hu, uu, tu)
    for i, (m, st) in enumerate(zip(members, states)):
        from mpaso.setup import fct_statics
        f = fct_statics(m, 1)
        h, uv, tr = S.sw_run(m, S.static(m, f), S.config(1, 1, **opts), 30.0, 3, *st)
        c0, c1 = offs[i][0], offs[i + 1][0]
        e0, e1 = offs[i][1], offs[i + 1][1]
        assert np.array_equal(H[c0:c1], h) and np.array_equal(U[e0:e1], uv)
        assert np.array_equal(TR[c0:c1], tr)
