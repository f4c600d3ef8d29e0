"""Generates the golden fixtures in tests/golden/ from the reference itself.

The reference's own task sources (apps/sw/tasks/solve.cc, apps/ocean/tasks/
solve.cc, apps/ocean/tasks/init_functions.cc), compiled unmodified through
oracle/shim/ (python oracle/build.py), are run on small generated meshes.
Each fixture stores everything a test needs to rerun the case anywhere --
the mesh datasets, the FCT statics computed by the reference's
init_functions.cc, the initial state -- and the reference's outputs.

Usage (needs the reference checkout, i.e. oracle/_ref/ built):
    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "mpas-o-flecsi-2.0_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import mpaso  # noqa: E402
from mpaso.initial import ocean_state, sw_state  # noqa: E402
from oracle import Oracle  # noqa: E402

CASES = [
    # name, mesh, app, L, T, options, dt, (steps...)
    ("sw_fct_icosa3_L1T1", ("icosa", 3), "sw", 1, 1,
     dict(fct=True, hmix=True, kappa=1e4, nu=1e4), 300.0, (1, 10)),
    ("sw_scalar_icosa3_L3T2", ("icosa", 3), "sw", 3, 2, dict(), 300.0, (1, 10)),
    ("sw_fct_icosa2_L5T5", ("icosa", 2), "sw", 5, 5,
     dict(fct=True, hmix=True, kappa=1e5, nu=0.0), 600.0, (1, 5)),
    ("ocean_icosa3_L3T2", ("icosa", 3), "ocean", 3, 2, dict(fct=True, hmix=True, kappa=1e4),
     600.0, (1, 10)),
    ("sw_hex16_L1T1", ("hex", 16, 16, 10e3), "sw", 1, 1, dict(nu=1e3), 30.0, (1, 10)),
]


def make_mesh(spec):
    if spec[0] == "icosa":
        return mpaso.Mesh.icosa(spec[1])
    return mpaso.Mesh.hex(spec[1], spec[2], spec[3], 1e-4)


def main():
    for name, spec, app, L, T, opts, dt, steps in CASES:
        R = Oracle("ref", L, T)
        mesh = make_mesh(spec)
        out = mesh.to_dict()
        fct = R.fct_statics(mesh, L, cfg=R.config(L, T)) if mesh.on_sphere else None
        if fct is not None:
            out.update({"fct_" + k: v for k, v in fct.items()})
        cfg = R.config(L, T, **opts)
        st = R.static(mesh, fct)
        if app == "sw":
            h, u, tr = sw_state(mesh, 1234, L, T)
            out.update(h0=h, u0=u, tr0=tr)
            for n in steps:
                h1, u1, tr1 = R.sw_run(mesh, st, cfg, dt, n, h, u, tr)
                out[f"h_{n}"], out[f"u_{n}"], out[f"tr_{n}"] = h1, u1, tr1
        else:
            h, hE, u, tr = ocean_state(mesh, 1234, L, T)
            out.update(h0=h, hE0=hE, u0=u, tr0=tr)
            for n in steps:
                out[f"tr_{n}"] = R.ocean_run(mesh, st, cfg, dt, n, h, hE, u, tr)
        out["case"] = np.array([name, app, str(L), str(T), repr(opts), repr(dt), repr(steps)])
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **out)
        print(path, os.path.getsize(path))


if __name__ == "__main__":
    main()
