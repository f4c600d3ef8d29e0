"""Shared helpers of the test suite (fixtures, norms)."""
import ast
import os

import numpy as np

import mpaso

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FCT_KEYS = ("maxLevelCell", "maxLevelEdgeTop", "nAdvCellsForEdge", "advCellsForEdge",
            "highOrderAdvMask", "meshScalingDel2", "edgeSignOnCell", "derivTwo", "advCoef",
            "advCoef_3rd")


class Golden:
    def __init__(self, name):
        z = np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False)
        self.d = {k: z[k] for k in z.files}
        case = self.d["case"]
        self.name, self.app = str(case[0]), str(case[1])
        self.L, self.T = int(case[2]), int(case[3])
        self.opts = ast.literal_eval(str(case[4]))
        self.dt = float(case[5])
        self.steps = ast.literal_eval(str(case[6]))
        self.mesh = mpaso.Mesh.from_dict(self.d)
        self.fct = ({k: self.d["fct_" + k] for k in FCT_KEYS} if "fct_advCoef" in self.d else None)

    def __getitem__(self, k):
        return self.d[k]


def golden_names():
    return sorted(f[:-4] for f in os.listdir(GOLDEN) if f.endswith(".npz"))


def rel_max(a, b):
    """Normwise relative max error max|a-b| / max|b| (the parity metric of the tests)."""
    a, b = np.asarray(a), np.asarray(b)
    den = np.abs(b).max()
    return float(np.abs(a - b).max() / (den if den > 0 else 1.0))


def have_gpu():
    try:
        from mpaso.gpu import device_count
        return device_count() > 0
    except Exception:
        return False


def _ocean_slice(args):
    """Oracle ocean run of one block of levels (a spawned worker)."""
    import sys
    level, f, opts, dt, nsteps, h, hE, u, tr, oracle_dir = args
    if oracle_dir not in sys.path:
        sys.path.insert(0, oracle_dir)
    from oracle import Oracle
    mesh = mpaso.Mesh.icosa(level)
    S = Oracle("restatement")
    L, T = h.shape[1], tr.shape[2]
    return S.ocean_run(mesh, S.static(mesh, f), S.config(L, T, **opts), dt, nsteps, h, hE, u, tr)


def ocean_oracle_by_levels(level, f, opts, dt, nsteps, h, hE, u, tr, blocks):
    """The oracle's ocean run (apps/ocean/run.cc:10-50) on a level-`level`
    sphere, computed as `blocks` blocks of levels in parallel processes.  The
    ocean app couples no levels (every task's level loop is independent) and
    full columns give every level the same statics, so each block runs as a
    column of its own levels with the statics cut to them -- identical to the
    whole run value for value."""
    import multiprocessing as mp
    L = h.shape[1]
    edges = np.linspace(0, L, blocks + 1).astype(int)
    jobs = []
    for a, b in zip(edges[:-1], edges[1:]):
        fs = dict(f)
        fs["maxLevelCell"] = np.full_like(f["maxLevelCell"], b - a)
        fs["maxLevelEdgeTop"] = np.full_like(f["maxLevelEdgeTop"], b - a)
        fs["highOrderAdvMask"] = np.ascontiguousarray(f["highOrderAdvMask"][:, a:b])
        cut = lambda x: np.ascontiguousarray(x[:, a:b])  # noqa: E731
        jobs.append((level, fs, opts, dt, nsteps, cut(h), cut(hE), cut(u), cut(tr),
                     os.path.join(os.path.dirname(GOLDEN), "..", "oracle")))
    with mp.get_context("spawn").Pool(min(blocks, os.cpu_count() or 1)) as pool:
        parts = pool.map(_ocean_slice, jobs)
    return np.concatenate(parts, axis=1)


def extremum_distance(mesh, x):
    """Rings from every cell to the nearest local extremum of the cell field x
    (a cell whose value is >= or <= all of its neighbours'), by breadth-first
    search over cellsOnCell."""
    f = mesh.fields
    coc = f["cellsOnCell"] - 1
    n = f["nEdgesOnCell"]
    valid = np.arange(coc.shape[1])[None, :] < n[:, None]
    nb = np.where(valid, coc, np.arange(mesh.nCells)[:, None])
    ext = np.all(x[:, None] >= x[nb], axis=1) | np.all(x[:, None] <= x[nb], axis=1)
    dist = np.full(mesh.nCells, -1, np.int64)
    front = np.flatnonzero(ext)
    dist[front] = 0
    d = 0
    while front.size:
        d += 1
        cand = np.unique(nb[front][valid[front]])
        cand = cand[dist[cand] < 0]
        dist[cand] = d
        front = cand
    return dist
