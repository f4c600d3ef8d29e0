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
