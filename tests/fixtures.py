"""Loading the golden vectors of tests/golden/ and comparing states."""
import glob
import os

import numpy as np

from picpp_gb300 import initstate as I

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden_names(prefix=""):
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, prefix + "*.npz")))


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    nx, ny, nz = (int(v) for v in z["box"])
    dx, dy, dz, dt, theta, eta, cfix = (float(v) for v in z["params"])
    box = I.Box(nx, ny, nz, dx, dy, dz, dt, theta, eta, cfix)
    species, out = [], []
    for s in range(int(z["nspecies"])):
        q, m, w = (float(v) for v in z[f"s{s}_qmw"])
        sp = dict(q=q, m=m, w=w)
        for k in ("cell", "ox", "oy", "oz", "px", "py", "pz"):
            sp[k] = z[f"s{s}_{k}"].copy()
        species.append(sp)
        out.append({k: z[f"s{s}_out_{k}"].copy() for k in ("x", "y", "z", "px", "py", "pz")})
    st = I.State(box, species, z["E0"].copy(), z["B0"].copy())
    extra = {k[2:]: z[k].copy() for k in z.files if k.startswith("x_")}
    return dict(state=st, solver=int(z["solver"]), steps=int(z["steps"]), out=out,
                E=z["E"].copy(), B=z["B"].copy(), extra=extra)


def smoothing_of(f):
    """(smoothingCount, smoothingParameter) a golden case was run with."""
    sm = f["extra"].get("smoothing")
    return (int(sm[0]), float(sm[1])) if sm is not None else (0, 0.5)


def copy_species(species):
    return [{k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in s.items()} for s in species]


def rel_err(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    scale = max(float(np.max(np.abs(b))), 1e-300)
    return float(np.max(np.abs(a - b))) / scale


def periodic_dist(a, b, L):
    d = np.asarray(a) - np.asarray(b)
    return np.abs((d + L / 2) % L - L / 2)


def wall_of(f):
    """(wall_x, e_right, b_right) of a golden case (the reflecting-wall
    cases carry the open boundary's fields; the others are periodic)."""
    w = f["extra"].get("wall")
    if w is None:
        return 0, (0.0, 0.0, 0.0), (0.0, 0.0, 0.0)
    return 1, tuple(float(v) for v in w[:3]), tuple(float(v) for v in w[3:6])


def survivors(out):
    """Indices of the particles a reference run kept (escaped ones come back
    as NaN)."""
    return np.nonzero(~np.isnan(np.asarray(out["x"])))[0]


def yee_physical(a, box, field):
    """The physical part of a staggered Yee field ("E" or "B") of a wall box,
    as one flat array: x-cell-centred components (Ex; By, Bz) on cells
    0 .. nx - 3, x-node components (Ey, Ez; Bx) on nodes 0 .. nx - 2."""
    a = np.asarray(a).reshape(3, box.nz, box.ny, box.nx)
    cells = (0,) if field == "E" else (1, 2)
    return np.concatenate([a[c, ..., : box.nx - (2 if c in cells else 1)].ravel() for c in range(3)])
