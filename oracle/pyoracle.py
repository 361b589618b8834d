"""ctypes front end of the C oracle (oracle/oracle.c) and of the reference
harness (oracle/ref/harness.cpp).

TEST INFRASTRUCTURE ONLY.  Imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg; never by the product package.
"""
from __future__ import annotations

import ctypes as C
import os
import struct
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_BIN = os.path.join(HERE, "_ref", "picpp_ref")
# PIC++ source directory (PIC++/*.cpp) for the reference build; the
# reference is only built where this environment variable names it.
REF_SRC = os.environ.get("PICPP_REFERENCE_SRC", "")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_lp = C.POINTER(C.c_long)


class Grid(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
                ("tx", C.c_int), ("ty", C.c_int), ("tz", C.c_int),
                ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double), ("dt", C.c_double),
                ("theta", C.c_double), ("eta", C.c_double), ("cfix", C.c_double),
                ("pressure_compat", C.c_int), ("gmres_max_iter", C.c_int), ("gmres_tol", C.c_double),
                ("smoothing_count", C.c_int), ("smoothing_parameter", C.c_double),
                ("wall_x", C.c_int), ("e_right", C.c_double * 3), ("b_right", C.c_double * 3)]


class Particles(C.Structure):
    _fields_ = [("q", C.c_double), ("m", C.c_double), ("w", C.c_double), ("n", C.c_long),
                ("cell", _ip), ("ox", _dp), ("oy", _dp), ("oz", _dp),
                ("px", _dp), ("py", _dp), ("pz", _dp)]


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.check_call(["make", "-s", "-C", HERE, "liboracle.so"])
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        L = _lib
        g = C.POINTER(Grid)
        p = C.POINTER(Particles)
        L.orc_yee_b_half.argtypes = [g, _dp, _dp]
        L.orc_yee_e.argtypes = [g, _dp, _dp, _dp]
        L.orc_boris_push.argtypes = [g, p, _dp, _dp]
        L.orc_zigzag.argtypes = [g, p, _dp]
        L.orc_buneman_step.argtypes = [g, p, C.c_int, _dp, _dp, _dp]
        L.orc_wall_yee_ghosts.argtypes = [g, _dp, _dp]
        L.orc_sort_key.argtypes = [g, C.c_int]
        L.orc_sort_key.restype = C.c_long
        L.orc_counting_sort.argtypes = [g, C.c_long, _ip, _lp]
        L.orc_implicit_deposit.argtypes = [g, p, _dp, _dp, _dp, _dp, _dp, _dp]
        L.orc_implicit_moments_finish.argtypes = [g, _dp, _dp, _dp, _dp]
        L.orc_wall_node_moments.argtypes = [g, _dp, _dp]
        L.orc_pi_size.argtypes = [g]
        L.orc_pi_size.restype = C.c_long
        L.orc_rho_ext_size.argtypes = [g]
        L.orc_rho_ext_size.restype = C.c_long
        L.orc_maxwell_rhs.argtypes = [g, _dp, _dp, _dp, _dp, _dp]
        L.orc_maxwell_apply.argtypes = [g, _dp, _dp, _dp]
        L.orc_gmres.argtypes = [g, _dp, _dp, _dp, _dp]
        L.orc_gmres.restype = C.c_int
        L.orc_field_update.argtypes = [g, _dp, _dp, _dp, _dp, _dp]
        L.orc_implicit_push.argtypes = [g, p, _dp, _dp, _dp]
        L.orc_implicit_step.argtypes = [g, p, C.c_int, _dp, _dp, _dp]
        L.orc_implicit_step.restype = C.c_int
        L.orc_implicit_work_size.argtypes = [g]
        L.orc_implicit_work_size.restype = C.c_long
        L.orc_energy.argtypes = [g, p, C.c_int, _dp, _dp, _dp]
        L.orc_density_moments.argtypes = [g, p, C.c_int, _dp, _dp, _dp, _dp]
        L.orc_smooth.argtypes = [g, _dp, C.c_int]
        L.orc_smooth_moments.argtypes = [g, _dp, _dp, _dp]
    return _lib


def _d(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def make_grid(box, tile=(8, 8, 8), pressure_compat=1, gmres_max_iter=50, gmres_tol=1e-8, smoothing_count=0,
              smoothing_parameter=0.5, wall_x=0, e_right=(0.0, 0.0, 0.0), b_right=(0.0, 0.0, 0.0)) -> Grid:
    """wall_x: conductor wall at x = 0 and open boundary at x = (nx - 2) dx,
    with the boundary's constant fields e_right, b_right (oracle.h)."""
    t = [min(tile[0], box.nx), min(tile[1], box.ny), min(tile[2], box.nz)]
    return Grid(box.nx, box.ny, box.nz, t[0], t[1], t[2], box.dx, box.dy, box.dz, box.dt,
                box.theta, box.eta, box.cfix, pressure_compat, gmres_max_iter, gmres_tol, smoothing_count,
                smoothing_parameter, int(wall_x), (C.c_double * 3)(*e_right), (C.c_double * 3)(*b_right))


def erase_escaped(species):
    """eraseEscapedPaticles (mover.cpp:167-192): drops the particles the
    mover marked escaped (cell = -1) from every array of each species dict,
    keeping the order of the others."""
    for sp in species:
        keep = np.asarray(sp["cell"]) >= 0
        if keep.all():
            continue
        for k, v in list(sp.items()):
            if isinstance(v, np.ndarray) and v.shape[:1] == keep.shape:
                sp[k] = np.ascontiguousarray(v[keep])


def _as_particles(sp: dict) -> Particles:
    for k in ("ox", "oy", "oz", "px", "py", "pz"):
        sp[k] = np.ascontiguousarray(sp[k], dtype=np.float64)
    sp["cell"] = np.ascontiguousarray(sp["cell"], dtype=np.int32)
    return Particles(sp["q"], sp["m"], sp["w"], len(sp["cell"]), sp["cell"].ctypes.data_as(_ip),
                     _d(sp["ox"]), _d(sp["oy"]), _d(sp["oz"]), _d(sp["px"]), _d(sp["py"]), _d(sp["pz"]))


def _plist(species):
    arr = (Particles * len(species))(*[_as_particles(s) for s in species])
    return arr


def buneman_step(grid: Grid, species, E, B, J=None):
    """In place on species/E/B; returns J of the step."""
    if J is None:
        J = np.zeros_like(E)
    arr = _plist(species)
    lib().orc_buneman_step(C.byref(grid), arr, len(species), _d(E), _d(B), _d(J))
    if grid.wall_x:
        erase_escaped(species)
    return J


def implicit_step(grid: Grid, species, E, B):
    work = np.zeros(lib().orc_implicit_work_size(C.byref(grid)))
    arr = _plist(species)
    it = lib().orc_implicit_step(C.byref(grid), arr, len(species), _d(E), _d(B), _d(work))
    if grid.wall_x:
        erase_escaped(species)
    return it


def implicit_moments(grid: Grid, species, E, B):
    """Returns J-hat, mu, rho-hat (with its low ghost layer, see
    orc_implicit_moments_finish), the folded Pi and the raw deposits."""
    N = grid.nx * grid.ny * grid.nz
    L = lib()
    J = np.zeros(3 * N); mu = np.zeros(9 * N); rho = np.zeros(N)
    Pi = np.zeros(L.orc_pi_size(C.byref(grid)))
    rho_ext = np.zeros(L.orc_rho_ext_size(C.byref(grid)))
    for s in species:
        ps = _as_particles(s)
        L.orc_implicit_deposit(C.byref(grid), C.byref(ps), _d(E), _d(B), _d(J), _d(mu), _d(rho), _d(Pi))
    L.orc_wall_node_moments(C.byref(grid), _d(J), _d(mu))
    raw = dict(J=J.copy(), rho=rho.copy(), Pi=Pi.copy())
    L.orc_implicit_moments_finish(C.byref(grid), _d(J), _d(rho), _d(Pi), _d(rho_ext))
    return J, mu, rho_ext, Pi, raw


def rho_interior(grid: Grid, rho_ext):
    """The periodic cells of a rho-hat array that carries a low ghost layer."""
    sh = [n + 1 if n > 1 else 1 for n in (grid.nz, grid.ny, grid.nx)]
    r = rho_ext.reshape(sh)
    sl = tuple(slice(1, None) if n > 1 else slice(0, 1) for n in (grid.nz, grid.ny, grid.nx))
    return np.ascontiguousarray(r[sl]).reshape(-1)


def maxwell_rhs(grid, E, B, J, rho_ext):
    rhs = np.zeros(3 * grid.nx * grid.ny * grid.nz)
    lib().orc_maxwell_rhs(C.byref(grid), _d(E), _d(B), _d(J), _d(rho_ext), _d(rhs))
    return rhs


def maxwell_apply(grid, mu, x):
    y = np.zeros_like(x)
    lib().orc_maxwell_apply(C.byref(grid), _d(mu), _d(x), _d(y))
    return y


def gmres(grid, mu, rhs):
    x = np.zeros_like(rhs)
    rel = C.c_double(0.0)
    it = lib().orc_gmres(C.byref(grid), _d(mu), _d(rhs), _d(x), C.byref(rel))
    return x, it, rel.value


def field_update(grid, Et, E, B):
    En = np.zeros_like(E); Bn = np.zeros_like(B)
    lib().orc_field_update(C.byref(grid), _d(Et), _d(E), _d(B), _d(En), _d(Bn))
    return En, Bn


def implicit_push(grid, sp, E, B, Et):
    ps = _as_particles(sp)
    lib().orc_implicit_push(C.byref(grid), C.byref(ps), _d(E), _d(B), _d(Et))


def counting_sort(grid, cell):
    cell = np.ascontiguousarray(cell, dtype=np.int32)
    perm = np.zeros(len(cell), dtype=np.int64)
    lib().orc_counting_sort(C.byref(grid), len(cell), cell.ctypes.data_as(_ip), perm.ctypes.data_as(_lp))
    return perm


def sort_keys(grid, cell):
    return np.array([lib().orc_sort_key(C.byref(grid), int(c)) for c in cell], dtype=np.int64)


def energy(grid, species, E, B):
    out = np.zeros(6)
    arr = _plist(species)
    lib().orc_energy(C.byref(grid), arr, len(species), _d(E), _d(B), _d(out))
    return out


def density_moments(grid, species):
    """updateDensityParameters: (conc[s][N], energy[s][N], vel[s][3][N], rho[N])."""
    N = grid.nx * grid.ny * grid.nz
    ns = len(species)
    conc, en, vel, rho = np.zeros(ns * N), np.zeros(ns * N), np.zeros(3 * ns * N), np.zeros(N)
    arr = _plist(species)
    lib().orc_density_moments(C.byref(grid), arr, ns, _d(conc), _d(en), _d(vel), _d(rho))
    return conc.reshape(ns, N), en.reshape(ns, N), vel.reshape(ns, 3, N), rho


# ---------------------------------------------------------------- reference
def reference_available() -> bool:
    return bool(REF_SRC) and os.path.isdir(REF_SRC)


def build_reference() -> str:
    if not reference_available():
        raise RuntimeError("PICPP_REFERENCE_SRC does not name the PIC++ source directory")
    subprocess.check_call(["make", "-s", "-j8", "-C", HERE, "ref", f"REF={REF_SRC}"])
    return REF_BIN


def run_reference(solver: int, box, species, E, B, steps: int, dump: bool = False, density: bool = False,
                  smoothing_count: int = 0, smoothing_parameter: float = 0.5, wall_x: int = 0,
                  e_right=(0.0, 0.0, 0.0), b_right=(0.0, 0.0, 0.0)):
    """Runs the PIC++ reference (compiled from its own sources) on the state
    and returns (species positions/momenta by input order, E, B, extras).
    With wall_x the reference runs SUPER_CONDUCTOR_LEFT on the nx - 2
    physical cells of the box; escaped particles come back as NaN."""
    from picpp_gb300.initstate import positions
    exe = build_reference()
    N = box.ncells
    with tempfile.TemporaryDirectory() as td:
        fin, fout = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        with open(fin, "wb") as f:
            f.write(struct.pack("<10i", solver, box.nx, box.ny, box.nz, len(species), steps, int(dump), int(density),
                                smoothing_count, int(wall_x)))
            f.write(struct.pack("<11d", box.dx, box.dt, box.theta, box.eta, smoothing_parameter, *e_right, *b_right))
            for sp in species:
                x, y, z = positions(box, sp)
                f.write(struct.pack("<3dq", sp["q"], sp["m"], sp["w"], len(sp["cell"])))
                for a in (x, y, z, sp["px"], sp["py"], sp["pz"]):
                    f.write(np.ascontiguousarray(a, dtype="<f8").tobytes())
            f.write(np.ascontiguousarray(E, dtype="<f8").tobytes())
            f.write(np.ascontiguousarray(B, dtype="<f8").tobytes())
        subprocess.check_call([exe, fin, fout], stdout=subprocess.DEVNULL)
        raw = np.fromfile(fout, dtype=np.uint8)
    off = 0

    def take(count, dt="<f8"):
        nonlocal off
        a = np.frombuffer(raw, dtype=dt, count=count, offset=off)
        off += a.nbytes
        return a.copy()

    out_sp = []
    for _ in species:
        n = int(take(1, "<i8")[0])
        vals = [take(n) for _ in range(6)]
        out_sp.append(dict(zip(("x", "y", "z", "px", "py", "pz"), vals)))
    Eo = take(3 * N).reshape(3, box.nz, box.ny, box.nx)
    Bo = take(3 * N).reshape(3, box.nz, box.ny, box.nx)
    extra = {}
    if solver == 0:
        extra["J"] = take(3 * N).reshape(3, box.nz, box.ny, box.nx)
    elif dump:
        for name, c in (("J", 3), ("mu", 9), ("rho", 1), ("Pi", 9), ("rhs", 3), ("Etheta", 3)):
            extra[name] = take(c * N)
    if density:
        ns = len(species)
        conc, en, vel = np.zeros((ns, N)), np.zeros((ns, N)), np.zeros((ns, 3, N))
        for s in range(ns):
            conc[s], en[s], vel[s] = take(N), take(N), take(3 * N).reshape(3, N)
        extra["density"] = (conc, en, vel, take(N))
    assert off == raw.nbytes
    return out_sp, Eo, Bo, extra
