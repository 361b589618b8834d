"""The C++ mirror of Simulation (include/picpp_gb300_simulation.hpp) driving
the step loop from a compiled C++ program (tests/cpp/mirror_steps.cpp)
against the oracle: the path a C++ caller of the drop-in takes.  Needs a
GB300 and g++."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import pyoracle as O
from fixtures import copy_species, periodic_dist, rel_err
from picpp_gb300 import initstate as I

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "picpp_gb300")


@pytest.fixture(scope="module")
def caller_exe(tmp_path_factory):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    import picpp_gb300 as P
    P.load_library()   # builds libpicpp_gb300.so if needed
    exe = str(tmp_path_factory.mktemp("cpp") / "mirror_steps")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "mirror_steps.cpp"), "-o", exe, "-L", PKG, "-lpicpp_gb300",
                    "-Wl,-rpath," + PKG], check=True, capture_output=True, text=True)
    return exe


def run(caller_exe, tmp_path, st, solver, real, steps):
    box = st.box
    N = box.ncells
    fin, fout = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    with open(fin, "wb") as f:
        # pressure_compat = 1: the reference's pressure-tensor placement, as the oracle
        np.array([box.nx, box.ny, box.nz, solver, real, steps, len(st.species), 1], "<i4").tofile(f)
        np.array([box.dx, box.dy, box.dz, box.dt, box.theta, box.eta, box.cfix], "<f8").tofile(f)
        for s in st.species:
            n = len(s["cell"])
            np.array([s["q"], s["m"], s["w"]], "<f8").tofile(f)
            np.array([n], "<i8").tofile(f)
            np.asarray(s["cell"], "<i4").tofile(f)
            for k in ("ox", "oy", "oz", "px", "py", "pz"):
                np.asarray(s[k], "<f8").tofile(f)
            np.arange(n, dtype="<i4").tofile(f)
        np.asarray(st.E, "<f8").tofile(f)
        np.asarray(st.B, "<f8").tofile(f)
    r = subprocess.run([caller_exe, fin, fout], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    raw = open(fout, "rb").read()
    pos = 0

    def take(dtype, n):
        nonlocal pos
        a = np.frombuffer(raw, dtype=dtype, count=n, offset=pos)
        pos += a.nbytes
        return a

    E, B = take("<f8", 3 * N), take("<f8", 3 * N)
    out = []
    for _ in st.species:
        n = int(take("<i8", 1)[0])
        d = {"cell": take("<i4", n)}
        for k in ("ox", "oy", "oz", "px", "py", "pz"):
            d[k] = take("<f8", n)
        d["id"] = take("<i4", n)
        o = np.argsort(d["id"])
        out.append({k: v[o] for k, v in d.items()})
    return E, B, out


def check_particles(box, got, ref, tol_p, tol_x):
    L = (box.nx * box.dx, box.ny * box.dy, box.nz * box.dz)
    x, y, z = I.positions(box, got)
    xr, yr, zr = I.positions(box, ref)
    for a, r, l, d in ((x, xr, L[0], box.dx), (y, yr, L[1], box.dy), (z, zr, L[2], box.dz)):
        assert periodic_dist(a, r, l).max() <= tol_x * d
    for k in ("px", "py", "pz"):
        assert rel_err(got[k], ref[k]) <= tol_p


def test_cpp_buneman_step_loop_matches_oracle(caller_exe, tmp_path):
    st = I.buneman_plasma(8, 8, 8, ppc=3, seed=51)
    steps = 3
    E, B, got = run(caller_exe, tmp_path, st, 0, 1, steps)
    g = O.make_grid(st.box)
    sp = copy_species(st.species)
    Eo, Bo = st.E.copy(), st.B.copy()
    for _ in range(steps):
        O.buneman_step(g, sp, Eo, Bo)
    assert rel_err(E, Eo.reshape(-1)) < 1e-11
    assert rel_err(B, Bo.reshape(-1)) < 1e-11
    for s in range(2):
        check_particles(st.box, got[s], sp[s], 1e-11, 1e-10)


def test_cpp_implicit_step_loop_matches_oracle(caller_exe, tmp_path):
    st = I.beams_plasma(8, 6, 5, ppc=2, beam_gamma=2.0, dt=0.2, seed=52)
    steps = 2
    E, B, got = run(caller_exe, tmp_path, st, 1, 1, steps)
    g = O.make_grid(st.box)
    sp = copy_species(st.species)
    Eo, Bo = st.E.reshape(-1).copy(), st.B.reshape(-1).copy()
    for _ in range(steps):
        O.implicit_step(g, sp, Eo, Bo)
    assert rel_err(E, Eo) < 1e-9
    assert rel_err(B, Bo) < 1e-9
    for s in range(2):
        check_particles(st.box, got[s], sp[s], 1e-9, 1e-8)
