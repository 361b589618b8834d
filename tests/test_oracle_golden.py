"""The C oracle against golden vectors produced by the PIC++ reference itself
(tests/golden/make_golden.py).  CPU only."""
import numpy as np
import pytest

import pyoracle as O
from fixtures import (copy_species, golden_names, load, periodic_dist, rel_err, smoothing_of, survivors, wall_of,
                      yee_physical)
from picpp_gb300 import initstate as I

# The oracle keeps cell + offset where the reference keeps absolute FP64
# coordinates; the two differ by rounding only.
TOL = 1e-11


@pytest.mark.parametrize("name", golden_names("buneman"))
def test_buneman_matches_reference(name):
    f = load(name)
    st = f["state"]
    sc, spar = smoothing_of(f)
    g = O.make_grid(st.box, smoothing_count=sc, smoothing_parameter=spar)
    sp = copy_species(st.species)
    E, B = st.E.copy(), st.B.copy()
    for _ in range(f["steps"]):
        J = O.buneman_step(g, sp, E, B)
    assert rel_err(E, f["E"]) < TOL
    assert rel_err(B, f["B"]) < TOL
    assert rel_err(J, f["extra"]["J"]) < TOL
    L = (st.box.nx * st.box.dx, st.box.ny * st.box.dy, st.box.nz * st.box.dz)
    for s, o in zip(sp, f["out"]):
        x, y, z = I.positions(st.box, s)
        for a, r, l in ((x, o["x"], L[0]), (y, o["y"], L[1]), (z, o["z"], L[2])):
            if l > st.box.dx * 1.5:
                assert periodic_dist(a, r, l).max() < 1e-12
        for k in ("px", "py", "pz"):
            assert rel_err(s[k], o[k]) < TOL


@pytest.mark.parametrize("name", golden_names("implicit"))
def test_implicit_moments_and_solve_match_reference(name):
    f = load(name)
    st = f["state"]
    g = O.make_grid(st.box)
    E, B = st.E.reshape(-1).copy(), st.B.reshape(-1).copy()
    J, mu, rho_ext, Pi, raw = O.implicit_moments(g, copy_species(st.species), E, B)
    x = f["extra"]
    assert rel_err(mu, x["mu"]) < TOL
    assert rel_err(J, x["J"]) < TOL
    assert rel_err(O.rho_interior(g, rho_ext), x["rho"]) < TOL
    rhs = O.maxwell_rhs(g, E, B, J, rho_ext)
    assert rel_err(rhs, x["rhs"]) < TOL
    Et, it, relres = O.gmres(g, mu, rhs)
    assert rel_err(Et, x["Etheta"]) < 1e-9
    assert it >= 1


@pytest.mark.parametrize("name", golden_names("implicit"))
def test_implicit_step_matches_reference(name):
    f = load(name)
    st = f["state"]
    g = O.make_grid(st.box)
    sp = copy_species(st.species)
    E, B = st.E.reshape(-1).copy(), st.B.reshape(-1).copy()
    for _ in range(f["steps"]):
        O.implicit_step(g, sp, E, B)
    assert rel_err(E, f["E"].reshape(-1)) < 1e-9
    assert rel_err(B, f["B"].reshape(-1)) < 1e-9
    L = (st.box.nx * st.box.dx, st.box.ny * st.box.dy, st.box.nz * st.box.dz)
    for s, o in zip(sp, f["out"]):
        x, y, z = I.positions(st.box, s)
        for a, r, l in ((x, o["x"], L[0]), (y, o["y"], L[1]), (z, o["z"], L[2])):
            assert periodic_dist(a, r, l).max() < 1e-10
        for k in ("px", "py", "pz"):
            assert rel_err(s[k], o[k]) < 1e-9


def test_counting_sort_is_stable_and_tile_major():
    box = I.Box(16, 8, 8, 0.1, 0.1, 0.1, 0.01)
    g = O.make_grid(box, tile=(8, 4, 4))
    rng = np.random.default_rng(0)
    cell = rng.integers(0, box.ncells, size=5000).astype(np.int32)
    perm = O.counting_sort(g, cell)
    keys = O.sort_keys(g, cell)
    sk = keys[perm]
    assert np.all(np.diff(sk) >= 0)
    # stability: equal keys keep their input order
    same = np.diff(sk) == 0
    assert np.all(np.diff(perm)[same] > 0)
    assert np.array_equal(np.sort(perm), np.arange(len(cell)))


def test_gmres_tiny_system_residual():
    """A small implicit operator solved to the reference's stopping rule; the
    true residual must be at the requested level (in the spirit of the
    reference's printf GMRES test program, test/test.cpp:70-192, with an assert)."""
    box = I.Box(5, 5, 5, 0.5, 0.5, 0.5, 0.5)
    g = O.make_grid(box, gmres_max_iter=200)
    rng = np.random.default_rng(3)
    N = box.ncells
    mu = np.zeros(9 * N)
    for a in range(3):
        mu[(4 * a) * N:(4 * a + 1) * N] = -0.3 * rng.random(N)
    rhs = rng.standard_normal(3 * N)
    x, it, rel = O.gmres(g, mu, rhs)
    r = O.maxwell_apply(g, mu, x) - rhs
    assert np.linalg.norm(r) / np.linalg.norm(rhs) < 1e-7


@pytest.mark.parametrize("name", golden_names("density"))
def test_oracle_density_moments_match_reference(name):
    """updateDensityParameters of the reference (per species concentration,
    energy density, bulk velocity; charge density) against the oracle; the
    density_wall cases are reflecting-wall boxes, where the ghost columns
    fold into the first and the last physical cell."""
    f = load(name)
    st = f["state"]
    wall, er, br = wall_of(f)
    g = O.make_grid(st.box, wall_x=wall, e_right=er, b_right=br)
    conc, en, vel, rho = O.density_moments(g, copy_species(st.species))
    x = f["extra"]
    assert rel_err(conc, x["conc"]) < 1e-13
    assert rel_err(en, x["energy"]) < 1e-13
    assert rel_err(vel, x["vel"]) < 1e-13
    assert rel_err(rho, x["rho"]) < 1e-13


def test_wall_density_fold_keeps_totals_and_empties_the_ghosts():
    """The wall box's density pass moves the ghost columns' deposits into the
    first and last physical cells: the ghost columns end empty, and every
    particle's weight is still counted once (its cell weights sum to one)."""
    st = I.shock_plasma(12, 6, 5, ppc=(3, 3, 2), flow_gamma=3.0, theta_e=0.3, seed=71)
    b = st.box
    g = O.make_grid(b, wall_x=1, e_right=st.e_right, b_right=st.b_right)
    conc, en, vel, rho = O.density_moments(g, copy_species(st.species))
    vol = b.dx * b.dy * b.dz
    for s, sp in enumerate(st.species):
        c = conc[s].reshape(b.nz, b.ny, b.nx)
        assert np.all(c[..., b.nx - 2:] == 0.0)
        assert np.all(en[s].reshape(b.nz, b.ny, b.nx)[..., b.nx - 2:] == 0.0)
        assert np.all(vel[s].reshape(3, b.nz, b.ny, b.nx)[..., b.nx - 2:] == 0.0)
        assert abs(c.sum() * vol / (sp["w"] * len(sp["cell"])) - 1.0) < 1e-12
    q = sum(sp["q"] * sp["w"] * len(sp["cell"]) for sp in st.species)
    assert abs(rho.sum() * vol - q) < 1e-12 * sum(abs(sp["q"]) * sp["w"] * len(sp["cell"]) for sp in st.species)


@pytest.mark.parametrize("name", golden_names("wall"))
def test_wall_moments_and_solve_match_reference(name):
    """Conductor wall at x = 0, open boundary at x = (nx - 2) dx: the first
    step's J-hat, mu, rho-hat, right part and E^{n+theta} on every node and
    cell the reference keeps (the storage column nx - 1 is the reference's
    ghost beyond the open boundary for nodes; its cell is the ghost left of
    the wall, which the reference does not write out)."""
    f = load(name)
    st = f["state"]
    w, er, br = wall_of(f)
    g = O.make_grid(st.box, wall_x=w, e_right=er, b_right=br)
    E, B = st.E.reshape(-1).copy(), st.B.reshape(-1).copy()
    J, mu, rho_ext, Pi, raw = O.implicit_moments(g, copy_species(st.species), E, B)
    x = f["extra"]
    b = st.box
    node = lambda a, c: a.reshape(c, b.nz, b.ny, b.nx)[..., : b.nx - 1]   # noqa: E731
    assert rel_err(node(mu, 9), node(x["mu"], 9)) < TOL
    assert rel_err(node(J, 3), node(x["J"], 3)) < TOL
    rho = O.rho_interior(g, rho_ext).reshape(b.nz, b.ny, b.nx)[..., : b.nx - 2]
    assert rel_err(rho, x["rho"].reshape(b.nz, b.ny, b.nx)[..., : b.nx - 2]) < TOL
    rhs = O.maxwell_rhs(g, E, B, J, rho_ext)
    assert rel_err(node(rhs, 3), node(x["rhs"], 3)) < TOL
    Et, it, relres = O.gmres(g, mu, rhs)
    assert rel_err(node(Et, 3), node(x["Etheta"], 3)) < 1e-10


@pytest.mark.parametrize("name", golden_names("wall"))
def test_wall_steps_match_reference(name):
    """Reflection at the wall, escape through the open boundary and the
    fields after several steps: the same particles survive, with the
    reference's positions and momenta."""
    f = load(name)
    st = f["state"]
    w, er, br = wall_of(f)
    g = O.make_grid(st.box, wall_x=w, e_right=er, b_right=br)
    sp = copy_species(st.species)
    for s in sp:
        s["id"] = np.arange(len(s["cell"]))
    E, B = st.E.reshape(-1).copy(), st.B.reshape(-1).copy()
    for _ in range(f["steps"]):
        O.implicit_step(g, sp, E, B)
    b = st.box
    sh = (3, b.nz, b.ny, b.nx)
    assert rel_err(E.reshape(sh)[..., : b.nx - 1], f["E"].reshape(sh)[..., : b.nx - 1]) < TOL
    assert rel_err(B.reshape(sh)[..., : b.nx - 2], f["B"].reshape(sh)[..., : b.nx - 2]) < TOL
    escaped = 0
    for s, o in zip(sp, f["out"]):
        keep = survivors(o)
        escaped += len(o["x"]) - len(keep)
        assert np.array_equal(s["id"], keep)
        x, y, z = I.positions(b, s)
        assert np.abs(x - o["x"][keep]).max() < 1e-12
        for k in ("px", "py", "pz"):
            assert rel_err(s[k], o[k][keep]) < TOL
    assert escaped > 0


@pytest.mark.parametrize("name", golden_names("tristan_wall"))
def test_tristan_wall_matches_reference(name):
    """The explicit path in a reflecting-wall box against the reference's
    own SUPER_CONDUCTOR_LEFT Buneman runs: reflection at node 18 (the
    zigzag current of a reflected particle mirrored there), E_y = E_z = 0 on
    the wall node and E0 on the open boundary node, escape and erase."""
    f = load(name)
    st = f["state"]
    w, er, br = wall_of(f)
    g = O.make_grid(st.box, wall_x=w, e_right=er, b_right=br)
    sp = copy_species(st.species)
    for s in sp:
        s["id"] = np.arange(len(s["cell"]))
    E, B = st.E.copy(), st.B.copy()
    for _ in range(f["steps"]):
        J = O.buneman_step(g, sp, E, B)
    b = st.box
    assert rel_err(yee_physical(E, b, "E"), yee_physical(f["E"], b, "E")) < TOL
    assert rel_err(yee_physical(B, b, "B"), yee_physical(f["B"], b, "B")) < TOL
    assert rel_err(J, f["extra"]["J"]) < TOL
    escaped = reflected = 0
    for s, s0, o in zip(sp, st.species, f["out"]):
        keep = survivors(o)
        escaped += len(o["x"]) - len(keep)
        reflected += int(np.sum(np.sign(s["px"]) != np.sign(s0["px"][keep])))
        assert np.array_equal(s["id"], keep)
        x, y, z = I.positions(b, s)
        assert np.abs(x - o["x"][keep]).max() < 1e-12
        assert x.min() >= I.TRISTAN_WALL_NODE * b.dx
        for k in ("px", "py", "pz"):
            assert rel_err(s[k], o[k][keep]) < TOL
    assert escaped > 0 and reflected > 0
