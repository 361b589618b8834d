"""Conductor wall at x = 0 and open boundary at x = (nx - 2) dx on the GPU
(pic_config.boundary_x = PIC_BOUNDARY_WALL_OPEN): against outputs of the
reference itself (tests/golden/wall_*, the reference's pressure-tensor
placement) and against the oracle with the periodic placement the bench
runs, with particles reflected at the wall, escaping through the open
boundary and injected there.  Needs a GB300."""
import numpy as np
import pytest

import pyoracle as O
from fixtures import copy_species, golden_names, load, rel_err, survivors, wall_of, yee_physical
from picpp_gb300 import initstate as I

pytestmark = pytest.mark.gpu

TOL64 = 1e-11
TOL32 = 1e-5


@pytest.fixture(scope="module")
def pg():
    import picpp_gb300 as P
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    P.load_library()
    return P


def by_id(d):
    o = np.argsort(d["id"])
    return {k: v[o] for k, v in d.items()}


def phys(a, box, ncomp, cells):
    """The physical nodes (cells=False: 0 .. nx - 2) or cells (0 .. nx - 3)."""
    a = np.asarray(a).reshape(ncomp, box.nz, box.ny, box.nx)
    return a[..., : box.nx - (2 if cells else 1)]


def wall_sim(pg, st, real, compat, sort_every, er, br):
    return pg.GpuSimulation(st.box, pg.IMPLICIT, particle_real=real, pressure_compat=compat, sort_every=sort_every,
                            tile=(0, 0, 0), boundary_x=pg.BOUNDARY_WALL_OPEN, e_right=er, b_right=br)


@pytest.mark.parametrize("sort_every", [0, 1])
@pytest.mark.parametrize("name", golden_names("wall"))
def test_wall_golden_vectors(pg, name, sort_every):
    """The reference's own wall runs (reference pressure placement): the first
    step's moments and right part, then every surviving particle and the
    fields of the physical domain after the run."""
    f = load(name)
    st = f["state"]
    w, er, br = wall_of(f)
    sim = wall_sim(pg, st, 1, 1, sort_every, er, br)
    sim.upload_state(st)
    sim.updateElectroMagneticParameters()
    J, mu, rho, rhs = sim.download_moments()
    x = f["extra"]
    b = st.box
    assert rel_err(phys(mu, b, 9, False), phys(x["mu"], b, 9, False)) < TOL64
    assert rel_err(phys(J, b, 3, False), phys(x["J"], b, 3, False)) < TOL64
    assert rel_err(phys(rhs, b, 3, False), phys(x["rhs"], b, 3, False)) < TOL64
    sim.evaluateElectricField(pg.solve_opts(pg.GMRES_REFERENCE))
    sim.evaluateMagneticField()
    sim.moveParticles()
    sim.updateFields()
    for _ in range(f["steps"] - 1):
        sim.implicit_step(pg.solve_opts(pg.GMRES_REFERENCE))
    E, B, _ = sim.download_fields()
    assert rel_err(phys(E, b, 3, False), phys(f["E"], b, 3, False)) < TOL64
    assert rel_err(phys(B, b, 3, True), phys(f["B"], b, 3, True)) < TOL64
    escaped = 0
    for s, o in enumerate(f["out"]):
        keep = survivors(o)
        escaped += len(o["x"]) - len(keep)
        got = by_id(sim.download_particles(s))
        assert np.array_equal(got["id"], keep)
        xg, yg, zg = I.positions(b, got)
        assert np.abs(xg - o["x"][keep]).max() < 1e-11
        for k in ("px", "py", "pz"):
            assert rel_err(got[k], o[k][keep]) < TOL64
    assert escaped > 0
    sim.close()


def _flow_state(seed=43):
    st = I.shock_plasma(12, 8, 8, ppc=(4, 4, 2), flow_gamma=3.0, theta_e=0.3, seed=seed)
    for sp in st.species:
        sp["px"][::3] = -sp["px"][::3]   # a third of each species heads for the open boundary
    return st


def _inject(st, step, rng):
    """One slab of new particles per species at the open boundary, in the
    last physical cell column, moving in with the flow (the caller's part of
    injectNewParticles)."""
    b = st.box
    out = []
    for s, sp in enumerate(st.species):
        n = b.ny * b.nz
        j = np.arange(n) % b.ny
        k = np.arange(n) // b.ny
        cell = ((k * b.ny + j) * b.nx + (b.nx - 3)).astype(np.int32)
        px, py, pz = I.sample_juttner(rng, n, st.temperatures[s], sp["m"], st.flow_gamma, -1.0)
        out.append(dict(cell=cell, ox=0.5 + 0.5 * rng.random(n), oy=rng.random(n), oz=rng.random(n),
                        px=px, py=py, pz=pz))
    return out


@pytest.mark.parametrize("real,sort_every", [(1, 1), (1, 0), (0, 1)])
def test_wall_steps_with_injection_match_oracle(pg, real, sort_every):
    """Periodic pressure placement (the production path): reflection,
    escape and particles appended at the open boundary before every step,
    against the oracle on the same appended particles."""
    st = _flow_state()
    er, br = st.e_right, st.b_right
    sim = wall_sim(pg, st, real, 0, sort_every, er, br)
    for sp in st.species:
        sim.add_species(sp["q"], sp["m"], sp["w"], 4 * len(sp["cell"]))
    for s, sp in enumerate(st.species):
        sim.upload_particles(s, sp)
    sim.upload_fields(st.E, st.B)
    g = O.make_grid(st.box, pressure_compat=0, wall_x=1, e_right=er, b_right=br)
    spo = copy_species(st.species)
    for sp in spo:
        sp["id"] = np.arange(len(sp["cell"]), dtype=np.int32)
    nxt = [len(sp["cell"]) for sp in spo]   # the next particle number of each species
    E, B = st.E.reshape(-1).copy(), st.B.reshape(-1).copy()
    rng = np.random.default_rng(7)
    for step in range(4):
        for s, new in enumerate(_inject(st, step, rng)):
            sim.append_particles(s, new)
            for k in ("cell", "ox", "oy", "oz", "px", "py", "pz"):
                spo[s][k] = np.concatenate([spo[s][k], new[k]]).astype(spo[s][k].dtype)
            spo[s]["id"] = np.concatenate([spo[s]["id"], np.arange(nxt[s], nxt[s] + len(new["cell"]), dtype=np.int32)])
            nxt[s] += len(new["cell"])
        sim.implicit_step(pg.solve_opts(pg.GMRES_REFERENCE))
        O.implicit_step(g, spo, E, B)
    tol = TOL64 if real else TOL32
    Eg, Bg, _ = sim.download_fields()
    b = st.box
    assert rel_err(phys(Eg, b, 3, False), phys(E, b, 3, False)) < tol
    assert rel_err(phys(Bg, b, 3, True), phys(B, b, 3, True)) < tol
    escaped = 0
    for s in range(len(spo)):
        got = by_id(sim.download_particles(s))
        ref = by_id({k: v for k, v in spo[s].items() if isinstance(v, np.ndarray)})
        escaped += nxt[s] - len(ref["id"])
        assert np.array_equal(got["id"], ref["id"])
        xg, _, _ = I.positions(b, got)
        xr, _, _ = I.positions(b, ref)
        assert np.abs(xg - xr).max() < (1e-11 if real else 1e-5) * b.dx
        for k in ("px", "py", "pz"):
            assert rel_err(got[k], ref[k]) < tol
    assert escaped > 0
    sim.close()


def test_wall_far_drift_takes_the_mover_deferred_pass(pg):
    """One-cell tiles and a sort every fifth step: after a few steps most
    particles lie more than the two-cell halo away from their tile, so the
    tiled mover leaves them to its deferred pass (the wall rules of the
    untiled mover: reflection at the wall, escape at the open boundary).
    FP64 fields and particles after 5 steps against the oracle."""
    st = _flow_state(seed=47)
    er, br = st.e_right, st.b_right
    sim = pg.GpuSimulation(st.box, pg.IMPLICIT, particle_real=1, pressure_compat=0, sort_every=5, tile=(1, 1, 1),
                           boundary_x=pg.BOUNDARY_WALL_OPEN, e_right=er, b_right=br)
    sim.upload_state(st)
    g = O.make_grid(st.box, pressure_compat=0, wall_x=1, e_right=er, b_right=br)
    spo = copy_species(st.species)
    for sp in spo:
        sp["id"] = np.arange(len(sp["cell"]), dtype=np.int32)
    E, B = st.E.reshape(-1).copy(), st.B.reshape(-1).copy()
    for _ in range(5):
        sim.implicit_step(pg.solve_opts(pg.GMRES_REFERENCE))
        O.implicit_step(g, spo, E, B)
    Eg, Bg, _ = sim.download_fields()
    b = st.box
    assert rel_err(phys(Eg, b, 3, False), phys(E, b, 3, False)) < TOL64
    assert rel_err(phys(Bg, b, 3, True), phys(B, b, 3, True)) < TOL64
    escaped = 0
    for s in range(len(spo)):
        got = by_id(sim.download_particles(s))
        ref = by_id({k: v for k, v in spo[s].items() if isinstance(v, np.ndarray)})
        escaped += len(st.species[s]["cell"]) - len(ref["id"])
        assert np.array_equal(got["id"], ref["id"])
        xg, _, _ = I.positions(b, got)
        xr, _, _ = I.positions(b, ref)
        assert np.abs(xg - xr).max() < 1e-11 * b.dx
        for k in ("px", "py", "pz"):
            assert rel_err(got[k], ref[k]) < TOL64
    assert escaped > 0
    sim.close()


def test_wall_rejects_particles_in_ghost_columns_and_other_setups(pg):
    st = _flow_state()
    er, br = st.e_right, st.b_right
    sim = wall_sim(pg, st, 1, 0, 1, er, br)
    sp = dict(st.species[0])
    sid = sim.add_species(sp["q"], sp["m"], sp["w"], len(sp["cell"]))
    bad = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in sp.items()}
    bad["cell"][0] = st.box.nx - 2   # the ghost cell beyond the open boundary
    with pytest.raises(pg.PicError):
        sim.upload_particles(sid, bad)
    sim.close()
    with pytest.raises(pg.PicError):   # explicit wall boxes reach 4 cells beyond the reflecting wall (nx >= 24)
        pg.GpuSimulation(st.box, pg.BUNEMAN, particle_real=1, boundary_x=pg.BOUNDARY_WALL_OPEN)
    flat = I.Box(12, 8, 1, 0.5, 0.5, 0.5, 0.4)
    with pytest.raises(pg.PicError):   # 3-D boxes only
        pg.GpuSimulation(flat, pg.IMPLICIT, particle_real=1, pressure_compat=0, boundary_x=pg.BOUNDARY_WALL_OPEN)


# ------------------------------------------------------------------ explicit (Tristan) path
def tristan_sim(pg, st, real, sort_every, er, br):
    return pg.GpuSimulation(st.box, pg.BUNEMAN, particle_real=real, sort_every=sort_every, tile=(0, 0, 0),
                            boundary_x=pg.BOUNDARY_WALL_OPEN, e_right=er, b_right=br)


@pytest.mark.parametrize("sort_every", [0, 1, 3])
@pytest.mark.parametrize("name", golden_names("tristan_wall"))
def test_tristan_wall_golden_vectors(pg, name, sort_every):
    """The reference's own explicit wall runs on the FP64 path: the unfused
    push and zigzag (sort_every 0) and the fused tile kernel (sorted
    particles; escaped ones wait marked for the sort every third step)."""
    f = load(name)
    st = f["state"]
    w, er, br = wall_of(f)
    sim = tristan_sim(pg, st, 1, sort_every, er, br)
    sim.upload_state(st)
    sim.buneman_step(f["steps"])
    E, B, J = sim.download_fields()
    b = st.box
    assert rel_err(yee_physical(E, b, "E"), yee_physical(f["E"], b, "E")) < TOL64
    assert rel_err(yee_physical(B, b, "B"), yee_physical(f["B"], b, "B")) < TOL64
    assert rel_err(J, f["extra"]["J"].reshape(J.shape)) < TOL64
    escaped = 0
    for s, o in enumerate(f["out"]):
        keep = survivors(o)
        escaped += len(o["x"]) - len(keep)
        got = by_id(sim.download_particles(s))
        assert np.array_equal(got["id"], keep)
        xg, yg, zg = I.positions(b, got)
        assert np.abs(xg - o["x"][keep]).max() < 1e-11
        for k in ("px", "py", "pz"):
            assert rel_err(got[k], o[k][keep]) < TOL64
    assert escaped > 0
    sim.close()


def _tristan_state(seed=53):
    st = I.shock_plasma(32, 8, 4, dx=0.5, dt=0.225, ppc=(4, 4, 2), flow_gamma=3.0, theta_e=0.3, seed=seed,
                        first_cell=I.TRISTAN_WALL_NODE)
    for sp in st.species:
        sp["px"][::3] = -sp["px"][::3]
    return st


@pytest.mark.parametrize("real,sort_every", [(1, 1), (1, 0), (0, 1), (0, 2)])
def test_tristan_wall_steps_with_injection_match_oracle(pg, real, sort_every):
    """Reflection, escape and particles appended at the open boundary before
    every explicit step, against the oracle on the same particles: FP64
    1e-11, FP32 particles and fields 1e-5."""
    st = _tristan_state()
    er, br = st.e_right, st.b_right
    sim = tristan_sim(pg, st, real, sort_every, er, br)
    for sp in st.species:
        sim.add_species(sp["q"], sp["m"], sp["w"], 4 * len(sp["cell"]))
    for s, sp in enumerate(st.species):
        sim.upload_particles(s, sp)
    sim.upload_fields(st.E, st.B)
    g = O.make_grid(st.box, wall_x=1, e_right=er, b_right=br)
    spo = copy_species(st.species)
    for sp in spo:
        sp["id"] = np.arange(len(sp["cell"]), dtype=np.int32)
    nxt = [len(sp["cell"]) for sp in spo]
    E, B = st.E.copy(), st.B.copy()
    rng = np.random.default_rng(9)
    for step in range(5):
        for s, new in enumerate(_inject(st, step, rng)):
            sim.append_particles(s, new)
            for k in ("cell", "ox", "oy", "oz", "px", "py", "pz"):
                spo[s][k] = np.concatenate([spo[s][k], new[k]]).astype(spo[s][k].dtype)
            spo[s]["id"] = np.concatenate([spo[s]["id"], np.arange(nxt[s], nxt[s] + len(new["cell"]), dtype=np.int32)])
            nxt[s] += len(new["cell"])
        sim.buneman_step(1)
        J = O.buneman_step(g, spo, E, B)
    tol = TOL64 if real else TOL32
    Eg, Bg, Jg = sim.download_fields()
    b = st.box
    assert rel_err(yee_physical(Eg, b, "E"), yee_physical(E, b, "E")) < tol
    assert rel_err(yee_physical(Bg, b, "B"), yee_physical(B, b, "B")) < tol
    assert rel_err(Jg, J.reshape(Jg.shape)) < tol
    escaped = 0
    for s in range(len(spo)):
        got = by_id(sim.download_particles(s))
        ref = by_id({k: v for k, v in spo[s].items() if isinstance(v, np.ndarray)})
        escaped += nxt[s] - len(ref["id"])
        assert np.array_equal(got["id"], ref["id"])
        xg, _, _ = I.positions(b, got)
        xr, _, _ = I.positions(b, ref)
        assert np.abs(xg - xr).max() < (1e-11 if real else 1e-5) * b.nx * b.dx
        for k in ("px", "py", "pz"):
            assert rel_err(got[k], ref[k]) < tol
    assert escaped > 0
    # the density pass of the same wall box (reflected fold at the wall,
    # open-boundary fold into the last cell)
    sim.updateDensityParameters()
    conc, en, vel, rho = O.density_moments(g, spo)
    for s in range(len(spo)):
        c, e, v, r = sim.download_density(s)
        assert rel_err(c, conc[s]) < tol
        assert rel_err(e, en[s]) < tol
        assert rel_err(v, vel[s]) < tol
    assert rel_err(r, rho) < tol
    sim.close()


def test_tristan_wall_fill_starts_at_the_reflecting_wall(pg):
    st = _tristan_state()
    sim = tristan_sim(pg, st, 0, 1, st.e_right, st.b_right)
    sid = sim.add_species(-1.0, 1.0, 0.01, 8 * st.box.ncells)
    sim.fill_species(sid, 2, seed=3, theta=0.01, drift_gamma=1.5, alternate_drift=-1)
    d = sim.download_particles(sid)
    i = d["cell"] % st.box.nx
    assert i.min() == I.TRISTAN_WALL_NODE and i.max() == st.box.nx - 3
    assert len(d["cell"]) == 2 * (st.box.nx - 2 - I.TRISTAN_WALL_NODE) * st.box.ny * st.box.nz
    sim.close()
