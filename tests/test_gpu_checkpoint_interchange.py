"""The binary checkpoint as the interchange format between the GPU and host
code: a checkpoint the GPU writes is read on the host and continued by the
oracle, and a checkpoint written on the host from a seeded state is loaded
and continued by the GPU; both against the GPU's own continuation.  Needs a
GB300."""
import numpy as np
import pytest

import pyoracle as O
from fixtures import copy_species, rel_err
from picpp_gb300 import checkpoint as K
from picpp_gb300 import initstate as I

pytestmark = pytest.mark.gpu

TOL64 = 1e-11


@pytest.fixture(scope="module")
def pg():
    import picpp_gb300 as P
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    P.load_library()
    return P


def _noisy(st, seed):
    rng = np.random.default_rng(seed)
    st.E = st.E + 0.05 * rng.standard_normal(st.E.shape)
    st.B = st.B + 0.05 * rng.standard_normal(st.B.shape)
    return st


def _by_id(d):
    o = np.argsort(d["id"])
    return {k: v[o] for k, v in d.items()}


def _oracle_steps(st, solver, steps):
    sp = copy_species(st.species)
    if solver == 0:
        g = O.make_grid(st.box)
        E, B = st.E.copy(), st.B.copy()
        for _ in range(steps):
            O.buneman_step(g, sp, E, B)
    else:
        g = O.make_grid(st.box, pressure_compat=0)
        E, B = st.E.reshape(-1).copy(), st.B.reshape(-1).copy()
        for _ in range(steps):
            O.implicit_step(g, sp, E, B)
    return sp, E.reshape(-1), B.reshape(-1)


def _gpu(pg, st, solver):
    if solver == 0:
        return pg.GpuSimulation(st.box, pg.BUNEMAN, particle_real=1, sort_every=1, tile=(4, 4, 4))
    return pg.GpuSimulation(st.box, pg.IMPLICIT, particle_real=1, pressure_compat=0, sort_every=1, tile=(4, 4, 4))


def _steps(pg, sim, solver, n):
    for _ in range(n):
        if solver == 0:
            sim.buneman_step(1)
        else:
            sim.implicit_step(pg.solve_opts(pg.GMRES_REFERENCE))


def _state(solver):
    if solver == 0:
        return _noisy(I.buneman_plasma(8, 8, 8, ppc=3, seed=61), 62)
    return _noisy(I.beams_plasma(8, 8, 8, ppc=2, beam_gamma=2.0, dt=0.2, seed=63), 64)


@pytest.mark.parametrize("solver", [0, 1])
def test_gpu_checkpoint_continues_on_the_oracle(pg, tmp_path, solver):
    st = _state(solver)
    sim = _gpu(pg, st, solver)
    sim.upload_state(st)
    _steps(pg, sim, solver, 2)
    path = str(tmp_path / "gpu.ckpt")
    sim.save_checkpoint(path)
    ck = K.read(path)
    assert ck.solver == solver and ck.particle_real == 1 and ck.step == 2 and ck.sorted
    mid = K.to_state(ck)
    _steps(pg, sim, solver, 2)
    E, B, _ = sim.download_fields()
    spo, Eo, Bo = _oracle_steps(mid, solver, 2)
    assert rel_err(E.reshape(-1), Eo) < TOL64
    assert rel_err(B.reshape(-1), Bo) < TOL64
    for s in range(len(st.species)):
        got = _by_id(sim.download_particles(s))
        for k in ("px", "py", "pz"):
            assert rel_err(got[k], spo[s][k]) < TOL64
        assert np.array_equal(got["cell"], spo[s]["cell"])
    sim.close()


@pytest.mark.parametrize("solver", [0, 1])
def test_host_written_checkpoint_continues_on_the_gpu(pg, tmp_path, solver):
    st = _state(solver)
    path = str(tmp_path / "host.ckpt")
    K.write(path, K.from_state(st, solver, 1, step=5))
    sim = _gpu(pg, st, solver)
    sim.load_checkpoint(path)
    _steps(pg, sim, solver, 2)
    E, B, _ = sim.download_fields()
    spo, Eo, Bo = _oracle_steps(st, solver, 2)
    assert rel_err(E.reshape(-1), Eo) < TOL64
    assert rel_err(B.reshape(-1), Bo) < TOL64
    for s in range(len(st.species)):
        got = _by_id(sim.download_particles(s))
        for k in ("px", "py", "pz"):
            assert rel_err(got[k], spo[s][k]) < TOL64
    # the GPU's next checkpoint carries the step count on
    sim.save_checkpoint(path)
    assert K.read(path).step == 7
    sim.close()
