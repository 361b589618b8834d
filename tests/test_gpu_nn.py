"""Learned preconditioner on the GPU: the network's forward pass and every
parameter gradient against the FP64 numpy restatement, training on a box
operator, and flexible GMRES with it (including the fall back to plain
GMRES).  Needs a GB300."""
import numpy as np
import pytest

import nn_oracle as NN
import pyoracle as O
from fixtures import rel_err
from picpp_gb300 import initstate as I

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pg():
    import picpp_gb300 as P
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    P.load_library()
    return P


def bf16(a):
    """Round to the nearest BF16 (ties to even), as the device input does."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def params(seed):
    rng = np.random.default_rng(seed)
    p = NN.init_params(seed)
    offs, _ = NN.layer_offsets()
    for name, ci, co, w0, b0 in offs:
        cout_real = NN.OUT_CH if name == "head" else co
        p[b0:b0 + cout_real] = 0.05 * rng.standard_normal(cout_real)
    return p


def net_input(shape, seed):
    rng = np.random.default_rng(seed)
    x0 = np.zeros(shape + (16,), dtype=np.float32)
    x0[..., :3] = rng.standard_normal(shape + (3,))
    x0[..., 3:6] = -0.3 * rng.random(shape + (3,))
    return x0


def sim_box(pg, n=8):
    box = I.Box(n, n, n, 0.5, 0.5, 0.5, 0.5)
    return pg.GpuSimulation(box, pg.IMPLICIT, particle_real=1)


# boxes smaller than one 1 x 16 x 8 output brick and spanning several, with
# ragged edges
@pytest.mark.parametrize("shape", [(1, 8, 8, 16), (1, 4, 20, 24)])
def test_forward_matches_oracle(pg, shape):
    sim = sim_box(pg)
    p = params(3)
    sim.nn_set_params(p)
    x0 = net_input(shape, 4)
    out = sim.nn_forward(x0)
    ref = NN.forward(p.astype(np.float64), bf16(x0).astype(np.float64))
    # BF16 activations between layers, FP32 accumulation
    assert rel_err(out[..., :3], ref[..., :3]) < 3e-2
    assert np.all(out[..., 3:] == 0)
    assert np.array_equal(sim.nn_get_params(), p)


def test_gradients_match_oracle(pg):
    sim = sim_box(pg)
    p = params(5)
    sim.nn_set_params(p)
    # level 0 (16 x 20 x 16): two output bricks in h, the second ragged
    x0 = net_input((2, 16, 20, 16), 6)
    t = np.random.default_rng(7).standard_normal((2, 16, 20, 16, 3)).astype(np.float32)
    L, g = sim.nn_loss_grad(x0, t)
    xb = bf16(x0).astype(np.float64)
    # the restatement rounding where the device rounds (weights, stored
    # activations, back-propagated gradients to BF16): per-layer agreement
    Le, ge = NN.loss_and_grad(p.astype(np.float64), xb, t.astype(np.float64), bf16=True)
    assert abs(L - Le) <= 2e-3 * Le
    offs, _ = NN.layer_offsets()
    for name, ci, co, w0, b0 in offs:
        # the coarsest level sums over 64x fewer voxels: a BF16 rounding
        # that differs between FP32 and FP64 accumulation weighs more there
        tol = 5e-2 if name.startswith("e2") else 2e-2
        assert rel_err(g[w0:b0], ge[w0:b0]) < tol, name
        assert rel_err(g[b0:b0 + co], ge[b0:b0 + co]) < tol, name
    # and the exact FP64 gradient as a whole, within the BF16 noise
    Lo, go = NN.loss_and_grad(p.astype(np.float64), xb, t.astype(np.float64))
    assert abs(L - Lo) <= 2e-2 * Lo
    assert rel_err(g, go) < 5e-2
    # padded channels receive exactly zero gradient
    name, ci, co, w0, b0 = offs[0]
    assert np.all(g[w0:b0].reshape(27, co, ci)[:, :, NN.IN_CH:] == 0)


def hard_operator(n=16, seed=11):
    """A stiff operator: dt = 2 dx, K / dx^2 = (c' theta dt / dx)^2 ~ 4.4."""
    box = I.Box(n, n, n, 0.5, 0.5, 0.5, 2.0, theta=0.5)
    rng = np.random.default_rng(seed)
    N = box.ncells
    mu = -0.02 * rng.random(9 * N)
    for a in range(3):
        mu[4 * a * N:(4 * a + 1) * N] = -0.6 * rng.random(N)
    rhs = rng.standard_normal(3 * N)
    return box, mu, rhs


def test_training_reduces_the_loss_and_fgmres_iterations(pg):
    box, mu, rhs = hard_operator()
    sim = pg.GpuSimulation(box, pg.IMPLICIT, particle_real=1)
    sim.maxwell_apply(mu, rhs)   # uploads the operator
    sim.nn_init(7)
    # white-noise fields, like the right-hand side below
    info = sim.nn_train(steps=1500, batch=2, lr=1e-3, seed=5, smooth_max=0)
    assert info["steps"] == 1500 and info["last_loss"] < 0.2 * info["first_loss"]
    opts = dict(restart=30, max_iter=3000, tol=1e-8)
    _, plain = sim.maxwell_solve(mu, rhs, pg.solve_opts(pg.GMRES_RESTARTED, **opts))
    x, learned = sim.maxwell_solve(mu, rhs, pg.solve_opts(pg.FGMRES_LEARNED, **opts))
    r = O.maxwell_apply(O.make_grid(box), mu, x) - rhs
    assert np.linalg.norm(r) / np.linalg.norm(rhs) <= 1.01e-8
    assert learned["used_fallback"] == 0
    assert learned["iterations"] < plain["iterations"], (learned, plain)


@pytest.mark.parametrize("shape", [(8, 6, 5), (8, 8, 1), (6, 1, 4)])
def test_operator_transpose_is_the_adjoint(pg, shape):
    """<A^T y, x> = <y, A x> for the matrix-free operator and its transpose
    (the training gradient runs through A^T)."""
    box = I.Box(*shape, 0.5, 0.4, 0.3, 0.7)
    rng = np.random.default_rng(8)
    N = box.ncells
    mu = -0.3 * rng.random(9 * N)
    x, y = rng.standard_normal(3 * N), rng.standard_normal(3 * N)
    sim = pg.GpuSimulation(box, pg.IMPLICIT, particle_real=1, tile=(0, 0, 0))
    Ax = sim.maxwell_apply(mu, x)
    Aty = sim.maxwell_apply_transpose(mu, y)
    assert abs(np.dot(Aty, x) - np.dot(y, Ax)) <= 1e-12 * np.linalg.norm(Aty) * np.linalg.norm(x)
    assert rel_err(Ax, O.maxwell_apply(O.make_grid(box), mu, x)) < 1e-13


def test_fgmres_falls_back_to_plain_gmres(pg):
    """A network whose directions are not finite (NaN parameters) ends its
    cycle; the solve finishes with plain GMRES to the same tolerance."""
    box, mu, rhs = hard_operator(8, seed=12)
    sim = pg.GpuSimulation(box, pg.IMPLICIT, particle_real=1)
    sim.nn_set_params(np.full(pg.load_library().pic_nn_param_count(), np.nan, dtype=np.float32))
    x, info = sim.maxwell_solve(mu, rhs, pg.solve_opts(pg.FGMRES_LEARNED, restart=20, max_iter=3000, tol=1e-8))
    assert info["used_fallback"] == 1
    r = O.maxwell_apply(O.make_grid(box), mu, x) - rhs
    assert np.linalg.norm(r) / np.linalg.norm(rhs) <= 1.01e-8


def test_gate_alone_is_the_identity_preconditioner(pg):
    """Zero network, gate 1: z = r, so FGMRES takes the same iterations as
    plain GMRES and reaches the same tolerance."""
    box, mu, rhs = hard_operator(8, seed=14)
    sim = pg.GpuSimulation(box, pg.IMPLICIT, particle_real=1)
    p = np.zeros(pg.load_library().pic_nn_param_count(), dtype=np.float32)
    p[-1] = 1.0
    sim.nn_set_params(p)
    opts = dict(restart=20, max_iter=3000, tol=1e-8)
    _, plain = sim.maxwell_solve(mu, rhs, pg.solve_opts(pg.GMRES_RESTARTED, **opts))
    x, learned = sim.maxwell_solve(mu, rhs, pg.solve_opts(pg.FGMRES_LEARNED, **opts))
    assert learned["used_fallback"] == 0
    assert abs(learned["iterations"] - plain["iterations"]) <= 1, (learned, plain)
    r = O.maxwell_apply(O.make_grid(box), mu, x) - rhs
    assert np.linalg.norm(r) / np.linalg.norm(rhs) <= 1.01e-8


def test_learned_solver_needs_a_network_and_a_box_of_fours(pg):
    box, mu, rhs = hard_operator(8, seed=13)
    sim = pg.GpuSimulation(box, pg.IMPLICIT, particle_real=1)
    with pytest.raises(pg.PicError) as e:
        sim.maxwell_solve(mu, rhs, pg.solve_opts(pg.FGMRES_LEARNED))
    assert e.value.status == 3
    box6 = I.Box(6, 8, 8, 0.5, 0.5, 0.5, 0.5)
    sim6 = pg.GpuSimulation(box6, pg.IMPLICIT, particle_real=1, tile=(0, 0, 0))
    sim6.nn_init(1)
    N = box6.ncells
    with pytest.raises(pg.PicError) as e:
        sim6.maxwell_solve(np.zeros(9 * N), np.ones(3 * N), pg.solve_opts(pg.FGMRES_LEARNED))
    assert e.value.status == 1


def test_training_on_recorded_solve_triples(pg):
    """The plain field solves of a few implicit steps of two runs (species
    reloaded) are recorded as (b, mu, x) triples, the first `capacity` kept;
    training on them lowers the combined supervised and residual loss, and
    FGMRES with the trained network reaches the tolerance on the next system
    of a third run."""
    box = I.Box(16, 16, 8, 0.5, 0.5, 0.5, 0.5, theta=0.5)
    sim = pg.GpuSimulation(box, pg.IMPLICIT, particle_real=0, pressure_compat=0, sort_every=1)
    w = I.density_weight(box, 1.0 / (4 * np.pi), 8)
    sim.add_species(-1.0, 1.0, w, 8 * box.ncells)
    sim.add_species(1.0, 25.0, w, 8 * box.ncells)
    E, B = I.zero_fields(box)
    B[2] = 0.5
    opts = pg.solve_opts(pg.GMRES_RESTARTED, restart=30, max_iter=600, tol=1e-8)
    sim.nn_record(5)
    for run in range(2):
        sim.fill_species(0, 8, 10 + 2 * run, 0.01, 10.0, True)
        sim.fill_species(1, 8, 11 + 2 * run, 0.01 / 25, 10.0, True)
        sim.upload_fields(E, B)
        for _ in range(3):
            sim.implicit_step(opts)
    assert sim.nn_record_count() == 5
    sim.nn_init(3)
    info = sim.nn_train(steps=300, batch=2, lr=1e-3, seed=4, source=1, supervised_weight=0.5)
    assert info["last_loss"] < info["first_loss"]
    sim.fill_species(0, 8, 30, 0.01, 10.0, True)
    sim.fill_species(1, 8, 31, 0.01 / 25, 10.0, True)
    sim.upload_fields(E, B)
    sim.implicit_step(opts)
    sim.updateElectroMagneticParameters()
    _, mu, _, rhs = sim.download_moments()
    x, learned = sim.maxwell_solve(mu, rhs, pg.solve_opts(pg.FGMRES_LEARNED, restart=30, max_iter=600, tol=1e-8))
    r = O.maxwell_apply(O.make_grid(box), mu, x) - rhs
    assert np.linalg.norm(r) / np.linalg.norm(rhs) <= 1.01e-8
    sim.nn_record(0)
    assert sim.nn_record_count() == 0
    sim.close()


def test_convolution_wait_bound_reports_and_the_context_stays_usable(pg):
    """A one-poll bound on the convolutions' MMA-completion wait makes the
    wait run out: the forward pass returns PIC_ERR_CUDA, the CTAs still wait
    for their MMAs (full bound) before releasing tensor memory, and with the
    bound restored the same context computes the same output as before."""
    box = I.Box(16, 16, 8, 0.5, 0.5, 0.5, 0.5)
    sim = pg.GpuSimulation(box, pg.IMPLICIT, particle_real=1)
    sim.nn_set_params(NN.init_params(3))
    rng = np.random.default_rng(21)
    x0 = np.zeros((1, 8, 16, 16, 16), dtype=np.float32)
    x0[..., :6] = rng.standard_normal((1, 8, 16, 16, 6))
    before = sim.nn_forward(x0)
    sim.nn_wait_limit(1)
    with pytest.raises(pg.PicError) as e:
        sim.nn_forward(x0)
    assert e.value.status == 2
    sim.nn_wait_limit(0)
    after = sim.nn_forward(x0)
    assert np.array_equal(after, before)
    sim.close()
