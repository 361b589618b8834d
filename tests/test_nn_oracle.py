"""The FP64 network restatement checks itself: analytic gradients against
central finite differences (CPU)."""
import numpy as np

import nn_oracle as NN


def _case(seed=0, shape=(2, 4, 4, 8)):
    rng = np.random.default_rng(seed)
    p = NN.init_params(seed).astype(np.float64)
    offs, n = NN.layer_offsets()
    for name, ci, co, w0, b0 in offs:   # non-zero biases so every ReLU sees both signs
        p[b0:b0 + co] = 0.05 * rng.standard_normal(co)
    x0 = np.zeros(shape + (16,))
    x0[..., :NN.IN_CH] = rng.standard_normal(shape + (NN.IN_CH,))
    t = rng.standard_normal(shape + (NN.OUT_CH,))
    return p, x0, t


def test_parameter_count_and_flops():
    # the layers plus the preconditioner's identity gate
    assert NN.n_params() == sum(27 * ci * co + co for _, ci, co, _ in NN.LAYERS) + 1
    assert 1.0e5 < NN.flops_per_voxel() < 1.5e5


def test_gradients_match_finite_differences():
    p, x0, t = _case()
    L, g = NN.loss_and_grad(p, x0, t)
    rng = np.random.default_rng(5)
    offs, n = NN.layer_offsets()
    idx = []
    for name, ci, co, w0, b0 in offs:
        cin_real = NN.IN_CH if name == "e0a" else ci
        cout_real = NN.OUT_CH if name == "head" else co
        for _ in range(3):
            tap, o, i = rng.integers(27), rng.integers(cout_real), rng.integers(cin_real)
            idx.append(w0 + (tap * co + o) * ci + i)
        idx.append(b0 + rng.integers(cout_real))
    h = 1e-6
    for k in idx:
        pp, pm = p.copy(), p.copy()
        pp[k] += h
        pm[k] -= h
        fd = (NN.loss_and_grad(pp, x0, t)[0] - NN.loss_and_grad(pm, x0, t)[0]) / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 * max(1.0, abs(g).max()) + 1e-4 * abs(fd), (k, fd, g[k])


def test_padding_channels_get_no_gradient():
    p, x0, t = _case(1)
    _, g = NN.loss_and_grad(p, x0, t)
    offs, _ = NN.layer_offsets()
    name, ci, co, w0, b0 = offs[0]
    W = g[w0:b0].reshape(27, co, ci)
    assert np.all(W[:, :, NN.IN_CH:] == 0)
    name, ci, co, w0, b0 = offs[-1]
    W = g[w0:b0].reshape(27, co, ci)
    assert np.all(W[:, NN.OUT_CH:, :] == 0) and np.all(g[b0 + NN.OUT_CH:b0 + co] == 0)
