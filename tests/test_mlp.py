"""The proposal network: its CPU oracle (pinned by finite differences) and the
CUDA training and inference kernels checked against it.

Tolerances of the GPU checks against the BF16-emulating oracle: the kernels
accumulate in FP32 where the oracle accumulates in float64, and a value that
lands within FP32 rounding of a BF16 rounding boundary may round one BF16 ulp
(2^-8 relative) the other way, so outputs are held to 5e-3 of their largest
magnitude and gradients to 2e-2 relative in norm per parameter block, with a
cosine similarity above 0.9995 for the whole vector.
"""
import numpy as np
import pytest

from oracle import mlp_ref as M

OUT_TOL, GRAD_TOL, COS_MIN = 5e-3, 2e-2, 0.9995


def _data(n, n_in, seed):
    rng = np.random.default_rng(seed)
    x = rng.normal(size=(n, n_in)).astype(np.float32)
    y = (np.sin(2.0 * x[:, 0]) + 0.5 * x[:, 1] * x[:, 2 % n_in]).astype(np.float32)
    return x, y


def test_oracle_gradient_matches_finite_differences():
    n_in, depth = 6, 3
    p = M.init_params(n_in, depth, 3)
    x, y = _data(41, n_in, 4)
    x, y = x.astype(np.float64), y.astype(np.float64)
    _, g = M.loss_grad(p, x, y, n_in, depth, emulate=False)
    idx = np.random.default_rng(5).choice(p.size, 40, replace=False)
    h = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (M.loss_grad(pp, x, y, n_in, depth, False)[0] - M.loss_grad(pm, x, y, n_in, depth, False)[0]) / (2 * h)
        assert abs(fd - g[i]) < 1e-7 + 1e-5 * abs(g[i]), (i, fd, g[i])


def test_oracle_bf16_rounding():
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -3.14159, 65504.0], np.float32)
    r = M.bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0                      # tie to even
    assert r[2] == 1.0 + 2 ** -7                            # above the tie rounds up
    assert abs(r[3] + 3.140625) < 1e-12
    assert np.all(np.abs(r - v) <= np.abs(v) * 2 ** -8)


def _blocks(n_in, depth):
    out, off = [], 0
    for l in range(depth):
        ni = n_in if l == 0 else M.WIDTH
        out += [(f"W{l}", off, off + M.WIDTH * ni), (f"b{l}", off + M.WIDTH * ni, off + M.WIDTH * ni + M.WIDTH)]
        off += M.WIDTH * ni + M.WIDTH
    out += [("wo", off, off + M.WIDTH), ("bo", off + M.WIDTH, off + M.WIDTH + 1)]
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("n_in,depth,rows", [(31, 4, 384), (5, 1, 128), (64, 2, 1000)])
def test_forward_and_gradient_match_oracle(gpu_lib, n_in, depth, rows):
    from mepinterp_gb300.mlp import Net
    x, y = _data(rows, n_in, 7)
    with Net(n_in, depth, seed=11) as net:
        p = M.init_params(n_in, depth, 12).astype(np.float32)
        net.params = p
        assert np.array_equal(net.params, p)
        f = net.forward(x)
        f_ref, _ = M.forward(p, x, n_in, depth)
        assert np.abs(f - f_ref).max() < OUT_TOL * np.abs(f_ref).max()
        loss, g = net.loss_grad(x, y)
        loss_ref, g_ref = M.loss_grad(p, x, y, n_in, depth)
    assert abs(loss - loss_ref) < 1e-2 * loss_ref
    for name, a, b in _blocks(n_in, depth):
        err = np.linalg.norm(g[a:b] - g_ref[a:b]) / max(np.linalg.norm(g_ref[a:b]), 1e-30)
        assert err < GRAD_TOL, (name, err)
    cos = float(g @ g_ref / (np.linalg.norm(g) * np.linalg.norm(g_ref)))
    assert cos > COS_MIN


@pytest.mark.gpu
def test_training_reduces_loss_and_is_deterministic(gpu_lib):
    from mepinterp_gb300.mlp import Net
    n_in = 8
    x, y = _data(3000, n_in, 8)
    runs = []
    for _ in range(2):
        with Net(n_in, 4, seed=21) as net:
            hist = net.train(x, y, epochs=60, batch=256, lr=2e-3, seed=5)
            runs.append((hist, net.params, net.forward(x[:500])))
    hist, params, f = runs[0]
    assert hist[-1] < 0.1 * hist[0], hist[[0, -1]]
    assert np.array_equal(params, runs[1][1])                 # bitwise reproducible
    assert np.array_equal(hist, runs[1][0])
    # the trained GPU network and the oracle agree on the trained parameters
    f_ref, _ = M.forward(params, x[:500], n_in, 4)
    assert np.abs(f - f_ref).max() < OUT_TOL * np.abs(f_ref).max()
    # and it generalises to held-out samples
    xt, yt = _data(800, n_in, 99)
    with Net(n_in, 4, seed=0) as net:
        net.params = params
        mse = float(np.mean((net.forward(xt) - yt) ** 2))
    assert mse < 0.2 * float(np.var(yt))


@pytest.mark.gpu
def test_argument_errors(gpu_lib):
    from mepinterp_gb300 import api
    from mepinterp_gb300.mlp import Net
    with pytest.raises(api.MepiError):
        Net(65, 2)
    with Net(4, 2) as net:
        with pytest.raises(api.MepiError):
            net.train(np.zeros((10, 4)), np.zeros(10), batch=100)     # not a multiple of 128
        with pytest.raises(ValueError):
            net.params = np.zeros(3)
