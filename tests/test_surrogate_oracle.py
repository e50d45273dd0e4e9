"""The FP64 oracle of the surrogate network (oracle/surrogate.c) pinned on
its own: backpropagation against central finite differences, the loss
against the forward pass, and the pooling / combine layout against numpy.
The GPU kernels are then checked against this oracle (test_gpu_surrogate.py).
"""
import numpy as np
import pytest


def small_net(orc, rng, cin=3, width=4, cout=2, kernels=(3, 1, 1, 3)):
    n = orc.surr_num_params(cin, width, cout, kernels)
    return rng.standard_normal(n) * 0.4


@pytest.mark.parametrize("kernels", [(3, 1, 1, 3), (1, 3, 3, 1)])
def test_oracle_backprop_matches_finite_differences(oracle_lib, kernels):
    orc = oracle_lib
    rng = np.random.default_rng(3)
    cin, width, cout, R, B, margin = 3, 4, 2, 6, 2, 1
    p = small_net(orc, rng, cin, width, cout, kernels)
    x = rng.standard_normal((B, cin, R, R))
    t = rng.standard_normal((B, cout, R, R))
    loss, g = orc.surr_loss_grad(x, t, p, width, kernels, margin)
    h = 1e-6
    idx = rng.choice(len(p), 40, replace=False)
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        lp, _ = orc.surr_loss_grad(x, t, pp, width, kernels, margin)
        lm, _ = orc.surr_loss_grad(x, t, pm, width, kernels, margin)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, g[i])


def test_oracle_loss_is_forward_mse(oracle_lib):
    orc = oracle_lib
    rng = np.random.default_rng(4)
    kernels, width, cout, margin = (3, 1, 1, 3), 5, 2, 2
    p = small_net(orc, rng, 3, width, cout, kernels)
    x = rng.standard_normal((2, 3, 8, 8))
    t = rng.standard_normal((2, cout, 8, 8))
    y = orc.surr_forward(x, p, width, cout, kernels)
    loss, _ = orc.surr_loss_grad(x, t, p, width, kernels, margin)
    inner = (y - t)[:, :, margin:-margin, margin:-margin]
    assert abs(loss - np.mean(inner ** 2)) <= 1e-12 * max(1.0, loss)


def test_oracle_pool_and_combine_layout(oracle_lib):
    orc = oracle_lib
    rng = np.random.default_rng(5)
    f, M = 2, 16
    d = rng.random((M, M))
    pooled = orc.surr_pool(d, f)
    np.testing.assert_allclose(pooled, d.reshape(M // f, f, M // f, f).mean(axis=(1, 3)), rtol=1e-14)
    # a constant coarse field upsamples to f times the constant; the residual
    # channel a f + b lands on fine bin (I f + a, J f + b)
    R = M // f
    cex = np.full((R, R), 0.5)
    cey = np.full((R, R), -0.25)
    y = np.zeros((2 * f * f, R, R))
    y[1, 3, 4] = 1.0        # Ex residual, sub-bin (0, 1) of coarse bin (3, 4)
    y[f * f + 2, 5, 6] = 2.0  # Ey residual, sub-bin (1, 0) of coarse bin (5, 6)
    ex, ey = orc.surr_combine(cex, cey, y, 3.0, f)
    expect_x = np.full((M, M), 1.0)
    expect_y = np.full((M, M), -0.5)
    expect_x[3 * f + 0, 4 * f + 1] += 3.0
    expect_y[5 * f + 1, 6 * f + 0] += 6.0
    np.testing.assert_allclose(ex, expect_x, atol=1e-14)
    np.testing.assert_allclose(ey, expect_y, atol=1e-14)
