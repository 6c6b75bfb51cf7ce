"""The importance-network oracle against finite differences (CPU only).

The network has no reference counterpart, so its oracle is pinned by
mathematics: in FP64 (no BF16 rounding) the analytic gradient of the
weighted squared-error loss must agree with central differences."""
import numpy as np

from oracle import mlp as om


def _data(n, seed):
    rng = np.random.default_rng(seed)
    x = rng.uniform(-1, 1, size=(n, 4))
    t = -2.0 * x[:, 0] + 0.5 * np.sin(3 * x[:, 1]) + 0.3 * x[:, 2] ** 2 - 0.4 * x[:, 3]
    w = rng.uniform(0.5, 1.5, size=n)
    return x, t, w


def test_param_count():
    assert om.N_PARAMS == 33793
    p = om.init_params(3)
    assert p.size == om.N_PARAMS
    np.testing.assert_array_equal(om.pack(om.unpack(p)), p)


def test_fp64_gradient_matches_finite_differences():
    x, t, w = _data(40, 1)
    p = om.init_params(7)
    loss, g = om.loss_and_grad(p, x, t, w, bf=False)
    rng = np.random.default_rng(2)
    # a few entries of every tensor, biases included
    idx, k = [], 0
    for name, shape in om.SIZES:
        n = int(np.prod(shape))
        idx += list(k + rng.choice(n, size=min(n, 6), replace=False))
        k += n
    h = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        lp, _ = om.loss_and_grad(pp, x, t, w, bf=False)
        lm, _ = om.loss_and_grad(pm, x, t, w, bf=False)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])) + 1e-8, (i, fd, g[i])


def test_bf16_rounding():
    v = np.array([1.0, 1.00390625, 1.005859375, -3.14159265, 0.0, 65504.0])
    r = om.bf16(v)
    assert r[0] == 1.0
    assert r[1] == 1.0  # halfway: ties to even (mantissa 0)
    assert r[2] == 1.0078125  # above halfway rounds up
    assert abs(r[3] - -3.140625) < 1e-12
    assert r[4] == 0.0
    assert r[5] == 65536.0


def test_bf16_gradient_close_to_fp64():
    x, t, w = _data(256, 4)
    p = om.init_params(5)
    _, g64 = om.loss_and_grad(p, x, t, w, bf=False)
    _, g16 = om.loss_and_grad(p, x, t, w, bf=True)
    rel = np.linalg.norm(g16 - g64) / np.linalg.norm(g64)
    assert rel < 0.05


def test_adam_first_step_is_signed_lr():
    p = np.zeros(5)
    g = np.array([1.0, -2.0, 0.5, 0.0, 3.0])
    p1, m, v = om.adam(p, np.zeros(5), np.zeros(5), g, 1, 1e-3)
    np.testing.assert_allclose(p1[[0, 1, 2, 4]], [-1e-3, 1e-3, -1e-3, -1e-3], rtol=1e-6)
    assert p1[3] == 0.0
