"""Host logic of the learned weight windows (CPU): mesh centres, features,
training pairs and MAGIC-normalised bounds."""
import numpy as np
import pytest

pytest.importorskip("openmc_gb300.lib", reason="library not built")


def _geom():
    from openmc_gb300.learned_ww import MeshGeometry
    return MeshGeometry(np.array([0.0, -5.0, -5.0]), np.array([20.0, 5.0, 5.0]), (4, 2, 2),
                        np.array([0.0, 1.0, 1e3, 2e7]))


def test_centres_x_fastest():
    g = _geom()
    c = g.centres()
    assert c.shape == (16, 3)
    np.testing.assert_allclose(c[0], [2.5, -2.5, -2.5])
    np.testing.assert_allclose(c[1], [7.5, -2.5, -2.5])
    np.testing.assert_allclose(c[4], [2.5, 2.5, -2.5])
    np.testing.assert_allclose(c[8], [2.5, -2.5, 2.5])


def test_training_pairs_and_features():
    from openmc_gb300.learned_ww import training_pairs
    g = _geom()
    # flux falling 10x per x bin, energy groups scaled 1, 2, 3
    c = g.centres()
    mean = np.zeros((g.n_mesh, g.n_groups))
    for e in range(3):
        mean[:, e] = (e + 1) * 10.0 ** (-(c[:, 0] - 2.5) / 5.0)
    std = 0.1 * mean
    std[3, 2] = 5 * mean[3, 2]  # rel err 5: excluded
    mean[5, 0] = 0.0            # unscored: excluded
    x4, t, w, f = training_pairs(mean, std, g)
    assert len(t) == g.n_mesh * g.n_groups - 2
    assert np.all(np.abs(x4) <= 1.0 + 1e-12)
    np.testing.assert_allclose(w.mean(), 1.0)
    np.testing.assert_allclose(t.mean(), 0.0, atol=1e-12)
    # the standardised target maps back to log flux
    inp = f.inputs().reshape(g.n_groups, g.n_mesh, 4)
    assert inp[0, 1, 0] > inp[0, 0, 0]  # x feature increases with x index
    assert inp[2, 0, 3] > inp[0, 0, 3]  # log-E feature increases with group


def test_bounds_follow_magic_normalisation():
    from openmc_gb300.learned_ww import bounds_from_log_flux
    g = _geom()
    lf = np.log(np.arange(1, g.n_mesh * g.n_groups + 1, dtype=float))
    lo, up = bounds_from_log_flux(lf, g, ratio=5.0)
    per = lo.reshape(g.n_groups, g.n_mesh)
    np.testing.assert_allclose(per.max(axis=1), 0.5)
    np.testing.assert_allclose(up, 5.0 * lo)
    flux = np.exp(lf).reshape(g.n_groups, g.n_mesh)
    np.testing.assert_allclose(per, flux / (2 * flux.max(axis=1, keepdims=True)))


def test_extrapolated_bounds_are_floored():
    from openmc_gb300.learned_ww import bounds_from_log_flux
    g = _geom()
    lf = -np.arange(g.n_mesh * g.n_groups, dtype=float) * 2.0
    scored = np.zeros(g.n_mesh * g.n_groups, bool)
    scored[:4] = True  # group 0, first four bins
    lo, _ = bounds_from_log_flux(lf, g, scored=scored, max_extrapolation=100.0)
    per = lo.reshape(g.n_groups, g.n_mesh)
    floor = per[0, :4].min() / 100.0
    assert np.all(per[0, 4:] >= floor * (1 - 1e-12))
    np.testing.assert_allclose(per[0, :4], 0.5 * np.exp(lf[:4] - lf[:16].max()))
    # groups without scored bins keep the plain prediction
    np.testing.assert_allclose(per[1], 0.5 * np.exp(lf[16:32] - lf[16:32].max()))
