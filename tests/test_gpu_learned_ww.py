"""Learned weight windows and split-to-slots on the deep-penetration shield
(GPU).

The importance network is trained on the GPU from a pilot run's mesh flux
tally; its windows must raise the back-face figure of merit over plain
transport while the back-face flux agrees with plain and MAGIC runs.
Split-to-slots mode changes which random numbers a split particle uses, not
the expected tallies: fixed windows with and without it must agree."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _layers(path, split, batches=6):
    from openmc_gb300 import lib
    lib.init(directory=path)
    try:
        lib.settings.xs_fp32 = 1
        lib.settings.split_to_slots = split
        lib.simulation_init()
        sec = 0
        for _ in range(batches):
            lib.next_batch()
            sec += lib.last_batch()["secondaries"]
        m, s = lib.tally_mean_std(lib.tally_ids()[2])
        lib.simulation_finalize()
    finally:
        lib.settings.split_to_slots = 0
        lib.finalize()
    return m.ravel(), s.ravel(), sec


def test_split_to_slots_unbiased(built, tmp_path):
    from openmc_gb300 import configs
    from openmc_gb300 import model as om
    mesh = om.RegularMesh()
    mesh.dimension = [12, 1, 1]
    mesh.lower_left = [0.0, -25.0, -25.0]
    mesh.upper_right = [120.0, 25.0, 25.0]
    # windows falling 2x per 10 cm, roughly the flux of this shield
    lower = 0.5 * 2.0 ** (-np.arange(12.0))
    ww = om.WeightWindows(mesh, lower, upper_bound_ratio=5.0, energy_bounds=[0.0, 2.0e7 * 1.000001])
    m, path = configs.shield(tmp_path, particles=100_000, batches=6, n_points=2000, length=120.0,
                             mesh_dim=(12, 2, 2), weight_windows=ww, density_scale=0.1)
    m.export_to_model_xml(path)
    ma, sa, na = _layers(path, 0)
    mb, sb, nb = _layers(path, 1)
    assert na > 0 and nb > 0
    ok = (sa > 0) & (sb > 0)
    z = np.abs(ma - mb)[ok] / np.hypot(sa, sb)[ok]
    assert ok.sum() >= 10
    assert z.max() < 4.0, z
    assert (z > 3.0).sum() <= 1, z


def test_learned_windows_raise_figure_of_merit(built, tmp_path):
    from openmc_gb300 import shield_study
    out = shield_study.run(tmp_path, length=120.0, mesh_dim=(120, 5, 5), n_points=2000,
                           pilot_particles=200_000, pilot_batches=3, particles=200_000, batches=8,
                           steps=800)
    print(out)
    lw = out["learned"]
    assert lw["loss_last"] < 0.2 * lw["loss_first"], lw
    assert lw["secondaries"] > 0
    assert out["plain"]["back_mean"] > 0
    assert lw["fom_gain"] >= 3.0, out
    # unbiased: back-face means agree within 3.5 combined sigma
    assert out["z_learned_plain"] < 3.5, out
    assert out["z_magic_plain"] < 3.5, out
