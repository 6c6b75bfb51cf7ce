"""Learned weight windows on a reduced deep-penetration shield (GPU).

The importance network is trained on the GPU from a pilot run's mesh flux
tally; its windows must raise the back-face figure of merit over plain
transport while the back-face flux agrees with plain and MAGIC runs."""
import pytest

pytestmark = pytest.mark.gpu


def test_learned_windows_raise_figure_of_merit(built, tmp_path):
    from openmc_gb300 import shield_study
    out = shield_study.run(tmp_path, length=80.0, mesh_dim=(80, 5, 5), n_points=2000,
                           pilot_particles=200_000, pilot_batches=3, particles=200_000, batches=8,
                           steps=800)
    lw = out["learned"]
    print(out)
    assert lw["loss_last"] < 0.2 * lw["loss_first"], lw
    assert lw["secondaries"] > 0
    assert out["plain"]["back_mean"] > 0
    assert lw["fom_gain"] >= 3.0, out
    # unbiased: back-face means agree within 3.5 combined sigma
    assert out["z_learned_plain"] < 3.5, out
    assert out["z_magic_plain"] < 3.5, out
