"""Host-side statistics of the studies and of the bench (CPU): bin-by-bin
tally agreement and the algorithmic-bytes model of the roofline."""
import numpy as np
import pytest


def _pair(rng, n, bias=0.0, rel=0.05):
    """Two independent estimates (mean, std of the mean) of the same n bins;
    a is scaled by (1 + bias)."""
    truth = rng.uniform(1.0, 10.0, n)
    sd = rel * truth
    a = truth * (1.0 + bias) + rng.normal(0.0, 1.0, n) * sd
    b = truth + rng.normal(0.0, 1.0, n) * sd
    return (a, sd), (b, sd)


def test_agreement_of_unbiased_estimates():
    fs = pytest.importorskip("openmc_gb300.full_scale_study")
    a, b = _pair(np.random.default_rng(5), 200_000)
    r = fs.agreement(a, b)
    assert r["scored_by_both"] == 200_000 and r["converged_by_both"] == 200_000
    assert abs(r["share_within_3_sigma"] - 0.9973) < 0.001
    assert abs(r["converged_mean_signed_z"]) < 0.01
    assert abs(r["converged_share_above_3_sigma"] - r["converged_share_below_3_sigma"]) < 0.001


def test_agreement_shows_a_bias_as_a_shifted_signed_z():
    fs = pytest.importorskip("openmc_gb300.full_scale_study")
    # a 10 % low against 5 % errors on both: mean z = -0.1 / (0.05 sqrt 2)
    a, b = _pair(np.random.default_rng(6), 200_000, bias=-0.1)
    r = fs.agreement(a, b)
    assert abs(r["converged_mean_signed_z"] + 0.1 / (0.05 * np.sqrt(2.0))) < 0.05
    assert r["converged_share_below_3_sigma"] > 10 * r["converged_share_above_3_sigma"]


def test_agreement_skips_unscored_and_unconverged_bins():
    fs = pytest.importorskip("openmc_gb300.full_scale_study")
    a = (np.array([1.0, 0.0, 2.0, 3.0]), np.array([0.01, 0.0, 1.0, 0.1]))
    b = (np.array([1.0, 5.0, 2.0, 3.0]), np.array([0.01, 0.5, 1.0, 0.1]))
    r = fs.agreement(a, b)
    assert r["scored_by_both"] == 3          # bin 1 unscored by a
    assert r["converged_by_both"] == 2       # bin 2 at 50 % relative error
    assert r["max_z"] == 0.0 and r["converged_mean_signed_z"] == 0.0


def test_bench_tally_comparison():
    import bench
    a, b = _pair(np.random.default_rng(7), 100_000, rel=0.005)
    r = bench.compare_tallies(a, b)
    assert r["bins_scored_by_both"] == 100_000
    assert abs(r["share_within_3_sigma"] - 0.9973) < 0.002
    assert r["converged_bins"] == 100_000     # 0.5 % < 1 % in both
    # the largest relative difference is a few combined relative errors
    assert r["max_rel_diff_converged"] < 6 * r["max_combined_rel_err_converged"]
    assert abs(r["total_z"]) < 4


def test_bench_algorithmic_bytes():
    """Per-event byte model (FP32 tables, 2 coordinate levels): XS 36 B per
    event + 16 B per calculation + 64 B per nuclide lookup; advance 280 B
    per event + 16 B per mesh segment; surface 312 B per crossing; collision
    128 B + 64 B per nuclide lookup."""
    import bench
    q = {"xs_events": 10, "xs_calc": 5, "xs_nuclide_lookups": 20, "mesh_segments": 12,
         "collision_nuclide_lookups": 3, "surface": 4, "collision": 2}
    zero = {k: 0 for k in q}
    b = bench.algorithmic_bytes({"queue": q, "tail": zero}, levels=2, fp32=True)
    assert b["xs"] == 10 * 36 + 5 * 16 + 20 * 64
    assert b["advance"] == 10 * 280 + 12 * 16
    assert b["surface"] == 4 * 312
    assert b["collision"] == 2 * 128 + 3 * 64
    assert b["xs+advance+surface"] == b["xs"] + b["advance"] + b["surface"]
    assert b["tail"] == 0
    b64 = bench.algorithmic_bytes({"queue": zero, "tail": q}, levels=2, fp32=False)
    assert b64["tail"] == (10 * 36 + 5 * 16 + 20 * 100) + (10 * 280 + 12 * 16) + 4 * 312 + (2 * 128 + 3 * 100)
