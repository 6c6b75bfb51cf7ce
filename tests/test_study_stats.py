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
    r = bench.compare_tallies(a, b, 1000, 1000)
    assert r["bins_scored_by_both"] == 100_000
    assert abs(r["share_within_3_sigma"] - 0.9973) < 0.002
    # ~2000 degrees of freedom per bin: the t law's tail is the normal one
    assert abs(r["expected_share_beyond_3_sigma_t"] - 0.0027) < 2e-4
    assert abs(r["mean_signed_z_converged"]) < 5 * r["mean_signed_z_converged_stderr"]
    assert r["converged_bins"] == 100_000     # 0.5 % < 1 % in both
    # the largest relative difference is a few combined relative errors
    assert r["max_rel_diff_converged"] < 6 * r["max_combined_rel_err_converged"]
    assert abs(r["total_z"]) < 4


def test_bench_tally_comparison_few_batches():
    """Sigmas from 5 batches each: z follows a t law with 4 to 8 degrees of
    freedom, whose share beyond 3 is ~1.7-4 %, not the normal 0.27 %; the
    observed share lies between the comparison's pooled and per-bin Welch
    expectations."""
    import bench
    rng = np.random.default_rng(8)
    n, nb = 50_000, 5
    x = rng.normal(1.0, 0.05, size=(nb, n))
    y = rng.normal(1.0, 0.05, size=(nb, n))
    a = (x.mean(0), x.std(0, ddof=1) / np.sqrt(nb))
    b = (y.mean(0), y.std(0, ddof=1) / np.sqrt(nb))
    r = bench.compare_tallies(a, b, nb, nb)
    assert r["expected_share_beyond_3_sigma_t"] > 0.01
    assert r["expected_share_beyond_3_sigma_pooled_t"] - 0.002 < r["share_beyond_3_sigma"] \
        < r["expected_share_beyond_3_sigma_t"] + 0.002


def test_bench_algorithmic_bytes():
    """Per-event byte model (FP32 tables, 2 coordinate levels): XS 36 B per
    event + 16 B per calculation + 64 B per nuclide lookup; advance 280 B
    per event; track-length tally 16 B per mesh segment (in the advance
    kernel when scoring is not deferred); surface 312 B per crossing;
    collision 128 B + 64 B per nuclide lookup."""
    import bench
    q = {"xs_events": 10, "xs_calc": 5, "xs_nuclide_lookups": 20, "mesh_segments": 12,
         "collision_nuclide_lookups": 3, "surface": 4, "collision": 2}
    zero = {k: 0 for k in q}
    b = bench.algorithmic_bytes({"queue": q, "tail": zero}, levels=2, fp32=True)
    assert b["xs"] == 10 * 36 + 5 * 16 + 20 * 64
    assert b["advance"] == 10 * 280 and b["tally"] == 12 * 16
    b_inline = bench.algorithmic_bytes({"queue": q, "tail": zero}, levels=2, fp32=True, deferred=False)
    assert b_inline["advance"] == 10 * 280 + 12 * 16 and "tally" not in b_inline
    assert b["surface"] == 4 * 312
    assert b["collision"] == 2 * 128 + 3 * 64
    assert b["xs+advance+surface"] == b["xs"] + b["advance"] + b["surface"]
    assert b["tail"] == 0
    b64 = bench.algorithmic_bytes({"queue": zero, "tail": q}, levels=2, fp32=False)
    assert b64["tail"] == (10 * 36 + 5 * 16 + 20 * 100) + (10 * 280 + 12 * 16) + 4 * 312 + (2 * 128 + 3 * 100)
