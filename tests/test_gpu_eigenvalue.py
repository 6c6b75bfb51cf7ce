"""Eigenvalue runs on the GPU (src/eigenvalue.cpp, src/physics.cpp:170-285,
src/bank.cpp:76-135) against the oracle and against a known answer.

A reflective cube of one homogeneous mixture of a fissile nuclide and a
light moderator whose cross sections do not depend on energy has
k-infinity = nu Sigma_f / Sigma_a exactly (the reference's
tests/unit_tests/test_temp_interp.py builds its known-answer nuclide the
same way).  FP64 tables: every generation's track-length k, the fission-bank
sizes, the histories of a later generation (which start from the combed,
sorted fission bank of the one before), the tallies and the combined
k-effective equal the oracle's.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DISCRETE = ("kind", "cell", "material", "surface_or_nuclide", "grid_hash", "n_coord")


def run_gpu(path, n_trace=0, cap=256, trace_batch=1, fp32=False, event_based=True):
    from openmc_gb300 import lib
    lib.init(directory=path)
    try:
        lib.settings.event_based = event_based
        lib.settings.xs_fp32 = 1 if fp32 else 0
        lib.settings.trace_batch = trace_batch
        if n_trace:
            lib.set_trace(n_trace, cap)
        lib.simulation_init()
        sites = []
        while True:
            status = lib.next_batch()
            kg, n_sites = lib.k_generation()
            sites.append(n_sites)
            if status != 0:
                break
        out = {"k_generation": kg, "sites": sites, "keff": lib.keff(), "batch": lib.last_batch()}
        if n_trace:
            out["trace"] = lib.get_trace()
        lib.simulation_finalize()
        out["tally"] = lib.tally_results(lib.tally_ids()[0]).copy()
        return out
    finally:
        lib.settings.trace_batch = 1
        lib.settings.event_based = True
        lib.finalize()


def run_oracle(xml, n_trace=0, cap=256, trace_batch=1):
    import oracle
    o = oracle.Oracle(xml)
    if n_trace:
        o.set_trace(n_trace, cap, batch=trace_batch)
    o.run(threads=8)
    return {"keff": o.keff(), "tally": o.tally(0), "trace": o.traces() if n_trace else None}


@pytest.fixture(scope="module")
def medium(built, tmp_path_factory):
    from openmc_gb300 import configs
    d = tmp_path_factory.mktemp("eig")
    m, path = configs.infinite_medium(d, particles=3000, batches=6, inactive=2, n_points=400)
    return m, m.export_to_model_xml(path), path


def test_eigenvalue_generations_match_oracle(medium):
    m, xml, path = medium
    g = run_gpu(path, n_trace=1000, cap=512, trace_batch=3)
    o = run_oracle(xml, n_trace=1000, cap=512, trace_batch=3)
    ok = o["keff"]
    # every generation's track-length k and the sizes of the fission banks
    np.testing.assert_allclose(g["k_generation"], ok["k_generation"], rtol=1e-10, atol=0)
    assert g["sites"][-1] == int(ok["fission_sites"])
    # the traced generation starts from the combed bank of generation 2
    rec, cnt = g["trace"]
    orec, ocnt = o["trace"]
    assert np.array_equal(cnt, ocnt)
    for f in DISCRETE:
        for h in range(len(cnt)):
            n = min(cnt[h], 512)
            assert np.array_equal(rec[f][h, :n], orec[f][h, :n]), (f, h + 1)
    for f in ("E", "dist", "wgt"):
        for h in range(len(cnt)):
            n = min(cnt[h], 512)
            assert np.allclose(rec[f][h, :n], orec[f][h, :n], rtol=1e-6, atol=1e-7 if f == "dist" else 0), (f, h + 1)
    # tallies of the 4 active batches and the combined k-effective
    np.testing.assert_allclose(g["tally"][..., 1].ravel(), o["tally"][:, 1], rtol=1e-5)
    assert abs(g["keff"][0] - ok["k_combined"][0]) <= 1e-9 * ok["k_combined"][0]
    assert abs(g["keff"][1] - ok["k_combined"][1]) <= 1e-6 * ok["k_combined"][1]


def test_eigenvalue_history_based_matches_event_based(medium):
    m, xml, path = medium
    a = run_gpu(path, n_trace=500, cap=512, trace_batch=4)
    b = run_gpu(path, n_trace=500, cap=512, trace_batch=4, event_based=False)
    np.testing.assert_allclose(a["k_generation"], b["k_generation"], rtol=1e-10, atol=0)
    for f in DISCRETE:
        assert np.array_equal(a["trace"][0][f], b["trace"][0][f]), f


def test_eigenvalue_infinite_medium_known_answer(built, tmp_path):
    """FP32 tables: the combined k-effective of 30 active generations of
    2 x 10^4 neutrons lies within 3 of its standard deviations of
    nu Sigma_f / Sigma_a."""
    from openmc_gb300 import configs
    m, path = configs.infinite_medium(tmp_path, particles=20_000, batches=40, inactive=10, n_points=400)
    m.export_to_model_xml(path)
    g = run_gpu(path, fp32=True)
    k, sd = g["keff"]
    assert len(g["k_generation"]) == 40
    assert 0 < sd < 0.01
    assert abs(k - m.k_inf) < 3.0 * sd + 1e-4, (k, sd, m.k_inf)
