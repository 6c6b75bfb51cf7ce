"""HDF5 input and output on the GPU path.

Nuclide libraries in OpenMC's incident-neutron HDF5 layout give the same
tables as the native container: the traced histories of runs on both are
bit-identical (every event's kind, cell, nuclide, energy, distance and
weight), and tallies, global tallies and every generation's k agree to the
last few bits (the device sums them with atomics, whose order varies from
run to run).  The statepoint written at the last
batch (src/simulation.cpp:432-441, src/state_point.cpp:36-357) holds the
tallies' SUM and SUM_SQ, the global tallies, the generation k values and the
combined k-effective exactly as the library's own entry points report them.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def run(path, eigen=False, n_trace=0):
    from openmc_gb300 import lib
    lib.init(directory=path)
    try:
        if n_trace:
            lib.set_trace(n_trace, 256)
        lib.simulation_init()
        status = 0
        while status == 0:
            status = lib.next_batch()
        out = {"batches": lib.current_batch()}
        if n_trace:
            out["trace"] = lib.get_trace()
        if eigen:
            out["k_generation"], out["sites"] = lib.k_generation()
            out["keff"] = lib.keff()
        lib.simulation_finalize()
        out["tallies"] = {t: (lib.tally_results(t).copy(), lib.tally_n_realizations(t)) for t in lib.tally_ids()}
        out["globals"] = lib.global_tallies().copy()
        return out
    finally:
        lib.finalize()


def assert_same_traces(ta, tb):
    (ra, ca), (rb, cb) = ta, tb
    assert np.array_equal(ca, cb) and ca.sum() > 0
    for f in ra.dtype.names:
        assert np.array_equal(ra[f], rb[f]), f


def check_statepoint(path, out, eigen=False):
    from openmc_gb300.statepoint import StatePoint
    w = len(str(out["batches"]))
    sp = StatePoint(path / f"statepoint.{out['batches']:0{w}d}.h5")
    assert sp.current_batch == out["batches"]
    assert set(sp.tallies) == set(out["tallies"])
    for tid, (res, n) in out["tallies"].items():
        t = sp.tallies[tid]
        assert t.num_realizations == n == sp.n_realizations
        assert np.array_equal(t.sum.ravel(), res[..., 1].ravel())
        assert np.array_equal(t.sum_sq.ravel(), res[..., 2].ravel())
    g = out["globals"]
    assert np.array_equal(sp.global_tallies["sum"], g[:, 1])
    assert np.array_equal(sp.global_tallies["sum_sq"], g[:, 2])
    if eigen:
        assert sp.run_mode == "eigenvalue"
        assert np.array_equal(sp.k_generation, out["k_generation"])
        assert sp.k_combined == tuple(out["keff"])
    return sp


def test_h5_library_bit_identical_fixed_source(built, tmp_path):
    from openmc_gb300 import configs
    outs = []
    for fmt in ("native", "h5"):
        d = tmp_path / fmt
        d.mkdir()
        m, d = configs.lattice17(d, particles=20000, batches=3, n_points=2000, mesh_dim=(17, 17, 5), n_ebins=8,
                                 library_format=fmt)
        m.export_to_model_xml(d / "model.xml")
        outs.append(run(d, n_trace=2000))
        check_statepoint(d, outs[-1])
    a, b = outs  # (the two models number their tallies independently)
    assert_same_traces(a["trace"], b["trace"])
    assert len(a["tallies"]) == len(b["tallies"])
    for (ra, na), (rb, nb) in zip(a["tallies"].values(), b["tallies"].values()):
        assert na == nb
        assert np.abs(ra[..., 1]).max() > 0
        np.testing.assert_allclose(ra, rb, rtol=1e-12, atol=1e-14 * np.abs(ra).max())
    np.testing.assert_allclose(a["globals"], b["globals"], rtol=1e-12, atol=0)


def test_h5_library_bit_identical_eigenvalue(built, tmp_path):
    from openmc_gb300 import configs
    outs = []
    for fmt in ("native", "h5"):
        d = tmp_path / fmt
        d.mkdir()
        m, d = configs.infinite_medium(d, particles=4000, batches=6, inactive=2, n_points=400, library_format=fmt)
        m.export_to_model_xml(d / "model.xml")
        outs.append(run(d, eigen=True, n_trace=1000))
        sp = check_statepoint(d, outs[-1], eigen=True)
        assert sp.n_inactive == 2 and len(sp.k_generation) == 6
    a, b = outs
    assert_same_traces(a["trace"], b["trace"])
    np.testing.assert_allclose(a["k_generation"], b["k_generation"], rtol=1e-12, atol=0)
    np.testing.assert_allclose(a["keff"], b["keff"], rtol=1e-10, atol=1e-14)
    np.testing.assert_allclose(a["globals"], b["globals"], rtol=1e-12, atol=0)


def test_model_run_returns_statepoint(built, tmp_path):
    from openmc_gb300 import configs
    from openmc_gb300.statepoint import StatePoint
    m, d = configs.lattice17(tmp_path, particles=5000, batches=12, n_points=1000, mesh_dim=(17, 17, 2), n_ebins=2)
    path = m.run(cwd=d)
    assert path.name == "statepoint.12.h5"
    sp = StatePoint(path)
    t = next(iter(sp.tallies.values()))
    assert t.num_realizations == 12 and np.all(t.mean >= 0) and t.mean.max() > 0
    rel = t.std_dev[t.mean > 0] / t.mean[t.mean > 0]
    assert np.median(rel) < 0.2
