"""HDF5 input and output on the GPU path.

Nuclide libraries in OpenMC's incident-neutron HDF5 layout give the same
tables as the native container: runs on both are bit-identical (tallies,
global tallies, every generation's k).  The statepoint written at the last
batch (src/simulation.cpp:432-441, src/state_point.cpp:36-357) holds the
tallies' SUM and SUM_SQ, the global tallies, the generation k values and the
combined k-effective exactly as the library's own entry points report them.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def run(path, eigen=False):
    from openmc_gb300 import lib
    lib.init(directory=path)
    try:
        lib.simulation_init()
        status = 0
        while status == 0:
            status = lib.next_batch()
        out = {"batches": lib.current_batch()}
        if eigen:
            out["k_generation"], out["sites"] = lib.k_generation()
            out["keff"] = lib.keff()
        lib.simulation_finalize()
        out["tallies"] = {t: (lib.tally_results(t).copy(), lib.tally_n_realizations(t)) for t in lib.tally_ids()}
        out["globals"] = lib.global_tallies().copy()
        return out
    finally:
        lib.finalize()


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
        outs.append(run(d))
        check_statepoint(d, outs[-1])
    a, b = outs
    for tid in a["tallies"]:
        assert np.array_equal(a["tallies"][tid][0], b["tallies"][tid][0])
        assert np.abs(a["tallies"][tid][0][..., 1]).max() > 0
    assert np.array_equal(a["globals"], b["globals"])


def test_h5_library_bit_identical_eigenvalue(built, tmp_path):
    from openmc_gb300 import configs
    outs = []
    for fmt in ("native", "h5"):
        d = tmp_path / fmt
        d.mkdir()
        m, d = configs.infinite_medium(d, particles=4000, batches=6, inactive=2, n_points=400, library_format=fmt)
        m.export_to_model_xml(d / "model.xml")
        outs.append(run(d, eigen=True))
        sp = check_statepoint(d, outs[-1], eigen=True)
        assert sp.n_inactive == 2 and len(sp.k_generation) == 6
    a, b = outs
    assert np.array_equal(a["k_generation"], b["k_generation"])
    assert a["keff"] == b["keff"]
    assert np.array_equal(a["globals"], b["globals"])


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
