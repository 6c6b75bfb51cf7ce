"""Host-side model building and oracle self-consistency (CPU only)."""
from pathlib import Path

import numpy as np
import pytest

import oracle
from oracle import flatten
from openmc_gb300 import configs, data


def test_nuclide_roundtrip(tmp_path):
    nuc = data.make_nuclide("X1", 56, 300, seed=5)
    data.write_nuclide(nuc, tmp_path / "x.nuc")
    back = data.read_nuclide(tmp_path / "x.nuc")
    assert back.name == "X1" and back.awr == nuc.awr and back.kT == nuc.kT
    assert np.array_equal(back.energy, nuc.energy)
    assert np.array_equal(back.elastic, nuc.elastic)
    assert np.all(np.diff(nuc.energy) > 0)
    assert nuc.energy[0] == data.E_MIN and nuc.energy[-1] == data.E_MAX


def test_region_tokens_complex():
    idx = {1: 0, 2: 1, 3: 2}
    toks, simple = flatten._region_tokens("-1 2", idx)
    assert simple and toks == [-1, 2]
    toks, simple = flatten._region_tokens("-1 | (2 -3)", idx)
    assert not simple
    # postfix: -1 2 -3 & |
    assert toks == [-1, 2, -3, flatten.OP_INTERSECTION, flatten.OP_UNION]
    toks, simple = flatten._region_tokens("~(1 | 2)", idx)
    assert not simple and toks[-1] == flatten.OP_COMPLEMENT


@pytest.fixture(scope="module")
def cube(tmp_path_factory):
    d = tmp_path_factory.mktemp("cube")
    m, path = configs.point_cube(d, particles=400, batches=2, n_points=400,
                                 mesh_dim=(5, 5, 5), n_ebins=6)
    return m.export_to_model_xml(path)


def test_flatten_cube(cube):
    a = flatten.load_model(cube)
    assert a["settings_i"][0] == 400 and a["settings_i"][1] == 2
    assert len(a["surf_type"]) == 8 and len(a["cell_id"]) == 3
    assert a["root_univ"][0] == 0
    assert a["filt_nbins"].tolist() == [125, 6]


def test_history_and_event_loops_agree(cube):
    """The reference's event-based and history-based loops give identical
    per-particle physics (tests/regression_tests run both modes against one
    results_true.dat); single-threaded, tallies are bit-identical."""
    h = oracle.Oracle(cube)
    h.run(threads=1, mode=0)
    e = oracle.Oracle(cube)
    e.run(threads=1, mode=1)
    for t in range(h.n_tallies):
        a, b = h.tally(t), e.tally(t)
        assert np.allclose(a, b, rtol=1e-13, atol=0)
    assert np.allclose(h.globals()[:2], e.globals()[:2], rtol=1e-13)


def test_oracle_threads_agree(cube):
    a = oracle.Oracle(cube)
    a.run(threads=1)
    b = oracle.Oracle(cube)
    b.run(threads=4)
    assert np.allclose(a.tally(0), b.tally(0), rtol=1e-10, atol=1e-14)


def test_trace_consistency(cube):
    o = oracle.Oracle(cube)
    o.set_trace(100, 128)
    o.transport(1, 1, 100)
    rec, cnt = o.traces()
    assert (cnt > 0).all()
    first = rec[:, 0]
    assert (first["E"] == 1.0e6).all()          # 1 MeV discrete source
    assert (first["material"] == 0).all()
    kinds = np.concatenate([rec["kind"][h, :min(c, 128)] for h, c in enumerate(cnt)])
    assert set(np.unique(kinds)) <= {1, 2}


def test_xsbench_oracle_matches_numpy():
    d = data.make_xsbench(n_nuc=6, n_points=500, seed=1, mat_counts=(7, 3))
    x = oracle.XSBenchOracle(d, n_log_bins=200)
    mats, e = data.xsbench_lookups(d, 300, seed=2)
    out, _ = x.lookup(mats, e)
    # independent numpy restatement with a plain searchsorted index
    for k in range(300):
        m, E = mats[k], e[k]
        tot = np.zeros(5)
        for j in range(d.mat_off[m], d.mat_off[m + 1]):
            n = d.mat_nuc[j]
            g = d.energy[n]
            i = int(np.searchsorted(g, E, side="left")) - 1
            i = min(max(i, 0), len(g) - 2)
            f = (E - g[i]) / (g[i + 1] - g[i])
            tot += d.mat_dens[j] * ((1 - f) * d.xs[n, i] + f * d.xs[n, i + 1])
        assert np.allclose(out[k], tot, rtol=1e-12)


def test_oracle_estimators_agree(tmp_path):
    """Track-length and collision estimates of the same cell, material and
    mesh fluxes agree within statistics (the reference's estimator-agreement
    check, tests/unit_tests/test_filter_mesh.py:10-61)."""
    import numpy as np
    import oracle
    from openmc_gb300 import configs
    m, path = configs.point_cube(tmp_path, particles=4000, batches=8, n_points=600,
                                 mesh_dim=(4, 4, 4), n_ebins=5, estimator_tallies=True)
    xml = m.export_to_model_xml(path)
    o = oracle.Oracle(xml)
    o.run(threads=4)
    n = 8

    def mean_std(k):
        r = o.tally(k)
        mu = r[:, 1] / n
        sd = np.sqrt(np.maximum(r[:, 2] / n - mu * mu, 0) / (n - 1))
        return mu, sd

    for k_tl, k_col in ((1, 4), (2, 5), (3, 6)):
        a, sa = mean_std(k_tl)
        b, sb = mean_std(k_col)
        ok = (sa > 0) & (sb > 0)
        assert ok.sum() > 0
        z = np.abs(a - b)[ok] / np.hypot(sa, sb)[ok]
        assert (z > 4).sum() == 0, (k_tl, z.max())
    # one material: its flux is the sum over the cells
    a, _ = mean_std(2)
    c, _ = mean_std(1)
    tot_cells = c.reshape(3, 4, 3)[:, :, 0].sum()
    # (up to tracks below the lowest energy group bound)
    assert abs(a.reshape(-1, 2)[0, 0] - tot_cells) <= 1e-5 * tot_cells


def test_time_cutoff_stops_histories(tmp_path):
    """A neutron time cutoff (src/particle.cpp:246-286, src/settings.cpp:
    723-724): flights end where the particle's time reaches the cutoff and
    the particle dies there, so a short cutoff removes flux from the slow
    neutrons of the cube, in both loops alike."""
    from openmc_gb300 import configs
    out = {}
    for cut in (None, 2e-7):
        d = tmp_path / str(cut)
        d.mkdir()
        m, path = configs.point_cube(d, particles=400, batches=2, n_points=300)
        m.settings.time_cutoff = cut
        xml = m.export_to_model_xml(path)
        assert (cut is None) == ("time_neutron" not in Path(xml).read_text())
        h = oracle.Oracle(xml)
        h.run(threads=1, mode=0)
        e = oracle.Oracle(xml)
        e.run(threads=1, mode=1)
        assert np.allclose(h.tally(0), e.tally(0), rtol=1e-13, atol=0)
        out[cut] = h.tally(0)[:, 1].sum()
    assert 0 < out[2e-7] < 0.9 * out[None]
