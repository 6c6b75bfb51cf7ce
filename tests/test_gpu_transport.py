"""GPU parity: the event-based CUDA path against the oracle (CPU restatement
of the reference) on the same seeded inputs.

FP64 mode: per history, the event sequence (event kind, cell, material,
surface crossed or nuclide sampled, hash of the nuclide grid indices, coordinate
depth) is identical to the oracle's and event counts are identical.  The only
arithmetic difference between the two builds is the device's log/sin/cos
against glibc's (each within 1-2 ulp); free-gas collisions amplify that
difference along a history, so energies and weights are compared to 1e-6
relative and flight distances to 1e-6 relative + 1e-7 cm (short chords at
grazing incidence magnify the relative difference).  Tally bins agree to 1e-5
relative of each bin plus 1e-9 of the largest bin.
FP32-table mode: every tally mean within 3 combined standard deviations of the
FP64 path except for the expected 3-sigma tail, none beyond 5 sigma.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DISCRETE = ("kind", "cell", "material", "surface_or_nuclide", "grid_hash", "n_coord")
CONT = ("E", "dist", "wgt")


def run_gpu(path, n_trace=0, cap=256, fp32=False, in_flight=0, sort=True, batches=None, ww_on=None,
            max_levels=0, fuse=3, event_based=True, stage_tables=0, contract=1, defer_tally=1):
    from openmc_gb300 import lib
    lib.init(directory=path)
    lib.settings.stage_tables = stage_tables
    lib.settings.contract = contract
    lib.settings.defer_tally = defer_tally
    try:
        lib.settings.event_based = event_based
        lib.settings.xs_fp32 = 1 if fp32 else 0
        lib.settings.particles_in_flight = in_flight
        lib.settings.sort_queue = 1 if sort else 0
        lib.settings.max_levels = max_levels
        lib.settings.fuse_xs = fuse
        lib.settings.split_to_slots = 0  # the reference's per-history secondary order
        if n_trace:
            lib.set_trace(n_trace, cap)
        lib.simulation_init()
        if ww_on is not None:
            lib.set_weight_windows_on(ww_on)
        status = 0
        nb = 0
        while status == 0:
            status = lib.next_batch()
            nb += 1
            if batches and nb >= batches:
                break
        out = {"batch": lib.last_batch(), "timing": lib.timing()}
        if n_trace:
            out["trace"] = lib.get_trace()
        lib.simulation_finalize()
        out["tallies"] = [(lib.tally_results(t).copy(), lib.tally_n_realizations(t))
                          for t in lib.tally_ids()]
        out["globals"] = lib.global_tallies().copy()
        return out
    finally:
        lib.settings.stage_tables = 0
        lib.settings.contract = 1
        lib.settings.defer_tally = 1
        lib.finalize()


def run_oracle(xml, n_trace=0, cap=256, batches=None, threads=1):
    import oracle
    o = oracle.Oracle(xml)
    if n_trace:
        o.set_trace(n_trace, cap)
    o.run(threads=threads, batches=batches)
    res = {"tallies": [o.tally(t) for t in range(o.n_tallies)], "globals": o.globals()}
    if n_trace:
        res["trace"] = o.traces()
    return res


def trace_mismatches(gpu_trace, orc_trace, cap, rtol=1e-6, dist_atol=1e-7):
    rec, cnt = gpu_trace
    orec, ocnt = orc_trace
    bad = []
    for h in range(len(cnt)):
        if cnt[h] != ocnt[h]:
            bad.append((h + 1, "count", int(cnt[h]), int(ocnt[h])))
            continue
        n = min(cnt[h], cap)
        for f in DISCRETE:
            if not np.array_equal(rec[f][h, :n], orec[f][h, :n]):
                k = int(np.nonzero(rec[f][h, :n] != orec[f][h, :n])[0][0])
                bad.append((h + 1, f, k, int(rec[f][h, k]), int(orec[f][h, k])))
                break
        else:
            for f in CONT:
                a, b = rec[f][h, :n], orec[f][h, :n]
                atol = dist_atol if f == "dist" else 0.0
                if not np.allclose(a, b, rtol=rtol, atol=atol):
                    k = int(np.nonzero(~np.isclose(a, b, rtol=rtol, atol=atol))[0][0])
                    bad.append((h + 1, f, k, float(a[k]), float(b[k])))
                    break
    return bad


def assert_tallies_close(gpu_tallies, orc_tallies, rtol=1e-5):
    assert len(gpu_tallies) >= len(orc_tallies)
    for (g, n), o in zip(gpu_tallies, orc_tallies):
        gs = g[..., 1].ravel()
        os_ = o[:, 1]
        scale = np.abs(os_).max()
        if scale == 0:
            assert np.all(gs == 0)
            continue
        assert np.allclose(gs, os_, rtol=rtol, atol=1e-9 * scale), \
            f"max rel diff {np.max(np.abs(gs - os_) / np.maximum(np.abs(os_), 1e-300))}"


@pytest.fixture(scope="module")
def cube(built, tmp_path_factory):
    from openmc_gb300 import configs
    d = tmp_path_factory.mktemp("cube")
    m, path = configs.point_cube(d, particles=3000, batches=2, n_points=2000)
    return m.export_to_model_xml(path), path


@pytest.fixture(scope="module")
def lattice(built, tmp_path_factory):
    from openmc_gb300 import configs
    d = tmp_path_factory.mktemp("lattice")
    m, path = configs.lattice17(d, particles=1500, batches=2, n_points=2000, mesh_dim=(17, 17, 10), n_ebins=20)
    return m.export_to_model_xml(path), path


def test_point_cube_history_parity(cube):
    xml, path = cube
    g = run_gpu(path, n_trace=3000, cap=512)
    o = run_oracle(xml, n_trace=3000, cap=512)
    bad = trace_mismatches(g["trace"], o["trace"], 512)
    assert not bad, f"{len(bad)} histories differ, first: {bad[:5]}"
    assert_tallies_close(g["tallies"], o["tallies"])
    assert g["batch"]["done"] == 3000 and g["batch"]["total_weight"] == 3000.0


def test_point_cube_no_sort_and_small_bank(cube):
    """Queue order and in-flight capacity do not change any history."""
    xml, path = cube
    g = run_gpu(path, n_trace=500, cap=512, sort=False, in_flight=257)
    o = run_oracle(xml, n_trace=500, cap=512)
    assert not trace_mismatches(g["trace"], o["trace"], 512)
    assert_tallies_close(g["tallies"], o["tallies"])


def test_time_cutoff_parity(built, tmp_path):
    """A neutron time cutoff (src/particle.cpp:246-286): a flight ends where
    the particle's time reaches the cutoff and the particle dies there.
    Histories and tallies equal the oracle's, and the cutoff removes the
    slow neutrons' flux and events."""
    from openmc_gb300 import configs
    runs = {}
    for cut in (None, 2e-7):
        d = tmp_path / str(cut)
        d.mkdir()
        m, path = configs.point_cube(d, particles=3000, batches=2, n_points=2000)
        m.settings.time_cutoff = cut
        xml = m.export_to_model_xml(path)
        runs[cut] = run_gpu(path, n_trace=3000, cap=512)
        if cut is not None:
            o = run_oracle(xml, n_trace=3000, cap=512)
            bad = trace_mismatches(runs[cut]["trace"], o["trace"], 512)
            assert not bad, f"{len(bad)} histories differ, first: {bad[:5]}"
            assert_tallies_close(runs[cut]["tallies"], o["tallies"])
    cut, free = runs[2e-7], runs[None]
    assert cut["batch"]["done"] == 3000
    assert 0 < cut["tallies"][0][0][..., 1].sum() < 0.9 * free["tallies"][0][0][..., 1].sum()
    assert cut["batch"]["events"] < free["batch"]["events"]


def test_lattice_history_parity(lattice):
    xml, path = lattice
    g = run_gpu(path, n_trace=1500, cap=1024)
    o = run_oracle(xml, n_trace=1500, cap=1024)
    bad = trace_mismatches(g["trace"], o["trace"], 1024)
    assert not bad, f"{len(bad)} histories differ, first: {bad[:5]}"
    assert_tallies_close(g["tallies"], o["tallies"])
    lk = g["batch"]["leakage"] / g["batch"]["total_weight"]
    assert 0.0 <= lk <= 1.0


def test_lattice_first_10k_histories(built, tmp_path):
    """FP64 tables: the first 10^4 histories of a lattice batch have the
    oracle's event kinds, cells, materials, surfaces / nuclides, grid-index
    hashes, coordinate depths and event counts."""
    from openmc_gb300 import configs
    m, path = configs.lattice17(tmp_path, particles=10_000, batches=1, n_points=2000,
                                mesh_dim=(17, 17, 5), n_ebins=10)
    xml = m.export_to_model_xml(path)
    g = run_gpu(path, n_trace=10_000, cap=256)
    o = run_oracle(xml, n_trace=10_000, cap=256)
    bad = trace_mismatches(g["trace"], o["trace"], 256)
    assert not bad, f"{len(bad)} of 10000 histories differ, first: {bad[:5]}"
    assert_tallies_close(g["tallies"], o["tallies"])


def assert_globals_match(gpu_globals, orc_globals, rtol=1e-12):
    """Global leakage tally (src/particle.cpp:475-512; per batch leakage /
    source weight, accumulated as SUM and SUM_SQ like tally.cpp:1059-1100)
    against the oracle's."""
    g = np.asarray(gpu_globals).reshape(4, 3)[3]
    assert np.isclose(g[1], orc_globals[0], rtol=rtol, atol=0), (g[1], orc_globals[0])
    assert np.isclose(g[2], orc_globals[1], rtol=rtol, atol=0), (g[2], orc_globals[1])


def test_lattice_full_size_first_10k_histories(built, tmp_path):
    """The headline 17x17 lattice at its full size (12 nuclides of 11,303
    grid points, flux on the 17x17x50 mesh x 100 log-energy bins), FP64
    tables: the first 10^4 histories of the batch have the oracle's event
    kinds, cells, materials, surfaces / nuclides, grid-index hashes,
    coordinate depths and event counts; every one of the 1.445 M tally bins
    agrees with the oracle's to 1e-5 relative, and so does the global
    leakage tally."""
    from openmc_gb300 import configs
    import os
    m, path = configs.lattice17(tmp_path, particles=10_000, batches=1)
    xml = m.export_to_model_xml(path)
    g = run_gpu(path, n_trace=10_000, cap=256)
    o = run_oracle(xml, n_trace=10_000, cap=256, threads=min(os.cpu_count() or 1, 16))
    bad = trace_mismatches(g["trace"], o["trace"], 256)
    assert not bad, f"{len(bad)} of 10000 histories differ, first: {bad[:5]}"
    (r, n), = g["tallies"]
    assert r.shape[0] == 17 * 17 * 50 * 100 and n == 1
    assert (r[..., 1] > 0).sum() > 10_000
    assert_tallies_close(g["tallies"], o["tallies"])
    assert_globals_match(g["globals"], o["globals"])
    assert g["batch"]["done"] == 10_000 and g["batch"]["lost"] == 0


def test_global_leakage_tally_matches_oracle(cube, shield_ww):
    """Global leakage of the point cube (vacuum boundary) and of the shield
    with weight windows (split and rouletted weights leak) against the
    oracle over two batches."""
    for xml, path in (cube, shield_ww):
        g = run_gpu(path)
        o = run_oracle(xml)
        assert_globals_match(g["globals"], o["globals"])
        assert np.asarray(g["globals"]).reshape(4, 3)[3, 1] > 0


def test_cell_material_filters_and_collision_estimator(built, tmp_path):
    """Cell and material filters with track-length and collision estimators
    (tally_scoring.cpp:2416-2600, filter_cell.cpp, filter_material.cpp)
    match the oracle bin by bin."""
    from openmc_gb300 import configs
    m, path = configs.point_cube(tmp_path, particles=3000, batches=2, n_points=600,
                                 mesh_dim=(4, 4, 4), n_ebins=5, estimator_tallies=True)
    xml = m.export_to_model_xml(path)
    g = run_gpu(path)
    o = run_oracle(xml)
    assert len(g["tallies"]) == 7
    assert_tallies_close(g["tallies"], o["tallies"])
    for k in range(1, 7):
        r, n = g["tallies"][k]
        assert n == 2 and r[..., 1].sum() > 0


def test_lattice_history_based_parity(lattice):
    """settings.event_based = False runs the history-based kernel (one thread
    per history, src/simulation.cpp:804-831); histories and tallies match the
    oracle as the event-based loop does."""
    xml, path = lattice
    g = run_gpu(path, n_trace=800, cap=1024, event_based=False)
    o = run_oracle(xml, n_trace=800, cap=1024)
    bad = trace_mismatches(g["trace"], o["trace"], 1024)
    assert not bad, f"{len(bad)} histories differ, first: {bad[:5]}"
    assert_tallies_close(g["tallies"], o["tallies"])
    assert g["batch"]["done"] > 0


def test_lattice_builds_agree(lattice):
    """The 2-level build (per-level state in registers) and the 4-level
    build, the unfused event kernels, the kernels reading their geometry and
    material tables from shared-memory copies (event- and history-based),
    and track-length tallies scored inside the advance kernel instead of
    from deferred track records give the same histories and tallies."""
    xml, path = lattice
    a = run_gpu(path, n_trace=600, cap=1024)
    b = run_gpu(path, n_trace=600, cap=1024, max_levels=4)
    c = run_gpu(path, n_trace=600, cap=1024, fuse=0)
    d = run_gpu(path, n_trace=600, cap=1024, stage_tables=1)
    e = run_gpu(path, n_trace=600, cap=1024, stage_tables=1, event_based=False)
    f = run_gpu(path, n_trace=600, cap=1024, defer_tally=0)
    for other in (b, c, d, e, f):
        assert not trace_mismatches(a["trace"], other["trace"], 1024)
        for (ra, na), (rb, nb) in zip(a["tallies"], other["tallies"]):
            assert na == nb
            np.testing.assert_allclose(ra[..., 1], rb[..., 1], rtol=1e-9, atol=1e-300)


@pytest.fixture(scope="module")
def shield_ww(built, tmp_path_factory):
    from openmc_gb300 import configs
    from openmc_gb300 import model as om
    d = tmp_path_factory.mktemp("shieldww")
    mesh = om.RegularMesh()
    mesh.dimension = [40, 1, 1]
    mesh.lower_left = [0.0, -25.0, -25.0]
    mesh.upper_right = [200.0, 25.0, 25.0]
    # importance rising threefold every 10 cm: particles split on entering
    # deeper window bins and are rouletted when they scatter back
    lower = 0.5 * 3.0 ** (-0.5 * np.arange(40))
    ww = om.WeightWindows(mesh, lower, upper_bound_ratio=5.0, energy_bounds=[0.0, 2.0e7 * 1.000001])
    m, path = configs.shield(d, particles=300, batches=2, n_points=2000, mesh_dim=(40, 2, 2),
                             weight_windows=ww)
    return m.export_to_model_xml(path), path


def test_shield_weight_window_parity(shield_ww):
    """Splitting, roulette and LIFO secondary revival match the oracle."""
    xml, path = shield_ww
    g = run_gpu(path, n_trace=300, cap=2048)
    o = run_oracle(xml, n_trace=300, cap=2048)
    assert g["batch"]["secondaries"] > 0
    bad = trace_mismatches(g["trace"], o["trace"], 2048)
    assert not bad, f"{len(bad)} histories differ, first: {bad[:5]}"
    assert_tallies_close(g["tallies"], o["tallies"])


@pytest.mark.parametrize("contract", [1, 0])
def test_fp32_tables_within_3_sigma(built, tmp_path, contract):
    """FP32 tables against FP64 tables, for the FP32-mode build with fused
    FP64 multiply-adds (the default) and for the one that rounds them
    separately."""
    from openmc_gb300 import configs
    m, path = configs.lattice17(tmp_path, particles=40000, batches=6, n_points=4000,
                                mesh_dim=(17, 17, 4), n_ebins=10)
    m.export_to_model_xml(path)
    a = run_gpu(path, fp32=False)
    b = run_gpu(path, fp32=True, contract=contract)
    (ra, n), (rb, _) = a["tallies"][0], b["tallies"][0]
    ma, mb = ra[..., 1] / n, rb[..., 1] / n
    sa = np.sqrt(np.maximum(ra[..., 2] / n - ma ** 2, 0) / (n - 1))
    sb = np.sqrt(np.maximum(rb[..., 2] / n - mb ** 2, 0) / (n - 1))
    sig = np.sqrt(sa ** 2 + sb ** 2)
    ok = sig > 0
    z = np.abs(ma - mb)[ok] / sig[ok]
    assert (z > 5).sum() == 0
    assert (z > 3).mean() < 0.01
    tot_a, tot_b = ma.sum(), mb.sum()
    assert abs(tot_a - tot_b) <= 3 * np.sqrt((sa ** 2).sum() + (sb ** 2).sum()) + 1e-12 * tot_a


def test_transport_macro_xs_against_oracle(lattice):
    """The transport kernels' own macroscopic XS lookup (material_xs on the
    device, the tables the batch uses) at seeded (material, E) pairs against
    the oracle: FP64 tables give the oracle's nuclide grid-index hashes and
    macroscopic XS within 1e-12; FP32 tables keep the hashes, and their
    largest relative error is below 1e-5 (FP32 rows and interpolation
    factor, FP32 accumulation over the material's nuclides)."""
    import oracle
    from openmc_gb300 import data, lib
    xml, path = lattice
    rng = np.random.default_rng(12)
    n = 20000
    e = np.exp(rng.uniform(np.log(data.E_MIN), np.log(data.E_MAX), n))
    e[:2] = [data.E_MIN, data.E_MAX]
    mats = rng.integers(0, 3, n).astype(np.int32)
    ot, oa, oh = oracle.Oracle(xml).macro_xs(mats, e)
    ref = np.stack([ot, oa])
    saved = lib.settings.xs_fp32
    out = {}
    for fp32 in (0, 1):
        lib.init(directory=path)
        try:
            lib.settings.xs_fp32 = fp32
            lib.simulation_init()
            t, a, h = lib.material_xs(mats, e)
            lib.simulation_finalize()
        finally:
            lib.settings.xs_fp32 = saved
            lib.finalize()
        out[fp32] = (np.stack([t, a]), h.view(np.int32))
    for fp32, tol in ((0, 1e-12), (1, 1e-5)):
        got, h = out[fp32]
        assert np.array_equal(h, oh)
        rel = np.abs(got - ref) / np.maximum(np.abs(ref), 1e-300)
        assert rel.max() <= tol, f"fp32={fp32}: max relative error {rel.max():.3g}"


def test_xs_lookup_parity(built):
    """Lookup microbenchmark tables (68 x 11,303 x 5): bit-exact grid indices
    (hash over each material's nuclides) and <=1e-12 relative macro XS in
    FP64; FP32 tables keep the indices and report their relative error."""
    import oracle
    from openmc_gb300 import data, lib
    d = data.make_xsbench()
    mats, e = data.xsbench_lookups(d, 20000, seed=11)
    ref, ref_h = oracle.XSBenchOracle(d).lookup(mats, e)
    t64 = lib.XSTables(d, fp32=False, max_lookups=len(e))
    out, h = t64.lookup(mats, e, sort=True)
    assert np.array_equal(h, ref_h)
    rel = np.abs(out - ref) / np.maximum(np.abs(ref), 1e-300)
    assert rel.max() <= 1e-12
    out_u, h_u = t64.lookup(mats, e, sort=False)
    assert np.array_equal(h_u, ref_h) and np.array_equal(out_u, out)
    t32 = lib.XSTables(d, fp32=True, max_lookups=len(e))
    out32, h32 = t32.lookup(mats, e)
    assert np.array_equal(h32, ref_h)
    rel32 = np.abs(out32 - ref) / np.maximum(np.abs(ref), 1e-300)
    assert rel32.max() < 1e-4


def test_xs_lookup_edges(built):
    """Energies on grid points, at the grid ends and at hash-bin edges."""
    import oracle
    from openmc_gb300 import data, lib
    d = data.make_xsbench(n_nuc=8, n_points=600, seed=5, mat_counts=(12, 3, 5))
    pts = np.concatenate([d.energy[0][:50], d.energy[3][-20:], [data.E_MIN, data.E_MAX],
                          np.exp(np.linspace(np.log(data.E_MIN), np.log(data.E_MAX), 400))])
    mats = np.arange(len(pts)) % 3
    ref, ref_h = oracle.XSBenchOracle(d, n_log_bins=500).lookup(mats, pts)
    t = lib.XSTables(d, n_log_bins=500, max_lookups=len(pts))
    out, h = t.lookup(mats, pts)
    assert np.array_equal(h, ref_h)
    assert np.allclose(out, ref, rtol=1e-12, atol=0)


def test_full_size_lattice_conservation(built, tmp_path):
    """Full-size 17x17 lattice (11,303-point grids, 17x17x50 x 100 energy
    bins), one batch of 10^6 histories: every source particle finishes,
    weights are conserved without windows, tallies are non-negative and the
    total flux agrees with an independent oracle sample within statistics."""
    from openmc_gb300 import configs
    m, path = configs.lattice17(tmp_path, particles=1_000_000, batches=1)
    xml = m.export_to_model_xml(path)
    g = run_gpu(path)
    b = g["batch"]
    assert b["done"] == 1_000_000
    assert b["total_weight"] == 1_000_000.0
    assert b["lost"] == 0
    r, n = g["tallies"][0]
    assert n == 1 and (r[..., 1] >= 0).all()
    gpu_total = r[..., 1].sum()
    import oracle
    o = oracle.Oracle(xml)
    o.transport(1, 1, 4000, threads=4)
    o.accumulate()
    t = o.tally(0)[:, 1].sum() * 1_000_000 / 4000
    assert abs(gpu_total - t) / gpu_total < 0.1
