"""Edge cases on the GPU: a single history, a single particle slot, a model
without tallies, empty lookups, out-of-range material indices, a one-row
network, lost particles (a
geometry with a hole) and a full split ring, the last two ending as error
codes of openmc_next_batch."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_single_history_and_single_slot(built, tmp_path):
    from openmc_gb300 import configs, lib
    import oracle
    m, path = configs.point_cube(tmp_path, particles=1, batches=3, n_points=400, mesh_dim=(3, 3, 3), n_ebins=4)
    xml = m.export_to_model_xml(path)
    lib.init(directory=path)
    try:
        lib.settings.particles_in_flight = 1
        lib.set_trace(1, 4096)
        lib.simulation_init()
        for _ in range(3):
            lib.next_batch()
            assert lib.last_batch()["done"] == 1
        mean, _ = lib.tally_mean_std(lib.tally_ids()[0])
        lib.simulation_finalize()
    finally:
        lib.settings.particles_in_flight = 0
        lib.finalize()
    o = oracle.Oracle(xml)
    o.run(threads=1)
    assert np.allclose(mean.ravel(), o.tally(0)[:, 1] / 3, rtol=1e-5, atol=1e-12)


def test_model_without_tallies(built, tmp_path):
    from openmc_gb300 import configs, lib
    from openmc_gb300 import model as om
    m, path = configs.point_cube(tmp_path, particles=2000, batches=2, n_points=400)
    m.tallies = om.Tallies([])
    m.export_to_model_xml(path)
    lib.init(directory=path)
    try:
        lib.run()
        assert lib.tally_ids() == []
        assert lib.last_batch()["done"] == 2000
    finally:
        lib.finalize()


def test_empty_and_single_lookups(built):
    from openmc_gb300 import data, lib
    d = data.make_xsbench(n_nuc=6, n_points=300, seed=2, mat_counts=(4, 2))
    t = lib.XSTables(d, n_log_bins=200, max_lookups=16)
    out, h = t.lookup(np.zeros(0, np.int32), np.zeros(0))
    assert out.shape == (0, 5) and h.shape == (0,)
    out, h = t.lookup(np.array([1], np.int32), np.array([data.E_MAX]))
    assert np.isfinite(out).all()
    t.close()


def test_lookup_material_index_out_of_range(built):
    """A material index outside [0, n_mat): the host-buffer lookup returns
    OPENMC_E_OUT_OF_BOUNDS before any work; the device-buffer lookup reads no
    table for it, writes NaN and hash 0, and leaves every other lookup as the
    all-valid call computes it (sorted and unsorted)."""
    import torch
    from openmc_gb300 import data, lib
    d = data.make_xsbench(n_nuc=6, n_points=300, seed=2, mat_counts=(4, 2, 3))
    mats, e = data.xsbench_lookups(d, 5000, seed=3)
    t = lib.XSTables(d, n_log_bins=200, max_lookups=len(e))
    try:
        good, good_h = t.lookup(mats, e)
        bad = mats.copy()
        bad[[7, 100, 4999]] = [-1, 3, 1 << 20]
        with pytest.raises(lib.OutOfBoundsError):
            t.lookup(bad, e)
        dev = torch.device("cuda", 0)
        dm, de = torch.from_numpy(bad).to(dev), torch.from_numpy(e).to(dev)
        for sort in (True, False):
            out = torch.zeros((len(e), 5), dtype=torch.float64, device=dev)
            h = torch.full((len(e),), -7, dtype=torch.int32, device=dev)
            torch.cuda.synchronize()  # the lookup runs on the library's own stream
            t.lookup_device(len(e), dm.data_ptr(), de.data_ptr(), out.data_ptr(), h.data_ptr(), sort=sort)
            torch.cuda.synchronize()
            o, hh = out.cpu().numpy(), h.cpu().numpy()
            ok = np.ones(len(e), bool)
            ok[[7, 100, 4999]] = False
            assert np.isnan(o[~ok]).all() and (hh[~ok] == 0).all()
            assert np.array_equal(o[ok], good[ok]) and np.array_equal(hh[ok], good_h[ok])
    finally:
        t.close()


def test_one_row_network(built):
    from openmc_gb300 import lib
    from oracle import mlp as om
    net = lib.ImportanceNetwork(max_rows=1, seed=9)
    x = np.array([[0.1, -0.2, 0.3, 0.9]], np.float32)
    net.set_data(x, np.array([0.5], np.float32))
    loss, g = net.gradients()
    loss_ref, g_ref = om.loss_and_grad(net.params.astype(np.float64), x.astype(np.float64), np.array([0.5]))
    assert abs(loss - loss_ref) <= 1e-3 * abs(loss_ref) + 1e-7
    assert np.linalg.norm(g - g_ref) <= 2e-2 * np.linalg.norm(g_ref)
    assert np.isfinite(net.predict(x)).all()
    net.close()


def test_tallies_out_written(built, tmp_path):
    """simulation_finalize writes tallies.out next to the input in the
    reference's layout (src/output.cpp:605-720)."""
    from openmc_gb300 import configs, lib
    m, path = configs.point_cube(tmp_path, particles=2000, batches=3, n_points=400, mesh_dim=(2, 2, 2), n_ebins=3)
    m.export_to_model_xml(path)
    lib.init(directory=path)
    try:
        lib.run()
        mean, std = lib.tally_mean_std(lib.tally_ids()[0])
    finally:
        lib.finalize()
    text = (path / "tallies.out").read_text().splitlines()
    title = f"TALLY {m.tallies[0].id}: MESH FLUX"
    assert text[0].strip().startswith("=") and f">     {title}     <" in text[0]
    assert text[2] == " Mesh Index (1, 1, 1)"
    assert text[3].startswith("   Incoming Energy [")
    assert text[4] == "     Total Material"
    fields = text[5].split()
    assert fields[0] == "Flux" and fields[2] == "+/-"
    assert abs(float(fields[1]) - mean.ravel()[0]) <= 1e-5 * abs(mean.ravel()[0]) + 1e-300
    assert abs(float(fields[3]) - std.ravel()[0]) <= 1e-5 * abs(std.ravel()[0]) + 1e-300


def _holed_cube(tmp_path, **settings):
    """The point cube without its annulus cell (1 < r < 3 cm): particles that
    leave the inner cylinder find no cell there and are lost."""
    from openmc_gb300 import configs
    m, path = configs.point_cube(tmp_path, particles=400, batches=1, n_points=400, mesh_dim=(3, 3, 3), n_ebins=4)
    del m.geometry.root_universe.cells[1]
    for k, v in settings.items():
        setattr(m.settings, k, v)
    return m.export_to_model_xml(path), path


def test_lost_particles_counted_like_the_oracle(built, tmp_path):
    """A particle that finds no cell is killed and counted
    (src/particle.cpp mark_as_lost); with the limits raised the batch ends
    normally and the count is the oracle's."""
    from openmc_gb300 import lib
    import oracle
    xml, path = _holed_cube(tmp_path, max_lost_particles=10 ** 9, rel_max_lost_particles=1.0)
    lib.init(directory=path)
    saved = lib.settings.xs_fp32
    try:
        lib.settings.xs_fp32 = 0
        lib.simulation_init()
        lib.next_batch()
        b = lib.last_batch()
        lib.simulation_finalize()
    finally:
        lib.settings.xs_fp32 = saved
        lib.finalize()
    o = oracle.Oracle(xml)
    o.run(threads=1)
    assert b["lost"] > 0 and b["done"] == 400
    assert b["lost"] == o.globals()[2]


def test_lost_particles_beyond_the_limit_are_a_geometry_error(built, tmp_path):
    """More lost particles than max_lost_particles (default 10) and
    rel_max_lost_particles x histories: OPENMC_E_GEOMETRY."""
    from openmc_gb300 import lib
    _, path = _holed_cube(tmp_path)
    lib.init(directory=path)
    try:
        lib.simulation_init()
        with pytest.raises(lib.GeometryError):
            lib.next_batch()
    finally:
        lib.finalize()


def test_full_split_ring_is_an_allocation_error(built, tmp_path):
    """Windows falling 10x per 1 cm mesh bin split every particle that moves
    deeper (windows are scaled by the particle's birth window,
    src/weight_windows.cpp:56-146, so only their variation matters); a
    16-entry split ring fills and the batch ends with OPENMC_E_ALLOCATE
    (nothing is written past the ring, and the split copies waiting in it
    are not started)."""
    from openmc_gb300 import configs, lib
    m, path = configs.shield(tmp_path, particles=2000, batches=1, n_points=400, tally_mesh_windows=True)
    m.export_to_model_xml(path)
    lib.init(directory=path)
    saved = (lib.settings.split_to_slots, lib.settings.secondary_capacity)
    try:
        lib.settings.split_to_slots = 1
        lib.settings.secondary_capacity = 16
        lo, _ = lib.WeightWindows(0).bounds
        ix = np.arange(lo.size) % 200  # x index of the 200 x 10 x 10 mesh bin (x fastest)
        lower = 0.1 ** ix
        lib.WeightWindows(0).bounds = (lower, 5.0 * lower)
        lib.simulation_init()
        with pytest.raises(lib.AllocationError):
            lib.next_batch()
    finally:
        lib.settings.split_to_slots, lib.settings.secondary_capacity = saved
        lib.finalize()
