"""Elastic-scattering kinematics against the known answer, with FP64 and
with FP32 tables (GPU).

A neutron scattering isotropically in the centre-of-mass frame off a nucleus
at rest (src/physics.cpp:754-818 takes the target at rest above 400 kT for
awr > 1) leaves with E'/E = [(1 + alpha) + (1 - alpha) mu_cm] / 2,
alpha = ((awr - 1) / (awr + 1))^2: uniform on [alpha, 1], mean
(1 + alpha) / 2, variance (1 - alpha)^2 / 12.  In a reflective box of one
scatterer with energy-independent cross sections the traced histories give
that ratio for every collision the particle survives, from the pre-event
energies of the collision and of the next event.  With FP32 tables the
kinematics run in FP32 and the outgoing direction is renormalised in FP64,
so the same law must hold to FP32 rounding."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def scatter_box(directory, awr_a=56):
    from openmc_gb300 import data
    from openmc_gb300 import model as om
    nuc = data.make_flat_nuclide("Sx56", awr_a, 400, 11, elastic=5.0, capture=0.05)
    xs_xml = data.write_library([nuc], directory)
    mat = om.Material(name="scatterer")
    mat.add_nuclide("Sx56", 1.0)
    mat.set_density("atom/b-cm", 0.05)
    mats = om.Materials([mat], cross_sections=xs_xml.name)
    planes = [om.XPlane(-20.0, boundary_type="reflective"), om.XPlane(20.0, boundary_type="reflective"),
              om.YPlane(-20.0, boundary_type="reflective"), om.YPlane(20.0, boundary_type="reflective"),
              om.ZPlane(-20.0, boundary_type="reflective"), om.ZPlane(20.0, boundary_type="reflective")]
    box = +planes[0] & -planes[1] & +planes[2] & -planes[3] & +planes[4] & -planes[5]
    geom = om.Geometry(om.Universe(cells=[om.Cell(fill=mat, region=box)]))
    settings = om.Settings(particles=2000, batches=1, event_based=True, seed=3)
    settings.source = [om.IndependentSource(space=om.Point((0.0, 0.0, 0.0)), angle=om.Isotropic(),
                                            energy=om.Discrete([1.0e6], [1.0]))]
    t = om.Tally(name="flux")
    t.scores = ["flux"]
    m = om.Model(geom, mats, settings, om.Tallies([t]))
    m.export_to_model_xml(directory / "model.xml")
    return nuc


def energy_ratios(path, fp32, e_min):
    from openmc_gb300 import lib
    lib.init(directory=path)
    try:
        lib.settings.xs_fp32 = 1 if fp32 else 0
        lib.set_trace(2000, 400)
        lib.simulation_init()
        lib.next_batch()
        rec, cnt = lib.get_trace()
        lib.simulation_finalize()
    finally:
        lib.finalize()
    out = []
    for h in range(rec.shape[0]):
        n = min(int(cnt[h]), rec.shape[1])
        r = rec[h, :n]
        # collisions followed by another event, above the free-gas threshold
        coll = np.nonzero((r["kind"][:-1] == 2) & (r["E"][:-1] > e_min))[0]
        out.append(r["E"][coll + 1] / r["E"][coll])
    return np.concatenate(out)


@pytest.mark.parametrize("fp32", [False, True], ids=["fp64", "fp32"])
def test_elastic_energy_transfer_law(built, tmp_path, fp32):
    nuc = scatter_box(tmp_path)
    alpha = ((nuc.awr - 1.0) / (nuc.awr + 1.0)) ** 2
    # the target is at rest above 400 kT (slower histories scatter off a
    # moving target, src/physics.cpp:754-818)
    q = energy_ratios(tmp_path, fp32, 400.0 * nuc.kT)
    n = q.size
    assert n > 100_000, n
    # kinematic limits, to the rounding of the arithmetic
    assert q.min() >= alpha * (1.0 - 1e-6), (q.min(), alpha)
    assert q.max() <= 1.0 + 1e-6, q.max()
    mean, var = (1.0 + alpha) / 2.0, (1.0 - alpha) ** 2 / 12.0
    assert abs(q.mean() - mean) < 5.0 * np.sqrt(var / n), (q.mean(), mean)
    # sample variance of a uniform law: relative standard error sqrt(0.8 / n)
    assert abs(q.var() / var - 1.0) < 5.0 * np.sqrt(0.8 / n), (q.var(), var)
    # uniform on [alpha, 1]: each tenth of the interval holds a tenth of the ratios
    hist, _ = np.histogram(q, bins=10, range=(alpha, 1.0))
    assert np.all(np.abs(hist / n - 0.1) < 5.0 * np.sqrt(0.09 / n)), hist / n


def inner_box_model(directory):
    """A 20 cm box around an inner 10 cm box cell, a 7x5x3 mesh over the
    inner box only, and a point source at the centre: tracks leave the mesh,
    re-enter it from outside and start on its faces."""
    from openmc_gb300 import configs, data
    from openmc_gb300 import model as om
    _, xs_xml = configs._library(directory, [("H1", 1), ("O16", 16), ("Fe56", 56)], 600, 5)
    mat = om.Material(name="mixture")
    for name, f in (("H1", 0.5), ("O16", 0.3), ("Fe56", 0.2)):
        mat.add_nuclide(name, f)
    mat.set_density("atom/b-cm", 0.03)
    mats = om.Materials([mat], cross_sections=xs_xml.name)
    outer = [om.XPlane(-10.0, boundary_type="reflective"), om.XPlane(10.0, boundary_type="vacuum"),
             om.YPlane(-10.0, boundary_type="vacuum"), om.YPlane(10.0, boundary_type="reflective"),
             om.ZPlane(-10.0, boundary_type="vacuum"), om.ZPlane(10.0, boundary_type="vacuum")]
    inner = [om.XPlane(-5.0), om.XPlane(5.0), om.YPlane(-5.0), om.YPlane(5.0), om.ZPlane(-5.0), om.ZPlane(5.0)]
    big = +outer[0] & -outer[1] & +outer[2] & -outer[3] & +outer[4] & -outer[5]
    small = +inner[0] & -inner[1] & +inner[2] & -inner[3] & +inner[4] & -inner[5]
    c_in = om.Cell(fill=mat, region=small)
    c_out = om.Cell(fill=mat, region=big & ~small)
    geom = om.Geometry(om.Universe(cells=[c_in, c_out]))
    settings = om.Settings(particles=20000, batches=2, event_based=True, seed=9)
    settings.source = [om.IndependentSource(space=om.Point((0.0, 0.0, 0.0)), angle=om.Isotropic(),
                                            energy=om.Discrete([2.0e6], [1.0]))]
    mesh = om.RegularMesh()
    mesh.dimension = [7, 5, 3]
    mesh.lower_left = [-5.0, -5.0, -5.0]
    mesh.upper_right = [5.0, 5.0, 5.0]
    tm = om.Tally(name="mesh flux")
    tm.filters = [om.MeshFilter(mesh)]
    tm.scores = ["flux"]
    tc = om.Tally(name="inner cell flux")
    tc.filters = [om.CellFilter([c_in])]
    tc.scores = ["flux"]
    tc.estimator = "tracklength"
    m = om.Model(geom, mats, settings, om.Tallies([tm, tc]))
    m.export_to_model_xml(directory / "model.xml")
    return m


@pytest.mark.parametrize("fp32", [False, True], ids=["fp64", "fp32"])
def test_mesh_walk_conserves_track_length(built, tmp_path, fp32):
    """Over a mesh that covers exactly one cell, the mesh bins' track-length
    flux sums to that cell's track-length flux in the same run (the walk of
    src/mesh.cpp:999-1146 splits each track without losing length): to FP64
    rounding with FP64 tables, to the FP32 walk's rounding with FP32 tables
    (its faces are exact in FP32 here, so only the fractions round)."""
    from openmc_gb300 import lib
    inner_box_model(tmp_path)
    lib.init(directory=tmp_path)
    try:
        lib.settings.xs_fp32 = 1 if fp32 else 0
        lib.simulation_init()
        status = 0
        while status == 0:
            status = lib.next_batch()
        lib.simulation_finalize()
        ids = lib.tally_ids()
        mesh_sum = lib.tally_results(ids[0])[..., 1].sum()
        cell = lib.tally_results(ids[1])[..., 1].sum()
    finally:
        lib.finalize()
    assert cell > 0
    assert abs(mesh_sum - cell) <= (1e-6 if fp32 else 1e-11) * cell, (mesh_sum, cell)
