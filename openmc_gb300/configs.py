"""The benchmark models of this project, built with :mod:`openmc_gb300.model`.

* ``point_cube``     20 cm vacuum cube, two concentric z-cylinders (r=1, 3 cm)
                     of one 4-nuclide mixture (A = 1, 12, 16, 56), 1 MeV
                     isotropic point source, flux on a 10x10x10 mesh x 50
                     log-energy bins.
* ``lattice17``      17x17 pin lattice (pitch 1.26 cm, pin r=0.41, clad
                     r=0.475, 200 cm tall), reflective radial and vacuum axial
                     boundaries, 3 materials from 12 nuclides, Maxwellian
                     (1.3 MeV) source uniform in the pins, flux on a
                     17x17x50 mesh x 100 log-energy bins.
* ``shield``         200x50x50 cm stack of alternating 10 cm light/heavy
                     layers, 1 MeV monodirectional plane source at x=0,
                     flux on a 200x10x10 mesh.
* ``infinite_medium`` eigenvalue run in a reflective cube of one fissile
                     mixture with energy-independent cross sections
                     (k-infinity known exactly).

Every builder writes the nuclide library it needs (seeded, deterministic) and
returns ``(model, directory)``; ``model.export_to_model_xml`` then produces the
``model.xml`` the C library reads.
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

from . import data
from . import model as om

# 24 guide tubes + 1 instrument tube of a 17x17 PWR assembly (row, col).
GUIDE_TUBES = [(2, 5), (2, 8), (2, 11), (3, 3), (3, 13), (5, 2), (5, 5),
               (5, 8), (5, 11), (5, 14), (8, 2), (8, 5), (8, 8), (8, 11),
               (8, 14), (11, 2), (11, 5), (11, 8), (11, 11), (11, 14),
               (13, 3), (13, 13), (14, 5), (14, 8), (14, 11)]


def _library(directory, specs, n_points, seed, fmt="native"):
    nucs = []
    for k, (name, A) in enumerate(specs):
        nucs.append(data.make_nuclide(name, A, n_points, seed * 1000 + k))
    xml = data.write_library(nucs, directory, fmt=fmt)
    return nucs, xml


def log_energy_bins(n, e_min=data.E_MIN, e_max=data.E_MAX):
    return np.exp(np.linspace(np.log(e_min), np.log(e_max), n + 1))


def point_cube(directory, particles=100_000, batches=10, n_points=2000,
               seed=1, event_based=True, mesh_dim=(10, 10, 10), n_ebins=50,
               estimator_tallies=False):
    directory = Path(directory)
    rng = np.random.default_rng(seed)
    specs = [("H1", 1), ("C12", 12), ("O16", 16), ("Fe56", 56)]
    _, xs_xml = _library(directory, specs, n_points, seed)
    frac = rng.uniform(0.2, 1.0, 4)
    frac[0] *= 3.0
    mat = om.Material(name="mixture")
    for (name, _), f in zip(specs, frac / frac.sum()):
        mat.add_nuclide(name, float(f))
    mat.set_density("atom/b-cm", 0.08)
    mats = om.Materials([mat], cross_sections=xs_xml.name)

    planes = [om.XPlane(-10.0, boundary_type="vacuum"), om.XPlane(10.0, boundary_type="vacuum"),
              om.YPlane(-10.0, boundary_type="vacuum"), om.YPlane(10.0, boundary_type="vacuum"),
              om.ZPlane(-10.0, boundary_type="vacuum"), om.ZPlane(10.0, boundary_type="vacuum")]
    box = +planes[0] & -planes[1] & +planes[2] & -planes[3] & +planes[4] & -planes[5]
    c1, c2 = om.ZCylinder(r=1.0), om.ZCylinder(r=3.0)
    cells = [om.Cell(fill=mat, region=-c1 & +planes[4] & -planes[5]),
             om.Cell(fill=mat, region=+c1 & -c2 & +planes[4] & -planes[5]),
             om.Cell(fill=mat, region=+c2 & box)]
    geom = om.Geometry(om.Universe(cells=cells))

    settings = om.Settings(particles=particles, batches=batches,
                           event_based=event_based, seed=1)
    settings.source = [om.IndependentSource(space=om.Point((0.0, 0.0, 0.0)),
                                            angle=om.Isotropic(),
                                            energy=om.Discrete([1.0e6], [1.0]))]
    mesh = om.RegularMesh()
    mesh.dimension = list(mesh_dim)
    mesh.lower_left = [-10.0, -10.0, -10.0]
    mesh.upper_right = [10.0, 10.0, 10.0]
    t = om.Tally(name="mesh flux")
    t.filters = [om.MeshFilter(mesh), om.EnergyFilter(log_energy_bins(n_ebins))]
    t.scores = ["flux"]
    tallies = [t]
    if estimator_tallies:
        # the same quantities with both estimators, binned by cell and by
        # material (src/tallies/filter_cell.cpp, filter_material.cpp)
        groups = om.EnergyFilter([data.E_MIN, 1.0, 1.0e3, 1.0e5, data.E_MAX])
        for est in ("tracklength", "collision"):
            tc = om.Tally(name=f"cell {est}")
            tc.filters = [om.CellFilter(cells), groups]
            tc.scores = ["flux", "total", "absorption"]
            tc.estimator = est
            tm = om.Tally(name=f"material {est}")
            tm.filters = [om.MaterialFilter([mat])]
            tm.scores = ["flux", "absorption"]
            tm.estimator = est
            te = om.Tally(name=f"mesh {est}")
            te.filters = [om.MeshFilter(mesh)]
            te.scores = ["flux"]
            te.estimator = est
            tallies += [tc, tm, te]
    return om.Model(geom, mats, settings, om.Tallies(tallies)), directory


def infinite_medium(directory, particles=20_000, batches=30, inactive=10, n_points=500, seed=7,
                    event_based=True, fissile_fraction=0.045, library_format="native"):
    """Eigenvalue run in an infinite homogeneous medium: a reflective 20 cm
    cube of one material made of a fissile nuclide and a light moderator
    whose cross sections do not depend on energy, so that
    k-infinity = nu Sigma_f / Sigma_a exactly (returned as the model's
    ``k_inf`` attribute); flux tally on a 4x4x4 mesh."""
    directory = Path(directory)
    nu, sf, sc_f, se_f = 2.43, 8.0, 5.0, 10.0
    sc_m, se_m = 0.3, 20.0
    nucs = [data.make_flat_nuclide("Fx235", 235, n_points, seed, se_f, sc_f, fission=sf, nu=nu),
            data.make_flat_nuclide("Mx1", 1, n_points, seed + 1, se_m, sc_m)]
    xs_xml = data.write_library(nucs, directory, fmt=library_format)
    mat = om.Material(name="fissile mixture")
    mat.add_nuclide("Fx235", fissile_fraction)
    mat.add_nuclide("Mx1", 1.0 - fissile_fraction)
    mat.set_density("atom/b-cm", 0.1)
    mats = om.Materials([mat], cross_sections=xs_xml.name)
    planes = [om.XPlane(-10.0, boundary_type="reflective"), om.XPlane(10.0, boundary_type="reflective"),
              om.YPlane(-10.0, boundary_type="reflective"), om.YPlane(10.0, boundary_type="reflective"),
              om.ZPlane(-10.0, boundary_type="reflective"), om.ZPlane(10.0, boundary_type="reflective")]
    box = +planes[0] & -planes[1] & +planes[2] & -planes[3] & +planes[4] & -planes[5]
    geom = om.Geometry(om.Universe(cells=[om.Cell(fill=mat, region=box)]))
    settings = om.Settings(run_mode="eigenvalue", particles=particles, batches=batches, inactive=inactive,
                           event_based=event_based, seed=1)
    settings.source = [om.IndependentSource(space=om.Box((-10.0, -10.0, -10.0), (10.0, 10.0, 10.0)),
                                            angle=om.Isotropic(), energy=om.Maxwell(1.3e6))]
    mesh = om.RegularMesh()
    mesh.dimension = [4, 4, 4]
    mesh.lower_left = [-10.0, -10.0, -10.0]
    mesh.upper_right = [10.0, 10.0, 10.0]
    t = om.Tally(name="mesh flux")
    t.filters = [om.MeshFilter(mesh)]
    t.scores = ["flux"]
    model = om.Model(geom, mats, settings, om.Tallies([t]))
    f = fissile_fraction
    model.k_inf = nu * f * sf / (f * (sc_f + sf) + (1.0 - f) * sc_m)
    return model, directory


def _pin_universe(fuel, clad, mod, r_pin=0.41, r_clad=0.475, guide=False):
    s1, s2 = om.ZCylinder(r=r_pin), om.ZCylinder(r=r_clad)
    inner = mod if guide else fuel
    return om.Universe(cells=[om.Cell(fill=inner, region=-s1),
                              om.Cell(fill=clad, region=+s1 & -s2),
                              om.Cell(fill=mod, region=+s2)])


def _lattice_materials(directory, n_points, seed, fmt="native"):
    specs = [("Hv235", 235), ("Hv238", 238), ("Ox16", 16), ("Hv240", 240),
             ("Cl56", 56), ("Cl58", 58), ("Cl90", 90), ("Cl91", 91),
             ("Lt1", 1), ("Lt2", 2), ("Lt16", 16), ("Lt10", 10)]
    _, xs_xml = _library(directory, specs, n_points, seed, fmt)
    rng = np.random.default_rng(seed + 17)

    def mixture(name, names, weights, density):
        m = om.Material(name=name)
        w = np.asarray(weights) * rng.uniform(0.9, 1.1, len(weights))
        for n, f in zip(names, w / w.sum()):
            m.add_nuclide(n, float(f))
        m.set_density("atom/b-cm", density)
        return m

    fuel = mixture("heavy absorber", ["Hv235", "Hv238", "Ox16", "Hv240"],
                   [0.03, 0.30, 0.66, 0.01], 0.069)
    clad = mixture("clad", ["Cl56", "Cl58", "Cl90", "Cl91"],
                   [0.6, 0.2, 0.15, 0.05], 0.043)
    mod = mixture("light scatterer", ["Lt1", "Lt2", "Lt16", "Lt10"],
                  [0.66, 0.001, 0.33, 0.009], 0.1)
    return fuel, clad, mod, xs_xml


def lattice17(directory, particles=10_000_000, batches=20, n_points=11303,
              seed=3, event_based=True, mesh_dim=(17, 17, 50), n_ebins=100,
              height=200.0, library_format="native"):
    directory = Path(directory)
    fuel, clad, mod, xs_xml = _lattice_materials(directory, n_points, seed, library_format)
    mats = om.Materials([fuel, clad, mod], cross_sections=xs_xml.name)
    pin = _pin_universe(fuel, clad, mod)
    gt = _pin_universe(fuel, clad, mod, r_pin=0.56, r_clad=0.60, guide=True)
    pitch, n = 1.26, 17
    half = pitch * n / 2.0
    lat = om.RectLattice()
    lat.pitch = [pitch, pitch]
    lat.lower_left = [-half, -half]
    rows = [[pin] * n for _ in range(n)]
    for (i, j) in GUIDE_TUBES:
        rows[i][j] = gt
    lat.universes = rows
    xs = [om.XPlane(-half, boundary_type="reflective"), om.XPlane(half, boundary_type="reflective"),
          om.YPlane(-half, boundary_type="reflective"), om.YPlane(half, boundary_type="reflective"),
          om.ZPlane(-height / 2, boundary_type="vacuum"), om.ZPlane(height / 2, boundary_type="vacuum")]
    region = +xs[0] & -xs[1] & +xs[2] & -xs[3] & +xs[4] & -xs[5]
    root = om.Universe(cells=[om.Cell(fill=lat, region=region)])
    geom = om.Geometry(root)
    settings = om.Settings(particles=particles, batches=batches,
                           event_based=event_based, seed=1)
    settings.source = [om.IndependentSource(
        space=om.Box((-half, -half, -height / 2), (half, half, height / 2)),
        angle=om.Isotropic(), energy=om.Maxwell(1.3e6),
        constraints={"domains": [fuel]})]
    mesh = om.RegularMesh()
    mesh.dimension = list(mesh_dim)
    mesh.lower_left = [-half, -half, -height / 2]
    mesh.upper_right = [half, half, height / 2]
    t = om.Tally(name="lattice flux")
    t.filters = [om.MeshFilter(mesh), om.EnergyFilter(log_energy_bins(n_ebins))]
    return om.Model(geom, mats, settings, om.Tallies([t])), directory


def shield_materials(directory, n_points, seed, density_scale=1.0):
    specs = [("Lt1", 1), ("Lt16", 16), ("Lt10", 10), ("Lt2", 2),
             ("Cl56", 56), ("Cl58", 58), ("Cl54", 54), ("Cl52", 52)]
    _, xs_xml = _library(directory, specs, n_points, seed)
    light = om.Material(name="light scatterer")
    for n, f in zip(["Lt1", "Lt16", "Lt10", "Lt2"], [0.66, 0.32, 0.019, 0.001]):
        light.add_nuclide(n, f)
    light.set_density("atom/b-cm", 0.1 * density_scale)
    heavy = om.Material(name="heavy absorber")
    for n, f in zip(["Cl56", "Cl58", "Cl54", "Cl52"], [0.72, 0.18, 0.06, 0.04]):
        heavy.add_nuclide(n, f)
    heavy.set_density("atom/b-cm", 0.085 * density_scale)
    return light, heavy, xs_xml


def shield(directory, particles=1_000_000, batches=10, n_points=11303, seed=4,
           event_based=True, length=200.0, width=50.0, layer=10.0,
           mesh_dim=(200, 10, 10), weight_windows=None, back_face=10.0,
           energy_groups=None, tally_mesh_windows=False, density_scale=1.0):
    """Deep-penetration slab shield.  energy_groups: bounds [eV] of an
    energy filter on the mesh flux tally; tally_mesh_windows: add weight
    windows on the flux tally's mesh and energy groups with every bound at
    -1 (no window until a generator or the caller sets them)."""
    directory = Path(directory)
    light, heavy, xs_xml = shield_materials(directory, n_points, seed, density_scale)
    mats = om.Materials([light, heavy], cross_sections=xs_xml.name)
    n_layers = int(round(length / layer))
    xp = [om.XPlane(k * layer) for k in range(n_layers + 1)]
    xp[0].boundary_type = "vacuum"
    xp[-1].boundary_type = "vacuum"
    hw = width / 2.0
    side = (+om.YPlane(-hw, boundary_type="vacuum") & -om.YPlane(hw, boundary_type="vacuum")
            & +om.ZPlane(-hw, boundary_type="vacuum") & -om.ZPlane(hw, boundary_type="vacuum"))
    cells = [om.Cell(fill=(light if k % 2 == 0 else heavy), region=+xp[k] & -xp[k + 1] & side)
             for k in range(n_layers)]
    geom = om.Geometry(om.Universe(cells=cells))
    settings = om.Settings(particles=particles, batches=batches,
                           event_based=event_based, seed=1)
    settings.source = [om.IndependentSource(
        space=om.Box((1.0e-6, -hw, -hw), (1.0e-6, hw, hw)),
        angle=om.Monodirectional((1.0, 0.0, 0.0)),
        energy=om.Discrete([1.0e6], [1.0]))]
    mesh = om.RegularMesh()
    mesh.dimension = list(mesh_dim)
    mesh.lower_left = [0.0, -hw, -hw]
    mesh.upper_right = [length, hw, hw]
    t = om.Tally(name="shield flux")
    t.filters = [om.MeshFilter(mesh)]
    ebounds = [0.0, 2.0e7 * 1.000001]
    if energy_groups is not None:
        ebounds = [float(e) for e in energy_groups]
        t.filters.append(om.EnergyFilter(ebounds))
    back = om.RegularMesh()
    back.dimension = [1, 1, 1]
    back.lower_left = [length - back_face, -hw, -hw]
    back.upper_right = [length, hw, hw]
    tb = om.Tally(name="back face flux")
    tb.filters = [om.MeshFilter(back)]
    depth = om.RegularMesh()
    depth.dimension = [n_layers, 1, 1]
    depth.lower_left = [0.0, -hw, -hw]
    depth.upper_right = [length, hw, hw]
    tp = om.Tally(name="flux per layer")
    tp.filters = [om.MeshFilter(depth)]
    if tally_mesh_windows:
        n = int(np.prod(mesh_dim)) * (len(ebounds) - 1)
        weight_windows = om.WeightWindows(mesh, -np.ones(n), upper_ww_bounds=-np.ones(n),
                                          energy_bounds=ebounds)
    if weight_windows is not None:
        settings.weight_windows = [weight_windows]
        settings.weight_windows_on = True
    return om.Model(geom, mats, settings, om.Tallies([t, tb, tp])), directory


def full_scale(directory, particles=100_000_000, batches=50, n_points=11303, seed=3,
               event_based=True, shield_layers=10, layer=10.0, height=200.0,
               mesh_dim=(100, 100, 60), n_ebins=50, ww_mesh_dim=None, ww_groups=None):
    """The 17x17 lattice wrapped in a layered shield: alternating 10 cm
    shells of the lattice's light scatterer and A=56-like clad material
    around the lattice box (vacuum outside and at the axial ends), 68
    synthetic nuclides (the lattice's 12 plus 56 trace nuclides spread over
    the materials), source in the fuel, flux on a 100 x 100 x 60 mesh x 50
    energy bins over the whole assembly (3e7 bins), and a flux tally on the
    outermost shell.  ww_mesh_dim / ww_groups add weight windows (all -1) on
    a mesh of that shape over the assembly with those energy bounds, plus a
    flux tally on the same mesh and groups (for pilot runs)."""
    directory = Path(directory)
    specs = [("Hv235", 235), ("Hv238", 238), ("Ox16", 16), ("Hv240", 240),
             ("Cl56", 56), ("Cl58", 58), ("Cl90", 90), ("Cl91", 91),
             ("Lt1", 1), ("Lt2", 2), ("Lt16", 16), ("Lt10", 10)]
    rng = np.random.default_rng(seed + 101)
    extra = [(f"Tr{k:02d}", int(a)) for k, a in enumerate(rng.integers(20, 245, 56))]
    _, xs_xml = _library(directory, specs + extra, n_points, seed)

    def mixture(name, names, weights, density):
        m = om.Material(name=name)
        w = np.asarray(weights, float)
        for n, f in zip(names, w / w.sum()):
            m.add_nuclide(n, float(f))
        m.set_density("atom/b-cm", density)
        return m

    tr = [n for n, _ in extra]
    fuel = mixture("heavy absorber", ["Hv235", "Hv238", "Ox16", "Hv240"] + tr[:32],
                   [0.03, 0.30, 0.66, 0.01] + [2e-4] * 32, 0.069)
    clad = mixture("clad", ["Cl56", "Cl58", "Cl90", "Cl91"] + tr[32:48],
                   [0.6, 0.2, 0.15, 0.05] + [1e-3] * 16, 0.043)
    mod = mixture("light scatterer", ["Lt1", "Lt2", "Lt16", "Lt10"] + tr[48:],
                  [0.66, 0.001, 0.33, 0.009] + [1e-4] * 8, 0.1)
    mats = om.Materials([fuel, clad, mod], cross_sections=xs_xml.name)
    pin = _pin_universe(fuel, clad, mod)
    gt = _pin_universe(fuel, clad, mod, r_pin=0.56, r_clad=0.60, guide=True)
    pitch, n = 1.26, 17
    half = pitch * n / 2.0
    lat = om.RectLattice()
    lat.pitch = [pitch, pitch]
    lat.lower_left = [-half, -half]
    rows = [[pin] * n for _ in range(n)]
    for (i, j) in GUIDE_TUBES:
        rows[i][j] = gt
    lat.universes = rows
    zlo = om.ZPlane(-height / 2, boundary_type="vacuum")
    zhi = om.ZPlane(height / 2, boundary_type="vacuum")
    hws = [half + k * layer for k in range(shield_layers + 1)]
    xm = [om.XPlane(-h) for h in hws]
    xp = [om.XPlane(h) for h in hws]
    ym = [om.YPlane(-h) for h in hws]
    yp = [om.YPlane(h) for h in hws]
    for s in (xm[-1], xp[-1], ym[-1], yp[-1]):
        s.boundary_type = "vacuum"

    def box(k):
        return +xm[k] & -xp[k] & +ym[k] & -yp[k]

    cells = [om.Cell(fill=lat, region=box(0) & +zlo & -zhi)]
    for k in range(shield_layers):
        cells.append(om.Cell(fill=(mod if k % 2 == 0 else clad),
                             region=box(k + 1) & ~box(k) & +zlo & -zhi))
    geom = om.Geometry(om.Universe(cells=cells))
    settings = om.Settings(particles=particles, batches=batches, event_based=event_based, seed=1)
    settings.source = [om.IndependentSource(
        space=om.Box((-half, -half, -height / 2), (half, half, height / 2)),
        angle=om.Isotropic(), energy=om.Maxwell(1.3e6),
        constraints={"domains": [fuel]})]
    outer = hws[-1]
    mesh = om.RegularMesh()
    mesh.dimension = list(mesh_dim)
    mesh.lower_left = [-outer, -outer, -height / 2]
    mesh.upper_right = [outer, outer, height / 2]
    t = om.Tally(name="assembly flux")
    t.filters = [om.MeshFilter(mesh), om.EnergyFilter(log_energy_bins(n_ebins))]
    # flux in the outermost shell: a 2x2x1 mesh bins the whole assembly; the
    # outer shell is recovered by the caller from the layer tally below
    shell = om.RegularMesh()
    shell.dimension = [2 * shield_layers + 1, 1, 1]
    shell.lower_left = [-outer, -half, -height / 2]
    shell.upper_right = [outer, half, height / 2]
    ts = om.Tally(name="flux across the shells (x slab through the lattice)")
    ts.filters = [om.MeshFilter(shell)]
    tallies = [t, ts]
    if ww_mesh_dim is not None:
        groups = [float(e) for e in (ww_groups if ww_groups is not None else [0.0, 2.0e7 * 1.000001])]
        wm = om.RegularMesh()
        wm.dimension = list(ww_mesh_dim)
        wm.lower_left = [-outer, -outer, -height / 2]
        wm.upper_right = [outer, outer, height / 2]
        tw = om.Tally(name="window mesh flux")
        tw.filters = [om.MeshFilter(wm)]
        if len(groups) > 2:
            tw.filters.append(om.EnergyFilter(groups))
        tallies.append(tw)
        nb = int(np.prod(ww_mesh_dim)) * (len(groups) - 1)
        settings.weight_windows = [om.WeightWindows(wm, -np.ones(nb), upper_ww_bounds=-np.ones(nb),
                                                    energy_bounds=groups)]
        settings.weight_windows_on = True
    return om.Model(geom, mats, settings, om.Tallies(tallies)), directory
