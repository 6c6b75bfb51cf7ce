"""Model building surface that writes OpenMC's ``model.xml`` schema.

The reference user builds an ``openmc.Model`` (``openmc/model/model.py:36``)
from materials, CSG geometry, settings and tallies, and either calls
``Model.run(event_based=True)`` or drives ``openmc.lib``.  The reference
Python package cannot be imported on the machines this package targets (it
needs h5py, lxml and pandas), so this module provides the subset of that API
the event-based transport path consumes, with the same class names, argument
names and XML output:

* materials with nuclide atom fractions and an ``atom/b-cm`` or ``sum`` density
  (``openmc/material.py``);
* x/y/z-planes and x/y/z-cylinders with vacuum/reflective/transmission
  boundaries, half-space regions with ``&``, ``|`` and ``~``
  (``openmc/surface.py``, ``openmc/region.py``);
* cells filled by a material, a universe or a rectangular lattice, with
  translation (``openmc/cell.py``, ``openmc/lattice.py``);
* independent sources: point or box space with optional domain constraints,
  isotropic or monodirectional angle, discrete or Maxwell energy
  (``openmc/source.py``, ``openmc/stats``);
* regular meshes, mesh/energy/particle/cell/material filters and
  flux/total/absorption scores with track-length or collision estimators
  (``openmc/tallies.py``, ``openmc/filter.py``);
* weight windows and MAGIC weight-window generators
  (``openmc/weight_windows.py``).
"""
from __future__ import annotations

import itertools
import os
import subprocess
from pathlib import Path
from xml.etree import ElementTree as ET

import numpy as np

_ids = {k: itertools.count(1) for k in
        ("material", "surface", "cell", "universe", "mesh", "filter", "tally",
         "weight_windows")}


def _next_id(kind, value):
    if value is not None:
        return int(value)
    return next(_ids[kind])


def reset_auto_ids():
    for k in _ids:
        _ids[k] = itertools.count(1)


def _fmt(values):
    return " ".join(repr(float(v)) if isinstance(v, (float, np.floating))
                    else str(v) for v in np.ravel(values).tolist())


# ---------------------------------------------------------------------------
# Materials
# ---------------------------------------------------------------------------

class Material:
    def __init__(self, material_id=None, name=""):
        self.id = _next_id("material", material_id)
        self.name = name
        self.nuclides = []  # (name, percent, type)
        self.density = None
        self.density_units = "atom/b-cm"
        self.temperature = None

    def add_nuclide(self, nuclide, percent, percent_type="ao"):
        if percent_type != "ao":
            raise ValueError("only atom fractions ('ao') are supported")
        self.nuclides.append((nuclide, float(percent), percent_type))

    def set_density(self, units, density=None):
        if units not in ("atom/b-cm", "sum"):
            raise ValueError("density units must be 'atom/b-cm' or 'sum'")
        self.density_units = units
        self.density = density

    def to_xml(self):
        el = ET.Element("material", id=str(self.id))
        if self.name:
            el.set("name", self.name)
        if self.temperature is not None:
            el.set("temperature", repr(float(self.temperature)))
        d = ET.SubElement(el, "density", units=self.density_units)
        if self.density is not None:
            d.set("value", repr(float(self.density)))
        for nuc, pct, typ in self.nuclides:
            ET.SubElement(el, "nuclide", name=nuc, **{typ: repr(pct)})
        return el


class Materials(list):
    def __init__(self, materials=(), cross_sections=None):
        super().__init__(materials)
        self.cross_sections = cross_sections

    def to_xml(self):
        el = ET.Element("materials")
        if self.cross_sections is not None:
            ET.SubElement(el, "cross_sections").text = str(self.cross_sections)
        for m in self:
            el.append(m.to_xml())
        return el


# ---------------------------------------------------------------------------
# Surfaces and regions
# ---------------------------------------------------------------------------

class Region:
    def __and__(self, other):
        return Intersection([self, other])

    def __or__(self, other):
        return Union([self, other])

    def __invert__(self):
        return Complement(self)


class Halfspace(Region):
    def __init__(self, surface, side):
        self.surface, self.side = surface, side

    def __str__(self):
        return f"{self.side}{self.surface.id}" if self.side == "-" else str(self.surface.id)


class Intersection(Region):
    def __init__(self, nodes):
        self.nodes = []
        for n in nodes:
            self.nodes.extend(n.nodes if isinstance(n, Intersection) else [n])

    def __str__(self):
        return " ".join(f"({n})" if isinstance(n, Union) else str(n) for n in self.nodes)


class Union(Region):
    def __init__(self, nodes):
        self.nodes = []
        for n in nodes:
            self.nodes.extend(n.nodes if isinstance(n, Union) else [n])

    def __str__(self):
        return " | ".join(f"({n})" if isinstance(n, Intersection) else str(n) for n in self.nodes)


class Complement(Region):
    def __init__(self, node):
        self.node = node

    def __str__(self):
        return f"~({self.node})"


class Surface:
    _type = None
    _coeff_names = ()

    def __init__(self, surface_id=None, boundary_type="transmission", **coeffs):
        self.id = _next_id("surface", surface_id)
        if boundary_type not in ("transmission", "vacuum", "reflective"):
            raise ValueError(f"unsupported boundary type {boundary_type}")
        self.boundary_type = boundary_type
        self.coeffs = [float(coeffs.get(k, 0.0)) for k in self._coeff_names]

    def __neg__(self):
        return Halfspace(self, "-")

    def __pos__(self):
        return Halfspace(self, "+")

    def to_xml(self):
        el = ET.Element("surface", id=str(self.id), type=self._type,
                        coeffs=_fmt(self.coeffs))
        if self.boundary_type != "transmission":
            el.set("boundary", self.boundary_type)
        return el


def _surface_class(name, tname, coeff_names):
    def __init__(self, *args, surface_id=None, boundary_type="transmission", **kw):
        kw.update(dict(zip(coeff_names, args)))
        Surface.__init__(self, surface_id, boundary_type, **kw)
    return type(name, (Surface,), {"_type": tname, "_coeff_names": coeff_names,
                                   "__init__": __init__})


XPlane = _surface_class("XPlane", "x-plane", ("x0",))
YPlane = _surface_class("YPlane", "y-plane", ("y0",))
ZPlane = _surface_class("ZPlane", "z-plane", ("z0",))
XCylinder = _surface_class("XCylinder", "x-cylinder", ("y0", "z0", "r"))
YCylinder = _surface_class("YCylinder", "y-cylinder", ("x0", "z0", "r"))
ZCylinder = _surface_class("ZCylinder", "z-cylinder", ("x0", "y0", "r"))
Sphere = _surface_class("Sphere", "sphere", ("x0", "y0", "z0", "r"))


# ---------------------------------------------------------------------------
# Cells, universes, lattices
# ---------------------------------------------------------------------------

class Cell:
    def __init__(self, cell_id=None, name="", fill=None, region=None):
        self.id = _next_id("cell", cell_id)
        self.name = name
        self.fill = fill
        self.region = region
        self.translation = None


class Universe:
    def __init__(self, universe_id=None, name="", cells=()):
        self.id = _next_id("universe", universe_id)
        self.name = name
        self.cells = list(cells)

    def add_cell(self, cell):
        self.cells.append(cell)


class RectLattice:
    def __init__(self, lattice_id=None, name=""):
        self.id = _next_id("universe", lattice_id)
        self.name = name
        self.lower_left = None
        self.pitch = None
        self.universes = None  # nested [z][y][x] or [y][x], y listed top-down
        self.outer = None


class Geometry:
    def __init__(self, root):
        self.root_universe = root if isinstance(root, Universe) else Universe(cells=root)

    def _collect(self):
        universes, lattices, cells, surfaces = {}, {}, {}, {}

        def region_surfaces(reg):
            if reg is None:
                return
            if isinstance(reg, Halfspace):
                surfaces[reg.surface.id] = reg.surface
            elif isinstance(reg, (Intersection, Union)):
                for n in reg.nodes:
                    region_surfaces(n)
            elif isinstance(reg, Complement):
                region_surfaces(reg.node)

        def visit_universe(u):
            if u.id in universes:
                return
            universes[u.id] = u
            for c in u.cells:
                cells[c.id] = (c, u.id)
                region_surfaces(c.region)
                if isinstance(c.fill, Universe):
                    visit_universe(c.fill)
                elif isinstance(c.fill, RectLattice):
                    visit_lattice(c.fill)

        def visit_lattice(lat):
            if lat.id in lattices:
                return
            lattices[lat.id] = lat
            for u in np.ravel(np.asarray(lat.universes, dtype=object)):
                visit_universe(u)
            if lat.outer is not None:
                visit_universe(lat.outer)

        visit_universe(self.root_universe)
        return universes, lattices, cells, surfaces

    def to_xml(self):
        universes, lattices, cells, surfaces = self._collect()
        el = ET.Element("geometry")
        for sid in sorted(surfaces):
            el.append(surfaces[sid].to_xml())
        for cid in sorted(cells):
            c, uid = cells[cid]
            ce = ET.SubElement(el, "cell", id=str(c.id), universe=str(uid))
            if c.name:
                ce.set("name", c.name)
            if c.fill is None:
                ce.set("material", "void")
            elif isinstance(c.fill, Material):
                ce.set("material", str(c.fill.id))
            else:
                ce.set("fill", str(c.fill.id))
            if c.region is not None:
                ce.set("region", str(c.region))
            if c.translation is not None:
                ce.set("translation", _fmt(c.translation))
        for lid in sorted(lattices):
            lat = lattices[lid]
            le = ET.SubElement(el, "lattice", id=str(lat.id))
            arr = np.asarray(lat.universes, dtype=object)
            dims = list(arr.shape[::-1])  # x, y, (z)
            ET.SubElement(le, "pitch").text = _fmt(lat.pitch)
            if lat.outer is not None:
                ET.SubElement(le, "outer").text = str(lat.outer.id)
            ET.SubElement(le, "dimension").text = _fmt(dims)
            ET.SubElement(le, "lower_left").text = _fmt(lat.lower_left)
            ids = np.vectorize(lambda u: u.id)(arr)
            ET.SubElement(le, "universes").text = "\n" + "\n".join(
                " ".join(str(v) for v in row) for row in ids.reshape(-1, dims[0])) + "\n"
        return el


# ---------------------------------------------------------------------------
# Source distributions (openmc.stats subset)
# ---------------------------------------------------------------------------

class Point:
    def __init__(self, xyz=(0.0, 0.0, 0.0)):
        self.xyz = tuple(float(v) for v in xyz)

    def to_xml(self, tag="space"):
        el = ET.Element(tag, type="point")
        ET.SubElement(el, "parameters").text = _fmt(self.xyz)
        return el


class Box:
    def __init__(self, lower_left, upper_right):
        self.lower_left, self.upper_right = tuple(lower_left), tuple(upper_right)

    def to_xml(self, tag="space"):
        el = ET.Element(tag, type="box")
        ET.SubElement(el, "parameters").text = _fmt(self.lower_left + self.upper_right)
        return el


class Isotropic:
    def to_xml(self, tag="angle"):
        return ET.Element(tag, type="isotropic")


class Monodirectional:
    def __init__(self, reference_uvw=(1.0, 0.0, 0.0)):
        self.reference_uvw = tuple(float(v) for v in reference_uvw)

    def to_xml(self, tag="angle"):
        return ET.Element(tag, type="monodirectional", reference_uvw=_fmt(self.reference_uvw))


class Discrete:
    def __init__(self, x, p):
        self.x, self.p = list(np.atleast_1d(x)), list(np.atleast_1d(p))

    def to_xml(self, tag="energy"):
        el = ET.Element(tag, type="discrete")
        ET.SubElement(el, "parameters").text = _fmt(self.x + self.p)
        return el


class Maxwell:
    def __init__(self, theta):
        self.theta = float(theta)

    def to_xml(self, tag="energy"):
        el = ET.Element(tag, type="maxwell")
        ET.SubElement(el, "parameters").text = repr(self.theta)
        return el


class IndependentSource:
    def __init__(self, space=None, angle=None, energy=None, strength=1.0,
                 constraints=None):
        self.space = space or Point()
        self.angle = angle or Isotropic()
        self.energy = energy or Discrete([1.0e6], [1.0])
        self.strength = float(strength)
        self.constraints = constraints or {}

    def to_xml(self):
        el = ET.Element("source", type="independent", strength=repr(self.strength),
                        particle="neutron")
        el.append(self.space.to_xml("space"))
        el.append(self.angle.to_xml("angle"))
        el.append(self.energy.to_xml("energy"))
        if self.constraints:
            ce = ET.SubElement(el, "constraints")
            dom = self.constraints.get("domains")
            if dom:
                kind = {Material: "material", Cell: "cell", Universe: "universe"}[type(dom[0])]
                ET.SubElement(ce, "domain_type").text = kind
                ET.SubElement(ce, "domain_ids").text = " ".join(str(d.id) for d in dom)
            if "energy_bounds" in self.constraints:
                ET.SubElement(ce, "energy_bounds").text = _fmt(self.constraints["energy_bounds"])
            if "rejection_strategy" in self.constraints:
                ET.SubElement(ce, "rejection_strategy").text = self.constraints["rejection_strategy"]
        return el


# ---------------------------------------------------------------------------
# Meshes, filters, tallies
# ---------------------------------------------------------------------------

class RegularMesh:
    def __init__(self, mesh_id=None, name=""):
        self.id = _next_id("mesh", mesh_id)
        self.name = name
        self.dimension = None
        self.lower_left = None
        self.upper_right = None

    @property
    def n_bins(self):
        return int(np.prod(self.dimension))

    def to_xml(self):
        el = ET.Element("mesh", id=str(self.id), type="regular")
        ET.SubElement(el, "dimension").text = _fmt(self.dimension)
        ET.SubElement(el, "lower_left").text = _fmt(self.lower_left)
        ET.SubElement(el, "upper_right").text = _fmt(self.upper_right)
        return el


class MeshFilter:
    def __init__(self, mesh, filter_id=None):
        self.id = _next_id("filter", filter_id)
        self.mesh = mesh

    def to_xml(self):
        el = ET.Element("filter", id=str(self.id), type="mesh")
        ET.SubElement(el, "bins").text = str(self.mesh.id)
        return el


class EnergyFilter:
    def __init__(self, values, filter_id=None):
        self.id = _next_id("filter", filter_id)
        self.values = np.asarray(values, dtype=float)

    def to_xml(self):
        el = ET.Element("filter", id=str(self.id), type="energy")
        ET.SubElement(el, "bins").text = _fmt(self.values)
        return el


class ParticleFilter:
    def __init__(self, bins=("neutron",), filter_id=None):
        self.id = _next_id("filter", filter_id)
        self.bins = list(bins)

    def to_xml(self):
        el = ET.Element("filter", id=str(self.id), type="particle")
        ET.SubElement(el, "bins").text = " ".join(self.bins)
        return el


class CellFilter:
    """Bins by cell at any coordinate level (openmc/filter.py CellFilter)."""

    def __init__(self, bins, filter_id=None):
        self.id = _next_id("filter", filter_id)
        self.bins = list(bins)

    def to_xml(self):
        el = ET.Element("filter", id=str(self.id), type="cell")
        ET.SubElement(el, "bins").text = " ".join(str(c.id if hasattr(c, "id") else int(c)) for c in self.bins)
        return el


class MaterialFilter:
    """Bins by the particle's material (openmc/filter.py MaterialFilter)."""

    def __init__(self, bins, filter_id=None):
        self.id = _next_id("filter", filter_id)
        self.bins = list(bins)

    def to_xml(self):
        el = ET.Element("filter", id=str(self.id), type="material")
        ET.SubElement(el, "bins").text = " ".join(str(m.id if hasattr(m, "id") else int(m)) for m in self.bins)
        return el


class Tally:
    def __init__(self, tally_id=None, name=""):
        self.id = _next_id("tally", tally_id)
        self.name = name
        self.filters = []
        self.scores = ["flux"]
        self.estimator = "tracklength"

    def to_xml(self):
        el = ET.Element("tally", id=str(self.id))
        if self.name:
            el.set("name", self.name)
        if self.filters:
            ET.SubElement(el, "filters").text = " ".join(str(f.id) for f in self.filters)
        ET.SubElement(el, "scores").text = " ".join(self.scores)
        ET.SubElement(el, "estimator").text = self.estimator
        return el


class Tallies(list):
    def to_xml(self, skip_mesh_ids=()):
        el = ET.Element("tallies")
        meshes, filters = {}, {}
        for t in self:
            for f in t.filters:
                filters[f.id] = f
                if isinstance(f, MeshFilter):
                    meshes[f.mesh.id] = f.mesh
        for mid in sorted(meshes):
            if mid not in skip_mesh_ids:
                el.append(meshes[mid].to_xml())
        for fid in sorted(filters):
            el.append(filters[fid].to_xml())
        for t in self:
            el.append(t.to_xml())
        return el


# ---------------------------------------------------------------------------
# Weight windows
# ---------------------------------------------------------------------------

class WeightWindows:
    def __init__(self, mesh, lower_ww_bounds, upper_ww_bounds=None,
                 upper_bound_ratio=None, energy_bounds=None,
                 particle_type="neutron", survival_ratio=3.0,
                 max_lower_bound_ratio=None, max_split=10, weight_cutoff=1.0e-38,
                 id=None):
        self.id = _next_id("weight_windows", id)
        self.mesh = mesh
        self.lower_ww_bounds = np.asarray(lower_ww_bounds, dtype=float)
        if upper_ww_bounds is None:
            if upper_bound_ratio is None:
                raise ValueError("upper_ww_bounds or upper_bound_ratio required")
            upper_ww_bounds = self.lower_ww_bounds * upper_bound_ratio
        self.upper_ww_bounds = np.asarray(upper_ww_bounds, dtype=float)
        self.energy_bounds = (np.asarray(energy_bounds, dtype=float)
                              if energy_bounds is not None else np.array([0.0, 2.0e7 * 1.000001]))
        self.particle_type = particle_type
        self.survival_ratio = survival_ratio
        self.max_lower_bound_ratio = max_lower_bound_ratio
        self.max_split = max_split
        self.weight_cutoff = weight_cutoff

    def to_xml(self):
        el = ET.Element("weight_windows", id=str(self.id))
        ET.SubElement(el, "mesh").text = str(self.mesh.id)
        ET.SubElement(el, "particle_type").text = self.particle_type
        ET.SubElement(el, "energy_bounds").text = _fmt(self.energy_bounds)
        ET.SubElement(el, "lower_ww_bounds").text = _fmt(self.lower_ww_bounds)
        ET.SubElement(el, "upper_ww_bounds").text = _fmt(self.upper_ww_bounds)
        ET.SubElement(el, "survival_ratio").text = repr(float(self.survival_ratio))
        if self.max_lower_bound_ratio is not None:
            ET.SubElement(el, "max_lower_bound_ratio").text = repr(float(self.max_lower_bound_ratio))
        ET.SubElement(el, "max_split").text = str(int(self.max_split))
        ET.SubElement(el, "weight_cutoff").text = repr(float(self.weight_cutoff))
        return el


class WeightWindowGenerator:
    def __init__(self, mesh, energy_bounds=None, particle_type="neutron",
                 method="magic", max_realizations=1, update_interval=1,
                 on_the_fly=True):
        self.mesh = mesh
        self.energy_bounds = energy_bounds
        self.particle_type = particle_type
        self.method = method
        self.max_realizations = max_realizations
        self.update_interval = update_interval
        self.on_the_fly = on_the_fly
        self.update_parameters = {"value": "mean", "threshold": 1.0, "ratio": 5.0}

    def to_xml(self):
        el = ET.Element("weight_windows_generator")
        ET.SubElement(el, "mesh").text = str(self.mesh.id)
        if self.energy_bounds is not None:
            ET.SubElement(el, "energy_bounds").text = _fmt(self.energy_bounds)
        ET.SubElement(el, "particle_type").text = self.particle_type
        ET.SubElement(el, "max_realizations").text = str(self.max_realizations)
        ET.SubElement(el, "update_interval").text = str(self.update_interval)
        ET.SubElement(el, "on_the_fly").text = str(self.on_the_fly).lower()
        ET.SubElement(el, "method").text = self.method
        up = ET.SubElement(el, "update_parameters")
        for k, v in self.update_parameters.items():
            ET.SubElement(up, k).text = str(v)
        return el


# ---------------------------------------------------------------------------
# Settings and Model
# ---------------------------------------------------------------------------

class Settings:
    def __init__(self, **kw):
        self.run_mode = "fixed source"
        self.particles = 1000
        self.batches = 1
        self.inactive = 0
        self.generations_per_batch = None
        self.source = []
        self.event_based = False
        self.seed = None
        self.max_particles_in_flight = None
        self.log_grid_bins = None
        self.weight_windows = []
        self.weight_windows_on = None
        self.weight_window_generators = []
        self.max_history_splits = None
        self.energy_cutoff = None
        self.time_cutoff = None  # neutron time cutoff in s (the reference's cutoff['time_neutron'])
        self.survival_biasing = False
        self.max_lost_particles = None
        self.rel_max_lost_particles = None
        for k, v in kw.items():
            setattr(self, k, v)

    def mesh_ids(self):
        """Ids of the meshes the weight windows and generators refer to."""
        wws = self.weight_windows if isinstance(self.weight_windows, (list, tuple)) else [self.weight_windows]
        ids = {ww.mesh.id for ww in wws if ww is not None}
        return ids | {g.mesh.id for g in self.weight_window_generators}

    def to_xml(self, skip_mesh_ids=()):
        el = ET.Element("settings")
        ET.SubElement(el, "run_mode").text = self.run_mode
        ET.SubElement(el, "particles").text = str(int(self.particles))
        ET.SubElement(el, "batches").text = str(int(self.batches))
        if self.inactive:
            ET.SubElement(el, "inactive").text = str(int(self.inactive))
        if self.generations_per_batch is not None:
            ET.SubElement(el, "generations_per_batch").text = str(int(self.generations_per_batch))
        srcs = self.source if isinstance(self.source, (list, tuple)) else [self.source]
        for s in srcs:
            el.append(s.to_xml())
        if self.event_based:
            ET.SubElement(el, "event_based").text = "true"
        if self.seed is not None:
            ET.SubElement(el, "seed").text = str(int(self.seed))
        if self.max_particles_in_flight is not None:
            ET.SubElement(el, "max_particles_in_flight").text = str(int(self.max_particles_in_flight))
        if self.log_grid_bins is not None:
            ET.SubElement(el, "log_grid_bins").text = str(int(self.log_grid_bins))
        if self.max_history_splits is not None:
            ET.SubElement(el, "max_history_splits").text = str(int(self.max_history_splits))
        if self.survival_biasing:
            # written so that the library rejects it instead of running without it
            ET.SubElement(el, "survival_biasing").text = "true"
        if self.max_lost_particles is not None:
            ET.SubElement(el, "max_lost_particles").text = str(int(self.max_lost_particles))
        if self.rel_max_lost_particles is not None:
            ET.SubElement(el, "rel_max_lost_particles").text = repr(float(self.rel_max_lost_particles))
        if self.energy_cutoff is not None or self.time_cutoff is not None:
            co = ET.SubElement(el, "cutoff")
            if self.energy_cutoff is not None:
                ET.SubElement(co, "energy_neutron").text = repr(float(self.energy_cutoff))
            if self.time_cutoff is not None:
                ET.SubElement(co, "time_neutron").text = repr(float(self.time_cutoff))
        meshes = {}
        wws = self.weight_windows if isinstance(self.weight_windows, (list, tuple)) else [self.weight_windows]
        for ww in wws:
            if ww is not None:
                meshes[ww.mesh.id] = ww.mesh
        for g in self.weight_window_generators:
            meshes[g.mesh.id] = g.mesh
        for mid in sorted(meshes):
            if mid not in skip_mesh_ids:
                el.append(meshes[mid].to_xml())
        for ww in wws:
            if ww is not None:
                el.append(ww.to_xml())
        if self.weight_windows_on is not None:
            ET.SubElement(el, "weight_windows_on").text = str(bool(self.weight_windows_on)).lower()
        if self.weight_window_generators:
            ge = ET.SubElement(el, "weight_window_generators")
            for g in self.weight_window_generators:
                ge.append(g.to_xml())
        return el


class Model:
    def __init__(self, geometry=None, materials=None, settings=None, tallies=None):
        self.geometry = geometry
        self.materials = materials if materials is not None else Materials()
        self.settings = settings if settings is not None else Settings()
        self.tallies = tallies if tallies is not None else Tallies()

    def to_xml(self):
        root = ET.Element("model")
        root.append(self.materials.to_xml())
        root.append(self.geometry.to_xml())
        # each mesh is written once, in settings when weight windows use it
        # (settings are read first), else with the tallies
        # (openmc/model/model.py export_to_model_xml, mesh_memo)
        root.append(self.settings.to_xml())
        if self.tallies:
            root.append(self.tallies.to_xml(skip_mesh_ids=self.settings.mesh_ids()))
        return root

    def export_to_model_xml(self, path="model.xml"):
        path = Path(path)
        if path.is_dir() or path.suffix != ".xml":
            path = path / "model.xml"
        path.parent.mkdir(parents=True, exist_ok=True)
        root = self.to_xml()
        ET.indent(root)
        ET.ElementTree(root).write(path, xml_declaration=True, encoding="utf-8")
        return path

    def run(self, cwd=".", event_based=None, particles=None, threads=None,
            use_lib=True):
        """Run the model through the GB300 library (``openmc.lib`` path).

        Mirrors ``Model.run`` (``openmc/model/model.py:755-900``): exports the
        XML, initialises the library in ``cwd``, sets ``event_based`` when
        given, runs all batches and returns the path of the statepoint file
        written at the last batch (read it with
        :class:`openmc_gb300.statepoint.StatePoint`).
        """
        from . import lib
        cwd = Path(cwd)
        self.export_to_model_xml(cwd / "model.xml")
        args = []
        if particles is not None:
            args += ["-n", str(int(particles))]
        lib.init(args=args, directory=cwd)
        try:
            if event_based is not None:
                lib.settings.event_based = bool(event_based)
            lib.run()
            w = len(str(int(self.settings.batches)))
            return cwd / f"statepoint.{lib.current_batch():0{w}d}.h5"
        finally:
            lib.finalize()
