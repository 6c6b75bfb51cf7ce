"""Seeded synthetic continuous-energy nuclear data and its on-disk format.

OpenMC reads incident-neutron data from HDF5 files listed in a
``cross_sections.xml`` library (``openmc/data/library.py:101``,
``src/cross_sections.cpp:183-343``).  Each nuclide holds one energy grid per
temperature, the atomic weight ratio, ``kTs`` and one group per reaction with
its ``threshold_idx`` and ``xs`` values (``docs/source/io_formats/
nuclear_data.rst:16-64``).  Neither libhdf5 nor h5py exists on the machines
this package runs on: ``write_nuclide_h5`` writes that HDF5 layout with the
package's own writer (``openmc_gb300.h5``), and the same content can also be
stored in a small native binary container with the same fields (the library
reads either; the file's first bytes decide):

====================  ==========================================
field                 meaning
====================  ==========================================
magic ``OMCGBNUC``    8 bytes
version               uint32 (=1)
name                  uint32 length + UTF-8 bytes
A, awr, kT            3 x float64 (kT in eV, one temperature)
n_points              uint32
n_reactions           uint32
energy                float64[n_points] (eV, ascending)
per reaction          uint32 MT, uint32 threshold_idx, uint32 n,
                      float64[n] cross section (barns)
fission (version 2)   uint32 flag; if 1: float64[2] nu polynomial
                      coefficients (increasing powers of E, the total
                      yield of the MT 18 neutron product), uint32
                      spectrum type (1 Maxwell, 2 Watt), float64[2]
                      parameters (theta, 0 or a, b; eV, 1/eV), float64
                      restriction energy U (eV); prompt neutrons only,
                      isotropic emission
====================  ==========================================

Version 1 files (no fission block) are still read.

The generator follows the recipe of the synthetic nuclides this project is
benchmarked on: a log-uniform grid between 1e-5 eV and 20 MeV with a seeded
+-5 % jitter of the interior points, an elastic cross section made of a
constant plus 20 Breit-Wigner peaks, and a capture (MT 102) cross section made
of a 1/v term plus the same peaks scaled by a seeded branching ratio.  This
mirrors the way ``tests/unit_tests/test_temp_interp.py:12-140`` of the
reference builds a fake nuclide (MT 2 + MT 102 on one grid).
"""
from __future__ import annotations

import struct
from dataclasses import dataclass, field
from pathlib import Path
from xml.etree import ElementTree as ET

import numpy as np

MAGIC = b"OMCGBNUC"
VERSION = 2
K_BOLTZMANN = 8.617333262e-5  # eV/K, include/openmc/constants.h:100
E_MIN = 1.0e-5
E_MAX = 2.0e7
MT_ELASTIC = 2
MT_FISSION = 18
MT_CAPTURE = 102
SPECTRUM_MAXWELL = 1
SPECTRUM_WATT = 2


@dataclass
class Fission:
    """Prompt fission neutrons of MT 18: yield nu(E) = nu[0] + nu[1] E
    (Polynomial, src/endf.cpp:125-134), energy from a Maxwell (theta) or
    Watt (a, b) spectrum with restriction energy U
    (src/distribution_energy.cpp:282-360), isotropic emission."""
    nu: tuple = (2.43, 0.0)
    spectrum: int = SPECTRUM_WATT
    params: tuple = (0.988e6, 2.249e-6)
    u: float = -2.0e7


@dataclass
class Nuclide:
    """One synthetic nuclide at one temperature (MT 2 and MT 102, and MT 18
    with its fission neutron data for a fissile nuclide)."""
    name: str
    A: float
    awr: float
    kT: float
    energy: np.ndarray
    reactions: dict = field(default_factory=dict)  # mt -> (threshold_idx, xs)
    fission: Fission | None = None

    @property
    def elastic(self) -> np.ndarray:
        return self.reactions[MT_ELASTIC][1]

    @property
    def capture(self) -> np.ndarray:
        return self.reactions[MT_CAPTURE][1]


def awr_of(A: float) -> float:
    """Atomic weight ratio of a synthetic nuclide of mass number A.

    Uses the A=1 value of hydrogen (0.999167) scaled linearly, so that the
    A=1 nuclide has awr <= 1 and is always treated with the free-gas model
    (``src/physics.cpp:857``).
    """
    return 0.99916733 * A


def log_grid(n_points: int, rng: np.random.Generator,
             e_min: float = E_MIN, e_max: float = E_MAX,
             jitter: float = 0.05) -> np.ndarray:
    """Log-uniform grid with a seeded +-5 % jitter of each interior point's
    lethargy, measured in units of the grid spacing; endpoints fixed.

    Jittering by a fraction of the spacing keeps the points in order and at
    least 0.9 spacings apart (a jitter of 5 % of the energy itself exceeds
    the 1.5 % spacing of a 2,000-point grid, reorders points and piles them
    up against the endpoints)."""
    u = np.linspace(np.log(e_min), np.log(e_max), n_points)
    du = u[1] - u[0]
    u[1:-1] += jitter * du * (2.0 * rng.random(n_points - 2) - 1.0)
    e = np.exp(u)
    e[0], e[-1] = e_min, e_max
    return e


# Base values (barns) by class of nuclide: (potential scattering, thermal
# capture at 0.0253 eV, peak height scale, branching range).
_CLASSES = {
    "light": (20.0, 0.33, 30.0, (0.01, 0.05)),
    "moderator": (4.5, 0.003, 20.0, (0.01, 0.05)),
    "structural": (11.0, 2.5, 400.0, (0.05, 0.5)),
    "absorber": (10.0, 30.0, 3000.0, (0.3, 0.95)),
}


def nuclide_class(A: float) -> str:
    if A <= 2:
        return "light"
    if A <= 20:
        return "moderator"
    if A <= 100:
        return "structural"
    return "absorber"


def make_nuclide(name: str, A: float, n_points: int, seed: int,
                 kind: str | None = None, n_peaks: int = 20,
                 temperature: float = 294.0, fissile: bool = False) -> Nuclide:
    """Build one synthetic nuclide from a seed (deterministic).  fissile adds
    MT 18: a 1/v fission cross section (585 b at 0.0253 eV) plus the
    resonance peaks times a seeded fission branching, with the default
    Fission yield and Watt spectrum."""
    rng = np.random.default_rng(seed)
    kind = kind or nuclide_class(A)
    pot, cap_th, height, (b_lo, b_hi) = _CLASSES[kind]
    E = log_grid(n_points, rng)
    # Breit-Wigner peaks in the resolved range, seeded.
    E0 = np.exp(rng.uniform(np.log(1.0), np.log(1.0e5), n_peaks))
    gamma = E0 * 10.0 ** rng.uniform(-3.0, -1.0, n_peaks)
    h = height * 10.0 ** rng.uniform(-1.0, 0.0, n_peaks)
    branch = rng.uniform(b_lo, b_hi, n_peaks)
    half = 0.5 * gamma
    shape = (half[None, :] ** 2) / ((E[:, None] - E0[None, :]) ** 2 + half[None, :] ** 2)
    peaks_el = shape @ h
    peaks_cap = shape @ (h * branch)
    elastic = pot * (1.0 + 0.02 * rng.standard_normal()) + peaks_el
    capture = cap_th * np.sqrt(0.0253 / E) + peaks_cap
    nuc = Nuclide(name=name, A=float(A), awr=awr_of(A),
                  kT=K_BOLTZMANN * temperature, energy=E)
    nuc.reactions[MT_ELASTIC] = (0, np.ascontiguousarray(elastic, dtype=np.float64))
    nuc.reactions[MT_CAPTURE] = (0, np.ascontiguousarray(capture, dtype=np.float64))
    if fissile:
        frac = rng.uniform(0.5, 2.0, n_peaks)
        fis = 585.0 * np.sqrt(0.0253 / E) + shape @ (h * frac) + 1.0
        nuc.reactions[MT_FISSION] = (0, np.ascontiguousarray(fis, dtype=np.float64))
        nuc.fission = Fission()
    return nuc


def make_flat_nuclide(name: str, A: float, n_points: int, seed: int, elastic: float, capture: float,
                      fission: float = 0.0, nu: float = 2.43, temperature: float = 294.0) -> Nuclide:
    """A nuclide whose cross sections do not depend on energy (on a seeded
    log grid): in an infinite homogeneous medium of such nuclides k-infinity
    is nu Sigma_f / Sigma_a exactly, the known answer the reference's
    tests/unit_tests/test_temp_interp.py builds the same way."""
    rng = np.random.default_rng(seed)
    E = log_grid(n_points, rng)
    nuc = Nuclide(name=name, A=float(A), awr=awr_of(A), kT=K_BOLTZMANN * temperature, energy=E)
    nuc.reactions[MT_ELASTIC] = (0, np.full(n_points, float(elastic)))
    nuc.reactions[MT_CAPTURE] = (0, np.full(n_points, float(capture)))
    if fission > 0.0:
        nuc.reactions[MT_FISSION] = (0, np.full(n_points, float(fission)))
        nuc.fission = Fission(nu=(float(nu), 0.0))
    return nuc


def write_nuclide(nuc: Nuclide, path: str | Path) -> None:
    path = Path(path)
    name = nuc.name.encode()
    with open(path, "wb") as f:
        f.write(MAGIC)
        f.write(struct.pack("<I", VERSION))
        f.write(struct.pack("<I", len(name)))
        f.write(name)
        f.write(struct.pack("<3d", nuc.A, nuc.awr, nuc.kT))
        f.write(struct.pack("<II", len(nuc.energy), len(nuc.reactions)))
        f.write(np.ascontiguousarray(nuc.energy, dtype="<f8").tobytes())
        for mt in sorted(nuc.reactions):
            thr, xs = nuc.reactions[mt]
            f.write(struct.pack("<III", mt, thr, len(xs)))
            f.write(np.ascontiguousarray(xs, dtype="<f8").tobytes())
        fis = nuc.fission
        f.write(struct.pack("<I", 1 if fis is not None else 0))
        if fis is not None:
            f.write(struct.pack("<2d", *fis.nu))
            f.write(struct.pack("<I", fis.spectrum))
            f.write(struct.pack("<3d", *fis.params, fis.u))


def write_nuclide_h5(nuc: Nuclide, path: str | Path) -> None:
    """Write a nuclide in OpenMC's incident-neutron HDF5 layout
    (docs/source/io_formats/nuclear_data.rst; what
    openmc.data.IncidentNeutron.export_to_hdf5 writes): the energy grid and
    kT under the temperature's name, one group per reaction with its
    cross section and threshold index, the elastic product (isotropic in the
    centre of mass), and for MT 18 the prompt neutron product with its
    Polynomial yield and an uncorrelated Maxwell or Watt energy
    distribution whose parameters are constant Tabulated1D functions."""
    from . import h5
    T = f"{int(round(nuc.kT / K_BOLTZMANN))}K"
    e_lo, e_hi = float(nuc.energy[0]), float(nuc.energy[-1])

    def const(v):
        return h5.Dataset(np.array([[e_lo, e_hi], [v, v]]),
                          {"type": np.bytes_(b"Tabulated1D"), "breakpoints": np.array([2], np.int32),
                           "interpolation": np.array([2], np.int32)})

    labels = {MT_ELASTIC: "(n,elastic)", MT_FISSION: "(n,fission)", MT_CAPTURE: "(n,gamma)"}
    reactions = h5.Node()
    for mt in sorted(nuc.reactions):
        thr, xs = nuc.reactions[mt]
        rx = h5.Node({T: h5.Node({"xs": h5.Dataset(np.asarray(xs, np.float64),
                                                   {"threshold_idx": np.int32(thr)})})},
                     {"mt": np.int32(mt), "label": np.bytes_(labels.get(mt, f"MT {mt}").encode()),
                      "Q_value": 0.0, "center_of_mass": np.int32(1 if mt == MT_ELASTIC else 0),
                      "redundant": np.int32(0)})
        n_product = 0
        if mt == MT_ELASTIC:
            rx["product_0"] = h5.Node({"yield": h5.Dataset(np.array([1.0]), {"type": np.bytes_(b"Polynomial")}),
                                       "distribution_0": h5.Node({}, {"type": np.bytes_(b"uncorrelated")})},
                                      {"particle": np.bytes_(b"neutron"), "emission_mode": np.bytes_(b"prompt"),
                                       "decay_rate": 0.0, "n_distribution": np.int32(1)})
            n_product = 1
        elif mt == MT_FISSION and nuc.fission is not None:
            f = nuc.fission
            if f.spectrum == SPECTRUM_MAXWELL:
                energy = h5.Node({"theta": const(f.params[0])}, {"type": np.bytes_(b"maxwell"), "u": f.u})
            else:
                energy = h5.Node({"a": const(f.params[0]), "b": const(f.params[1])},
                                 {"type": np.bytes_(b"watt"), "u": f.u})
            rx["product_0"] = h5.Node(
                {"yield": h5.Dataset(np.array(f.nu, np.float64), {"type": np.bytes_(b"Polynomial")}),
                 "distribution_0": h5.Node({"energy": energy}, {"type": np.bytes_(b"uncorrelated")})},
                {"particle": np.bytes_(b"neutron"), "emission_mode": np.bytes_(b"prompt"), "decay_rate": 0.0,
                 "n_distribution": np.int32(1)})
            n_product = 1
        rx.attrs["n_product"] = np.int32(n_product)
        reactions[f"reaction_{mt:03d}"] = rx
    group = h5.Node({"energy": h5.Node({T: np.asarray(nuc.energy, np.float64)}),
                     "kTs": h5.Node({T: np.float64(nuc.kT)}),
                     "reactions": reactions},
                    {"Z": np.int32(0), "A": np.int32(int(round(nuc.A))), "metastable": np.int32(0),
                     "atomic_weight_ratio": float(nuc.awr), "n_reaction": np.int32(len(nuc.reactions))})
    root = h5.Node({nuc.name: group}, {"filetype": np.bytes_(b"data_neutron"),
                                       "version": np.array([3, 0], np.int32)})
    h5.write(path, root)


def read_nuclide(path: str | Path) -> Nuclide:
    buf = Path(path).read_bytes()
    if buf[:8] != MAGIC:
        raise ValueError(f"{path}: not a nuclide file")
    off = 8
    (version,) = struct.unpack_from("<I", buf, off); off += 4
    if version not in (1, 2):
        raise ValueError(f"{path}: unsupported version {version}")
    (nlen,) = struct.unpack_from("<I", buf, off); off += 4
    name = buf[off:off + nlen].decode(); off += nlen
    A, awr, kT = struct.unpack_from("<3d", buf, off); off += 24
    n, nrx = struct.unpack_from("<II", buf, off); off += 8
    energy = np.frombuffer(buf, "<f8", n, off).copy(); off += 8 * n
    nuc = Nuclide(name=name, A=A, awr=awr, kT=kT, energy=energy)
    for _ in range(nrx):
        mt, thr, m = struct.unpack_from("<III", buf, off); off += 12
        xs = np.frombuffer(buf, "<f8", m, off).copy(); off += 8 * m
        nuc.reactions[mt] = (thr, xs)
    if version >= 2:
        (flag,) = struct.unpack_from("<I", buf, off); off += 4
        if flag:
            nu = struct.unpack_from("<2d", buf, off); off += 16
            (spec,) = struct.unpack_from("<I", buf, off); off += 4
            a, b, u = struct.unpack_from("<3d", buf, off); off += 24
            nuc.fission = Fission(nu=tuple(nu), spectrum=spec, params=(a, b), u=u)
    return nuc


def write_library(nuclides, directory: str | Path, fmt: str = "native") -> Path:
    """Write nuclide files plus a ``cross_sections.xml`` (OpenMC schema);
    fmt "h5" writes OpenMC's HDF5 layout (write_nuclide_h5) instead of the
    native container."""
    directory = Path(directory)
    directory.mkdir(parents=True, exist_ok=True)
    root = ET.Element("cross_sections")
    for nuc in nuclides:
        fname = f"{nuc.name}.h5" if fmt == "h5" else f"{nuc.name}.nuc"
        if fmt == "h5":
            write_nuclide_h5(nuc, directory / fname)
        else:
            write_nuclide(nuc, directory / fname)
        ET.SubElement(root, "library", materials=nuc.name, path=fname,
                      type="neutron")
    ET.indent(root)
    out = directory / "cross_sections.xml"
    ET.ElementTree(root).write(out, xml_declaration=True, encoding="utf-8")
    return out


def read_library(xml_path: str | Path) -> dict:
    """Map nuclide name -> file path from a cross_sections.xml."""
    xml_path = Path(xml_path)
    root = ET.parse(xml_path).getroot()
    out = {}
    for lib in root.iter("library"):
        if lib.get("type", "neutron") != "neutron":
            continue
        p = Path(lib.get("path"))
        if not p.is_absolute():
            p = xml_path.parent / p
        for m in lib.get("materials").split():
            out[m] = p
    return out


# ---------------------------------------------------------------------------
# Macroscopic cross-section lookup microbenchmark data (XSBench-shaped)
# ---------------------------------------------------------------------------

@dataclass
class XSBenchData:
    """Flat tables for the lookup microbenchmark.

    energy:   float64 [n_nuc, G]
    xs:       float64 [n_nuc, G, 5] channels (total, elastic, absorption,
              aux1, aux2)
    mat_nuc:  int32 concatenated nuclide indices per material
    mat_off:  int32 [n_mat+1] offsets into mat_nuc
    mat_dens: float64 atom densities aligned with mat_nuc
    mat_prob: float64 [n_mat] material sampling probabilities
    """
    energy: np.ndarray
    xs: np.ndarray
    mat_nuc: np.ndarray
    mat_off: np.ndarray
    mat_dens: np.ndarray
    mat_prob: np.ndarray


XSBENCH_MAT_COUNTS = (321, 5, 4, 4, 27, 21, 21, 21, 21, 21, 9, 9)
# Probabilities with which the 12 materials are drawn before seeding noise
# (fuel-dominated, as in a light-water reactor lookup mix).
_XSBENCH_MAT_WEIGHTS = (0.140, 0.052, 0.275, 0.134, 0.154, 0.064, 0.066,
                        0.055, 0.008, 0.015, 0.025, 0.013)


def make_xsbench(n_nuc: int = 68, n_points: int = 11303, seed: int = 42,
                 mat_counts=XSBENCH_MAT_COUNTS) -> XSBenchData:
    """68 nuclides x 11,303 points x 5 channels, 12 materials, all seeded.

    Material 0 has 321 entries drawn with replacement from the 68 nuclides
    (the standalone microbenchmark sums duplicates like distinct entries).
    """
    rng = np.random.default_rng(seed)
    energy = np.empty((n_nuc, n_points))
    xs = np.empty((n_nuc, n_points, 5))
    for i in range(n_nuc):
        sub = np.random.default_rng(rng.integers(1 << 62))
        A = float(sub.integers(1, 240))
        nuc = make_nuclide(f"X{i:03d}", A, n_points, int(sub.integers(1 << 62)))
        energy[i] = nuc.energy
        el, cap = nuc.elastic, nuc.capture
        aux1 = sub.uniform(0.1, 2.0) * el
        aux2 = sub.uniform(0.0, 1.0) * cap + sub.uniform(0.0, 1.0)
        xs[i, :, 0] = el + cap
        xs[i, :, 1] = el
        xs[i, :, 2] = cap
        xs[i, :, 3] = aux1
        xs[i, :, 4] = aux2
    mat_nuc, mat_off, mat_dens = [], [0], []
    for m, cnt in enumerate(mat_counts):
        if m == 0:
            idx = rng.integers(0, n_nuc, cnt)
        else:
            idx = rng.choice(n_nuc, cnt, replace=False)
        mat_nuc.extend(int(v) for v in idx)
        mat_dens.extend(rng.uniform(1e-5, 5e-2, cnt))
        mat_off.append(len(mat_nuc))
    base = np.resize(np.asarray(_XSBENCH_MAT_WEIGHTS), len(mat_counts))
    w = base * rng.uniform(0.9, 1.1, len(mat_counts))
    return XSBenchData(energy=energy, xs=xs,
                       mat_nuc=np.asarray(mat_nuc, np.int32),
                       mat_off=np.asarray(mat_off, np.int32),
                       mat_dens=np.asarray(mat_dens, np.float64),
                       mat_prob=w / w.sum())


def xsbench_lookups(data: XSBenchData, n: int, seed: int = 7):
    """Seeded (material, energy) pairs; energies log-uniform over the grid range."""
    rng = np.random.default_rng(seed)
    mats = rng.choice(len(data.mat_prob), size=n, p=data.mat_prob).astype(np.int32)
    e = np.exp(rng.uniform(np.log(E_MIN), np.log(E_MAX), n))
    return mats, e
