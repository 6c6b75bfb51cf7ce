"""ctypes bindings to ``libopenmc_gb300.so`` mirroring ``openmc.lib``.

The reference's ``openmc.lib`` (``openmc/lib/core.py``, ``tally.py``,
``weight_windows.py``, ``settings.py``, ``error.py``) loads ``libopenmc.so``
with ``CDLL``, declares argtypes/restype per C function, maps negative return
codes to exception classes through ``openmc_err_msg``, and exposes settings as
``_DLLGlobal`` descriptors over exported C globals.  This module does the same
for the GB300 library; the function names and argument meanings follow the
reference so that code written against ``openmc.lib`` runs unchanged for the
event-based fixed-source path.

The library is required: importing this module raises if the CUDA library is
missing or cannot be loaded (there is no CPU fallback).
"""
from __future__ import annotations

import ctypes as C
import os
import warnings
from contextlib import contextmanager
from pathlib import Path

import numpy as np

from . import build as _build

_LIB = _build.LIB
if not _LIB.exists():
    raise ImportError(
        f"{_LIB} is missing: build it with `python -m openmc_gb300.build` "
        "(nvcc, sm_103a); the GB300 library has no CPU fallback")
_dll = C.CDLL(str(_LIB))


# ------------------------------------------------------------- exceptions
class OpenMCError(Exception):
    """Root exception (openmc/exceptions.py)."""


class AllocationError(OpenMCError):
    pass


class OutOfBoundsError(OpenMCError):
    pass


class InvalidArgumentError(OpenMCError):
    pass


class InvalidTypeError(OpenMCError):
    pass


class InvalidIDError(OpenMCError):
    pass


class GeometryError(OpenMCError):
    pass


class DataError(OpenMCError):
    pass


class PhysicsError(OpenMCError):
    pass


# Exported error-code globals of the C API and the exception each one raises
# (the reference's openmc.lib maps the same codes to the same exception
# names; OPENMC_E_WARNING becomes a Python warning instead).
_ERROR_CLASSES = {
    "OPENMC_E_ALLOCATE": AllocationError,
    "OPENMC_E_OUT_OF_BOUNDS": OutOfBoundsError,
    "OPENMC_E_INVALID_ARGUMENT": InvalidArgumentError,
    "OPENMC_E_INVALID_TYPE": InvalidTypeError,
    "OPENMC_E_INVALID_ID": InvalidIDError,
    "OPENMC_E_GEOMETRY": GeometryError,
    "OPENMC_E_DATA": DataError,
    "OPENMC_E_PHYSICS": PhysicsError,
}
_code_to_class = None


def _error_handler(err, func, args):
    """ctypes errcheck: 0 passes through; OPENMC_E_WARNING (a positive code)
    issues a warning; a negative code raises the exception its exported
    OPENMC_E_* global names, with the library's openmc_err_msg as the
    message."""
    global _code_to_class
    if err == 0:
        return err
    msg = (C.c_char * 256).in_dll(_dll, "openmc_err_msg").value.decode()
    if err == C.c_int.in_dll(_dll, "OPENMC_E_WARNING").value:
        warnings.warn(msg)
        return err
    if err > 0:
        return err
    if _code_to_class is None:
        _code_to_class = {C.c_int.in_dll(_dll, name).value: cls for name, cls in _ERROR_CLASSES.items()}
    cls = _code_to_class.get(err, OpenMCError)
    raise cls(msg or f"error code {err} from {getattr(func, '__name__', 'the library')}")


def _fn(name, argtypes, restype=C.c_int, check=True):
    f = getattr(_dll, name)
    f.argtypes = argtypes
    f.restype = restype
    if check and restype is C.c_int:
        f.errcheck = _error_handler
    return f


_p = C.POINTER
_fn("openmc_init", [C.c_int, _p(C.c_char_p), C.c_void_p])
_fn("openmc_run", [])
_fn("openmc_simulation_init", [])
_fn("openmc_simulation_finalize", [])
_fn("openmc_next_batch", [_p(C.c_int)])
_fn("openmc_finalize", [])
_fn("openmc_reset", [])
_fn("openmc_hard_reset", [])
_fn("openmc_reset_timers", [])
_fn("openmc_statepoint_write", [C.c_char_p, _p(C.c_bool)])
_fn("openmc_get_seed", [], C.c_int64)
_fn("openmc_set_seed", [C.c_int64], None)
_fn("openmc_get_stride", [], C.c_uint64)
_fn("openmc_set_stride", [C.c_uint64], None)
_fn("openmc_tally_results", [C.c_int32, _p(_p(C.c_double)), _p(C.c_size_t)])
_fn("openmc_get_tally_index", [C.c_int32, _p(C.c_int32)])
_fn("openmc_tally_get_id", [C.c_int32, _p(C.c_int32)])
_fn("openmc_tally_get_n_realizations", [C.c_int32, _p(C.c_int32)])
_fn("openmc_global_tallies", [_p(_p(C.c_double))])
_fn("tallies_size", [], C.c_size_t)
_fn("openmc_weight_windows_size", [], C.c_size_t)
_fn("openmc_get_weight_windows_index", [C.c_int32, _p(C.c_int32)])
_fn("openmc_weight_windows_get_id", [C.c_int32, _p(C.c_int32)])
_fn("openmc_weight_windows_get_bounds", [C.c_int32, _p(_p(C.c_double)), _p(_p(C.c_double)), _p(C.c_size_t)])
_fn("openmc_weight_windows_set_bounds", [C.c_int32, _p(C.c_double), _p(C.c_double), C.c_size_t])
_fn("openmc_weight_windows_get_energy_bounds", [C.c_int32, _p(_p(C.c_double)), _p(C.c_size_t)])
_fn("openmc_weight_windows_update_magic", [C.c_int32, C.c_int32, C.c_char_p, C.c_double, C.c_double])
_fn("openmc_weight_windows_get_mesh", [C.c_int32, _p(C.c_int32)])
_fn("openmc_gb300_last_batch", [_p(C.c_double)])
_fn("openmc_gb300_timing", [_p(C.c_double)])
_fn("openmc_gb300_last_batch_detail", [_p(C.c_double)])
_fn("openmc_gb300_set_trace", [C.c_int64, C.c_int])
_fn("openmc_gb300_get_trace", [C.c_void_p, _p(C.c_int32)])
_fn("openmc_gb300_set_weight_windows_on", [C.c_int])
_fn("openmc_gb300_model_info", [_p(C.c_int64)])
_fn("openmc_gb300_material_xs", [C.c_int64, _p(C.c_int32), _p(C.c_double), _p(C.c_double), _p(C.c_double),
                                 _p(C.c_uint32)])
_fn("openmc_gb300_xs_tables_create", [C.c_int, C.c_int, _p(C.c_double), _p(C.c_double), C.c_int,
                                      _p(C.c_int32), _p(C.c_int32), _p(C.c_double), C.c_int, C.c_int,
                                      C.c_int64, _p(C.c_void_p)])
_fn("openmc_gb300_xs_tables_free", [C.c_void_p])
_fn("openmc_gb300_xs_lookup", [C.c_void_p, C.c_int64, _p(C.c_int32), _p(C.c_double), _p(C.c_double),
                               _p(C.c_int32), C.c_int])
_fn("openmc_gb300_xs_lookup_device", [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                                      C.c_void_p, C.c_int])
_fn("openmc_gb300_xs_last_times", [C.c_void_p, _p(C.c_float)])
_fn("openmc_gb300_xs_stream", [C.c_void_p, _p(C.c_void_p)])
_fn("openmc_gb300_xs_lookup_noalloc", [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.c_void_p, C.c_void_p])
_fn("openmc_gb300_mlp_n_params", [], C.c_int, check=False)
_fn("openmc_gb300_mlp_create", [C.c_int64, C.c_uint64, _p(C.c_void_p)])
_fn("openmc_gb300_mlp_free", [C.c_void_p])
_fn("openmc_gb300_mlp_set_data", [C.c_void_p, C.c_int64, _p(C.c_float), _p(C.c_float), _p(C.c_float)])
_fn("openmc_gb300_mlp_train", [C.c_void_p, C.c_int, C.c_double, _p(C.c_float)])
_fn("openmc_gb300_mlp_gradients", [C.c_void_p, _p(C.c_float), _p(C.c_float)])
_fn("openmc_gb300_mlp_predict", [C.c_void_p, C.c_int64, _p(C.c_float), _p(C.c_float)])
_fn("openmc_gb300_mlp_get_params", [C.c_void_p, _p(C.c_float), C.c_int64])
_fn("openmc_gb300_mlp_set_params", [C.c_void_p, _p(C.c_float), C.c_int64])
_fn("openmc_gb300_mlp_last_ms", [C.c_void_p, _p(C.c_float)])


# ------------------------------------------------------------- globals
class _DLLGlobal:
    """Data descriptor over an exported C global (openmc/lib/core.py:724-735)."""

    def __init__(self, ctype, name):
        self.ctype, self.name = ctype, name

    def __get__(self, instance, owner):
        return self.ctype.in_dll(_dll, self.name).value

    def __set__(self, instance, value):
        self.ctype.in_dll(_dll, self.name).value = value


class _Settings:
    """openmc.lib.settings subset (openmc/lib/settings.py:27-44)."""
    event_based = _DLLGlobal(C.c_bool, "event_based")
    particles = _DLLGlobal(C.c_int64, "n_particles")
    inactive = _DLLGlobal(C.c_int32, "n_inactive")
    generations_per_batch = _DLLGlobal(C.c_int32, "gen_per_batch")
    max_lost_particles = _DLLGlobal(C.c_int32, "max_lost_particles")
    rel_max_lost_particles = _DLLGlobal(C.c_double, "rel_max_lost_particles")
    run_CE = _DLLGlobal(C.c_bool, "run_CE")
    verbosity = _DLLGlobal(C.c_int, "verbosity")
    weight_windows_on = _DLLGlobal(C.c_bool, "weight_windows_on")
    restart_run = _DLLGlobal(C.c_bool, "restart_run")
    # GB300 extensions
    xs_fp32 = _DLLGlobal(C.c_int, "openmc_gb300_xs_fp32")
    particles_in_flight = _DLLGlobal(C.c_int64, "openmc_gb300_in_flight")
    sort_queue = _DLLGlobal(C.c_int, "openmc_gb300_sort")
    fuse_xs = _DLLGlobal(C.c_int, "openmc_gb300_fuse")
    trace_batch = _DLLGlobal(C.c_int, "openmc_gb300_trace_batch")
    trace_first = _DLLGlobal(C.c_int64, "openmc_gb300_trace_first")
    profile_next = _DLLGlobal(C.c_int, "openmc_gb300_profile_next")
    tail_threshold = _DLLGlobal(C.c_int64, "openmc_gb300_tail_threshold")
    secondary_capacity = _DLLGlobal(C.c_int64, "openmc_gb300_secondary_capacity")
    split_to_slots = _DLLGlobal(C.c_int, "openmc_gb300_split_to_slots")
    max_levels = _DLLGlobal(C.c_int, "openmc_gb300_max_levels")
    stage_tables = _DLLGlobal(C.c_int, "openmc_gb300_stage_tables")
    contract = _DLLGlobal(C.c_int, "openmc_gb300_contract")
    defer_tally = _DLLGlobal(C.c_int, "openmc_gb300_defer_tally")
    mlp_fused = _DLLGlobal(C.c_int, "openmc_gb300_mlp_fused")

    @property
    def seed(self):
        return _dll.openmc_get_seed()

    @seed.setter
    def seed(self, v):
        _dll.openmc_set_seed(int(v))

    @property
    def stride(self):
        return _dll.openmc_get_stride()

    @stride.setter
    def stride(self, v):
        _dll.openmc_set_stride(int(v))


settings = _Settings()


def current_batch():
    return C.c_int.in_dll(_dll, "current_batch").value


def is_initialized():
    return C.c_bool.in_dll(_dll, "initialized").value


# ------------------------------------------------------------- lifecycle
def init(args=None, intracomm=None, output=True, directory=None):
    """Initialise from the model in ``directory`` (or the working directory)."""
    argv = ["openmc"] + [str(a) for a in (args or [])]
    if directory is not None:
        argv.append(str(directory))
    arr = (C.c_char_p * len(argv))(*[a.encode() for a in argv])
    _dll.openmc_init(len(argv), arr, None)


def finalize():
    _dll.openmc_finalize()


def run(output=True):
    _dll.openmc_run()


def simulation_init():
    _dll.openmc_simulation_init()


def simulation_finalize():
    _dll.openmc_simulation_finalize()


def next_batch():
    status = C.c_int()
    _dll.openmc_next_batch(C.byref(status))
    return status.value


def reset():
    _dll.openmc_reset()


def hard_reset():
    _dll.openmc_hard_reset()


@contextmanager
def run_in_memory(**kwargs):
    init(**kwargs)
    try:
        yield
    finally:
        finalize()


# ------------------------------------------------------------- tallies
def tally_index(tally_id):
    idx = C.c_int32()
    _dll.openmc_get_tally_index(int(tally_id), C.byref(idx))
    return idx.value


def tally_results(tally_id):
    """Borrowed view of the results array [bins, scores, 3] (VALUE, SUM, SUM_SQ)."""
    ptr = _p(C.c_double)()
    shape = (C.c_size_t * 3)()
    _dll.openmc_tally_results(tally_index(tally_id), C.byref(ptr), shape)
    n = shape[0] * shape[1] * shape[2]
    return np.ctypeslib.as_array(ptr, shape=(n,)).reshape(shape[0], shape[1], shape[2])


def tally_ids():
    """Ids of all tallies in library order (openmc/lib/tally.py:440-460)."""
    out = []
    for k in range(_dll.tallies_size()):
        v = C.c_int32()
        _dll.openmc_tally_get_id(k, C.byref(v))
        out.append(v.value)
    return out


def tally_n_realizations(tally_id):
    n = C.c_int32()
    _dll.openmc_tally_get_n_realizations(tally_index(tally_id), C.byref(n))
    return n.value


def tally_mean_std(tally_id):
    """Mean and standard deviation of the mean (openmc/tallies.py:528-566)."""
    r = tally_results(tally_id)
    n = tally_n_realizations(tally_id)
    s, s2 = r[..., 1], r[..., 2]
    mean = s / n
    if n > 1:
        std = np.sqrt(np.maximum(s2 / n - mean * mean, 0.0) / (n - 1))
    else:
        std = np.zeros_like(mean)
    return mean, std


def global_tallies():
    ptr = _p(C.c_double)()
    _dll.openmc_global_tallies(C.byref(ptr))
    return np.ctypeslib.as_array(ptr, shape=(12,)).reshape(4, 3).copy()


# --------------------------------------------------------- weight windows
# ---- read-only model views (openmc/lib/cell.py, material.py, mesh.py,
# core.py): objects addressed by index, mappings keyed by id
_fn("openmc_get_cell_index", [C.c_int32, _p(C.c_int32)])
_fn("openmc_cell_get_id", [C.c_int32, _p(C.c_int32)])
_fn("openmc_cell_get_fill", [C.c_int32, _p(C.c_int), _p(_p(C.c_int32)), _p(C.c_int32)])
_fn("openmc_cell_get_num_instances", [C.c_int32, _p(C.c_int32)])
_fn("openmc_cell_get_translation", [C.c_int32, _p(C.c_double)])
_fn("openmc_cell_bounding_box", [C.c_int32, _p(C.c_double), _p(C.c_double)])
_fn("openmc_global_bounding_box", [_p(C.c_double), _p(C.c_double)])
_fn("openmc_get_material_index", [C.c_int32, _p(C.c_int32)])
_fn("openmc_material_get_id", [C.c_int32, _p(C.c_int32)])
_fn("openmc_material_get_densities", [C.c_int32, _p(_p(C.c_int)), _p(_p(C.c_double)), _p(C.c_int)])
_fn("openmc_material_get_density", [C.c_int32, _p(C.c_double)])
_fn("openmc_nuclide_name", [C.c_int, _p(C.c_char_p)])
_fn("openmc_get_mesh_index", [C.c_int32, _p(C.c_int32)])
_fn("openmc_mesh_get_id", [C.c_int32, _p(C.c_int32)])
_fn("openmc_regular_mesh_get_dimension", [C.c_int32, _p(_p(C.c_int)), _p(C.c_int)])
_fn("openmc_regular_mesh_get_params", [C.c_int32, _p(_p(C.c_double)), _p(_p(C.c_double)),
                                       _p(_p(C.c_double)), _p(C.c_int)])
_fn("openmc_get_keff", [_p(C.c_double)])
_fn("openmc_gb300_k_generation", [_p(C.c_double), C.c_int, _p(C.c_int64)], check=False)

FILL_TYPES = {0: "material", 1: "universe", 2: "lattice"}


class Cell:
    """A cell of the loaded model (openmc/lib/cell.py Cell, read-only)."""

    def __init__(self, index):
        self._index = int(index)

    @property
    def id(self):
        v = C.c_int32()
        _dll.openmc_cell_get_id(self._index, v)
        return v.value

    @property
    def fill(self):
        """(type name, index of the material, universe or lattice)."""
        t, idx, n = C.c_int(), _p(C.c_int32)(), C.c_int32()
        _dll.openmc_cell_get_fill(self._index, t, idx, n)
        return FILL_TYPES[t.value], idx[0]

    @property
    def num_instances(self):
        v = C.c_int32()
        _dll.openmc_cell_get_num_instances(self._index, v)
        return v.value

    @property
    def translation(self):
        xyz = (C.c_double * 3)()
        _dll.openmc_cell_get_translation(self._index, xyz)
        return np.array(xyz)

    @property
    def bounding_box(self):
        lo, hi = (C.c_double * 3)(), (C.c_double * 3)()
        _dll.openmc_cell_bounding_box(self._index, lo, hi)
        return np.array(lo), np.array(hi)


class Material:
    """A material of the loaded model (openmc/lib/material.py, read-only)."""

    def __init__(self, index):
        self._index = int(index)

    @property
    def id(self):
        v = C.c_int32()
        _dll.openmc_material_get_id(self._index, v)
        return v.value

    def _densities(self):
        nuc, dens, n = _p(C.c_int)(), _p(C.c_double)(), C.c_int()
        _dll.openmc_material_get_densities(self._index, nuc, dens, n)
        return [nuc[k] for k in range(n.value)], np.array([dens[k] for k in range(n.value)])

    @property
    def nuclides(self):
        names = []
        for i in self._densities()[0]:
            name = C.c_char_p()
            _dll.openmc_nuclide_name(i, name)
            names.append(name.value.decode())
        return names

    @property
    def densities(self):
        """Atom densities [atom/b-cm] in the order of ``nuclides``."""
        return self._densities()[1]

    def get_density(self, units="g/cm3"):
        if units != "g/cm3":
            raise ValueError("only g/cm3 is available")
        v = C.c_double()
        _dll.openmc_material_get_density(self._index, v)
        return v.value


class RegularMesh:
    """A regular mesh of the loaded model (openmc/lib/mesh.py, read-only)."""

    def __init__(self, index):
        self._index = int(index)

    @property
    def id(self):
        v = C.c_int32()
        _dll.openmc_mesh_get_id(self._index, v)
        return v.value

    @property
    def dimension(self):
        dims, n = _p(C.c_int)(), C.c_int()
        _dll.openmc_regular_mesh_get_dimension(self._index, dims, n)
        return tuple(dims[k] for k in range(n.value))

    def _params(self):
        ll, ur, w, n = _p(C.c_double)(), _p(C.c_double)(), _p(C.c_double)(), C.c_int()
        _dll.openmc_regular_mesh_get_params(self._index, ll, ur, w, n)
        return [np.array([p[k] for k in range(n.value)]) for p in (ll, ur, w)]

    @property
    def lower_left(self):
        return self._params()[0]

    @property
    def upper_right(self):
        return self._params()[1]

    @property
    def width(self):
        return self._params()[2]


class _IdMap:
    """id -> object mapping over the loaded model (openmc.lib.cells, ...)."""

    def __init__(self, cls, index_fn, id_fn, count):
        self._cls, self._index_fn, self._id_fn, self._count = cls, index_fn, id_fn, count

    def __getitem__(self, key):
        idx = C.c_int32()
        try:
            self._index_fn(key, idx)
        except InvalidIDError:
            raise KeyError(key)
        return self._cls(idx.value)

    def __len__(self):
        return self._count()

    def __iter__(self):
        v = C.c_int32()
        for i in range(len(self)):
            self._id_fn(i, v)
            yield v.value

    def keys(self):
        return list(iter(self))

    def values(self):
        return [self[k] for k in self]

    def items(self):
        return [(k, self[k]) for k in self]


def _model_count(k):
    info = (C.c_int64 * 8)()
    _dll.openmc_gb300_model_info(info)
    return int(info[k])


def _mesh_count():
    n, v = 0, C.c_int32()
    while True:
        try:
            _dll.openmc_mesh_get_id(n, v)
        except OutOfBoundsError:
            return n
        n += 1


cells = _IdMap(Cell, _dll.openmc_get_cell_index, _dll.openmc_cell_get_id, lambda: _model_count(2))
materials = _IdMap(Material, _dll.openmc_get_material_index, _dll.openmc_material_get_id, lambda: _model_count(1))
meshes = _IdMap(RegularMesh, _dll.openmc_get_mesh_index, _dll.openmc_mesh_get_id, _mesh_count)


def global_bounding_box():
    """(lower-left, upper-right) of the root universe (openmc/lib/core.py)."""
    lo, hi = (C.c_double * 3)(), (C.c_double * 3)()
    _dll.openmc_global_bounding_box(lo, hi)
    return np.array(lo), np.array(hi)


def keff():
    """(k, standard deviation) of openmc_get_keff (openmc/lib/core.py): the
    combined estimate of an eigenvalue run; 1 with an infinite (one
    realization or fewer) or zero spread in a fixed-source run."""
    k = (C.c_double * 2)()
    _dll.openmc_get_keff(k)
    return k[0], k[1]


def statepoint_write(filename=None, write_source=True):
    """Write a statepoint file (openmc/lib/core.py: statepoint_write); no
    source bank is written.  filename None: statepoint.<batch>.h5 in the
    output path."""
    flag = C.c_bool(bool(write_source))
    _dll.openmc_statepoint_write(None if filename is None else str(filename).encode(), C.byref(flag))


def k_generation():
    """Eigenvalue run: (track-length k of every generation so far, the last
    generation's fission-bank size)."""
    n = _dll.openmc_gb300_k_generation(None, 0, None)
    k = (C.c_double * max(n, 1))()
    sites = C.c_int64()
    _dll.openmc_gb300_k_generation(k, n, C.byref(sites))
    return np.array(k[:n]), sites.value


class WeightWindows:
    """openmc.lib.WeightWindows subset (openmc/lib/weight_windows.py)."""

    def __init__(self, index):
        self._index = index

    @classmethod
    def from_id(cls, ww_id):
        idx = C.c_int32()
        _dll.openmc_get_weight_windows_index(int(ww_id), C.byref(idx))
        return cls(idx.value)

    @property
    def id(self):
        v = C.c_int32()
        _dll.openmc_weight_windows_get_id(self._index, C.byref(v))
        return v.value

    @property
    def bounds(self):
        lo, up = _p(C.c_double)(), _p(C.c_double)()
        n = C.c_size_t()
        _dll.openmc_weight_windows_get_bounds(self._index, C.byref(lo), C.byref(up), C.byref(n))
        return (np.ctypeslib.as_array(lo, shape=(n.value,)).copy(),
                np.ctypeslib.as_array(up, shape=(n.value,)).copy())

    @bounds.setter
    def bounds(self, lu):
        lower = np.ascontiguousarray(lu[0], dtype=np.float64).ravel()
        upper = np.ascontiguousarray(lu[1], dtype=np.float64).ravel()
        _dll.openmc_weight_windows_set_bounds(self._index, lower.ctypes.data_as(_p(C.c_double)),
                                              upper.ctypes.data_as(_p(C.c_double)), lower.size)

    @property
    def energy_bounds(self):
        ptr = _p(C.c_double)()
        n = C.c_size_t()
        _dll.openmc_weight_windows_get_energy_bounds(self._index, C.byref(ptr), C.byref(n))
        return np.ctypeslib.as_array(ptr, shape=(n.value,)).copy()

    def update_magic(self, tally_index, value="mean", threshold=1.0, ratio=5.0):
        _dll.openmc_weight_windows_update_magic(self._index, int(tally_index), value.encode(),
                                                float(threshold), float(ratio))


def weight_windows_size():
    return _dll.openmc_weight_windows_size()


def set_weight_windows_on(on):
    _dll.openmc_gb300_set_weight_windows_on(1 if on else 0)


# ---------------------------------------------------- GB300 extensions
TRACE_DTYPE = np.dtype([("kind", "<i4"), ("cell", "<i4"), ("material", "<i4"),
                        ("surface_or_nuclide", "<i4"), ("grid_hash", "<i4"),
                        ("n_coord", "<i4"), ("E", "<f8"), ("dist", "<f8"),
                        ("wgt", "<f8")])


def set_trace(n_hist, cap=256):
    """Record per-event traces for particle ids 1..n_hist of each batch."""
    _dll.openmc_gb300_set_trace(int(n_hist), int(cap))
    set_trace._shape = (int(n_hist), int(cap))


def get_trace():
    n, cap = set_trace._shape
    rec = np.zeros((n, cap), dtype=TRACE_DTYPE)
    cnt = np.zeros(n, dtype=np.int32)
    _dll.openmc_gb300_get_trace(rec.ctypes.data_as(C.c_void_p), cnt.ctypes.data_as(_p(C.c_int32)))
    return rec, cnt


def last_batch():
    out = (C.c_double * 10)()
    _dll.openmc_gb300_last_batch(out)
    keys = ("ms", "iterations", "events", "total_weight", "leakage", "lost", "done", "secondaries",
            "longest_events", "longest_id")
    return dict(zip(keys, list(out)))


def last_batch_detail():
    """Event statistics of the last batch for the queue and tail phases, and
    per-kernel milliseconds when the batch ran with settings.profile_next."""
    out = (C.c_double * 23)()
    _dll.openmc_gb300_last_batch_detail(out)
    v = list(out)
    keys = ("xs_events", "xs_calc", "xs_nuclide_lookups", "mesh_segments",
            "collision_nuclide_lookups", "surface", "collision")
    d = {"queue": dict(zip(keys, v[0:7])), "tail": dict(zip(keys, v[7:14]))}
    d["kernel_ms"] = dict(zip(("xs", "advance", "surface", "collision", "tail", "refill", "sort", "other",
                               "tally"), v[14:23]))
    return d


def timing():
    out = (C.c_double * 5)()
    _dll.openmc_gb300_timing(out)
    keys = ("time_active", "time_inactive", "time_wall_active", "calculation_rate", "in_flight")
    return dict(zip(keys, list(out)))


def material_xs(materials, energies):
    """Macroscopic (total, absorption) cross sections and the nuclide
    grid-index hash at (material index, E) pairs, from the transport kernels'
    own device lookup of the initialised simulation."""
    mats = np.ascontiguousarray(materials, np.int32)
    e = np.ascontiguousarray(energies, np.float64)
    n = len(e)
    tot, ab = np.empty(n), np.empty(n)
    gh = np.empty(n, np.uint32)
    _dll.openmc_gb300_material_xs(n, mats.ctypes.data_as(_p(C.c_int32)), e.ctypes.data_as(_p(C.c_double)),
                                  tot.ctypes.data_as(_p(C.c_double)), ab.ctypes.data_as(_p(C.c_double)),
                                  gh.ctypes.data_as(_p(C.c_uint32)))
    return tot, ab, gh


def loaded_library():
    return str(_LIB)


class XSTables:
    """Device tables for the macroscopic-XS lookup microbenchmark."""

    def __init__(self, data, n_log_bins=8000, fp32=False, max_lookups=0):
        n_nuc, G = data.energy.shape
        e = np.ascontiguousarray(data.energy, np.float64)
        x = np.ascontiguousarray(data.xs, np.float64)
        mo = np.ascontiguousarray(data.mat_off, np.int32)
        mn = np.ascontiguousarray(data.mat_nuc, np.int32)
        md = np.ascontiguousarray(data.mat_dens, np.float64)
        h = C.c_void_p()
        _dll.openmc_gb300_xs_tables_create(n_nuc, G, e.ctypes.data_as(_p(C.c_double)),
                                           x.ctypes.data_as(_p(C.c_double)), len(mo) - 1,
                                           mo.ctypes.data_as(_p(C.c_int32)), mn.ctypes.data_as(_p(C.c_int32)),
                                           md.ctypes.data_as(_p(C.c_double)), n_log_bins, 1 if fp32 else 0,
                                           int(max_lookups), C.byref(h))
        self.h = h

    def close(self):
        if self.h:
            _dll.openmc_gb300_xs_tables_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def lookup(self, mats, energies, sort=True, grid_hash=True):
        mats = np.ascontiguousarray(mats, np.int32)
        e = np.ascontiguousarray(energies, np.float64)
        out = np.empty((len(e), 5))
        gh = np.empty(len(e), np.int32) if grid_hash else None
        _dll.openmc_gb300_xs_lookup(self.h, len(e), mats.ctypes.data_as(_p(C.c_int32)),
                                    e.ctypes.data_as(_p(C.c_double)), out.ctypes.data_as(_p(C.c_double)),
                                    gh.ctypes.data_as(_p(C.c_int32)) if gh is not None else None,
                                    1 if sort else 0)
        return out, gh

    def lookup_device(self, n, d_mat, d_E, d_out, d_hash=None, sort=True):
        """Device pointers (ints) in, asynchronous on the library stream."""
        _dll.openmc_gb300_xs_lookup_device(self.h, int(n), d_mat, d_E, d_out, d_hash, 1 if sort else 0)

    def lookup_noalloc(self, n, d_mat, d_E, d_out, d_hash=None, stream=None):
        """Sorted lookups without any device allocation in the call: the sort
        scratch is a static array of the library (at most 4,194,304 lookups
        per call; calls that overlap on the GPU race).  Device pointers (ints)
        in; queued on `stream` (a cudaStream_t handle, None for the default
        stream) without waiting."""
        _dll.openmc_gb300_xs_lookup_noalloc(self.h, int(n), d_mat, d_E, d_out, d_hash, stream)

    def last_times(self):
        ms = (C.c_float * 2)()
        _dll.openmc_gb300_xs_last_times(self.h, ms)
        return float(ms[0]), float(ms[1])

    def stream(self):
        s = C.c_void_p()
        _dll.openmc_gb300_xs_stream(self.h, C.byref(s))
        return s.value


def _f32(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float32)
    if shape is not None:
        a = a.reshape(shape)
    return a


class ImportanceNetwork:
    """The learned-weight-window network on the GPU: (x, y, z, log E) -> a
    regression target (log flux), 4 -> 128 -> 128 -> 128 -> 1 with SiLU,
    BF16 tensor-core products accumulating in FP32, full-batch Adam."""

    n_params = int(_dll.openmc_gb300_mlp_n_params())

    def __init__(self, max_rows=1 << 16, seed=1):
        h = C.c_void_p()
        _dll.openmc_gb300_mlp_create(int(max_rows), int(seed), C.byref(h))
        self.h = h

    def close(self):
        if self.h:
            _dll.openmc_gb300_mlp_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_data(self, x4, target, weight=None):
        x4 = _f32(x4)
        n = x4.shape[0]
        x4 = x4.reshape(n, 4)
        t = _f32(target, (n,))
        w = _f32(weight, (n,)) if weight is not None else None
        self._keep = (x4, t, w)
        _dll.openmc_gb300_mlp_set_data(self.h, n, x4.ctypes.data_as(_p(C.c_float)),
                                       t.ctypes.data_as(_p(C.c_float)),
                                       w.ctypes.data_as(_p(C.c_float)) if w is not None else None)

    def train(self, steps, lr=1e-3):
        """Runs `steps` Adam steps; returns the loss before each update."""
        loss = np.zeros(max(int(steps), 1), np.float32)
        _dll.openmc_gb300_mlp_train(self.h, int(steps), float(lr), loss.ctypes.data_as(_p(C.c_float)))
        return loss[:int(steps)]

    def gradients(self):
        """(loss, dLoss/dparams) over the staged rows, without an update."""
        g = np.zeros(self.n_params, np.float32)
        loss = C.c_float()
        _dll.openmc_gb300_mlp_gradients(self.h, g.ctypes.data_as(_p(C.c_float)), C.byref(loss))
        return float(loss.value), g

    def predict(self, x4):
        x4 = _f32(x4)
        n = x4.shape[0]
        x4 = x4.reshape(n, 4)
        y = np.zeros(n, np.float32)
        _dll.openmc_gb300_mlp_predict(self.h, n, x4.ctypes.data_as(_p(C.c_float)),
                                      y.ctypes.data_as(_p(C.c_float)))
        return y

    @property
    def params(self):
        p = np.zeros(self.n_params, np.float32)
        _dll.openmc_gb300_mlp_get_params(self.h, p.ctypes.data_as(_p(C.c_float)), self.n_params)
        return p

    @params.setter
    def params(self, p):
        p = _f32(p, (self.n_params,))
        _dll.openmc_gb300_mlp_set_params(self.h, p.ctypes.data_as(_p(C.c_float)), self.n_params)

    def last_train_ms(self):
        ms = C.c_float()
        _dll.openmc_gb300_mlp_last_ms(self.h, C.byref(ms))
        return float(ms.value)
