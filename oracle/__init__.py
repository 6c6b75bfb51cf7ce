"""ORACLE — test infrastructure only.

ctypes wrapper over ``oracle/_build/liboracle.so`` (the CPU restatement of the
reference transport path in ``oracle.cpp``) and over
``oracle/_ref/librandom_lcg_ref.so`` (the reference's own ``random_lcg.cpp``
compiled from source).  Only the tests, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` may use this package, and only to check
results or as a timed baseline: nothing in ``openmc_gb300`` imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

from . import flatten

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "liboracle.so"
# the same source built with the reference's default release flags
# (RelWithDebInfo: -O2 -g -DNDEBUG, the compiler's default FP contraction) for
# timing; the parity build keeps every multiply and add separately rounded
TIMING_LIB_PATH = HERE / "_build" / "liboracle_timing.so"
REF_PATH = HERE / "_ref" / "librandom_lcg_ref.so"

TRACE_DTYPE = np.dtype([("kind", "<i4"), ("cell", "<i4"), ("material", "<i4"),
                        ("surface_or_nuclide", "<i4"), ("grid_hash", "<i4"),
                        ("n_coord", "<i4"), ("E", "<f8"), ("dist", "<f8"),
                        ("wgt", "<f8")])

_libs = {}


def build(force=False):
    """Compile the oracle libraries (make) if missing."""
    if force or not LIB_PATH.exists() or not TIMING_LIB_PATH.exists():
        subprocess.run(["make", "-C", str(HERE)], check=True,
                       stdout=subprocess.DEVNULL)
    return LIB_PATH


def lib(timing=False):
    """The parity build of the oracle library, or with timing=True the
    timing build of the same source."""
    if timing not in _libs:
        build()
        L = C.CDLL(str(TIMING_LIB_PATH if timing else LIB_PATH))
        vp, i64, i32, dbl = C.c_void_p, C.c_int64, C.c_int32, C.c_double
        pd = C.POINTER(C.c_double)
        pi32 = C.POINTER(C.c_int32)
        pu64 = C.POINTER(C.c_uint64)
        L.oracle_create.restype = vp
        L.oracle_create.argtypes = [C.c_char_p, C.c_size_t, C.c_char_p, C.c_int]
        L.oracle_destroy.argtypes = [vp]
        L.oracle_set_trace.argtypes = [vp, i64, C.c_int, C.c_int]
        L.oracle_trace_data.restype = vp
        L.oracle_trace_data.argtypes = [vp]
        L.oracle_trace_counts.restype = pi32
        L.oracle_trace_counts.argtypes = [vp]
        L.oracle_transport.restype = C.c_int
        L.oracle_transport.argtypes = [vp, C.c_int, i64, i64, C.c_int, C.c_int, i64]
        L.oracle_accumulate.argtypes = [vp]
        L.oracle_n_tallies.restype = C.c_int
        L.oracle_n_tallies.argtypes = [vp]
        L.oracle_tally_size.restype = i64
        L.oracle_tally_size.argtypes = [vp, C.c_int]
        L.oracle_tally_results.restype = pd
        L.oracle_tally_results.argtypes = [vp, C.c_int]
        L.oracle_globals.argtypes = [vp, pd]
        L.oracle_macro_xs.argtypes = [vp, i64, pi32, pd, pd, pd, pi32]
        L.oracle_grid_index.restype = C.c_int
        L.oracle_grid_index.argtypes = [vp, C.c_int, pi32, C.c_int]
        L.oracle_error.restype = C.c_char_p
        L.oracle_error.argtypes = [vp]
        L.oracle_prn.restype = dbl
        L.oracle_prn.argtypes = [pu64]
        L.oracle_future_seed.restype = C.c_uint64
        L.oracle_future_seed.argtypes = [C.c_uint64, C.c_uint64]
        L.oracle_init_seed.restype = C.c_uint64
        L.oracle_init_seed.argtypes = [i64, C.c_int, i64, C.c_uint64]
        L.oracle_lower_bound_index.restype = C.c_int64
        L.oracle_lower_bound_index.argtypes = [C.POINTER(C.c_double), C.c_int64, dbl]
        L.oracle_maxwell_spectrum.restype = dbl
        L.oracle_maxwell_spectrum.argtypes = [dbl, pu64]
        L.oracle_watt_spectrum.restype = dbl
        L.oracle_watt_spectrum.argtypes = [dbl, dbl, pu64]
        L.oracle_rotate_angle.argtypes = [pd, dbl, pd, pu64]
        L.oracle_xsb_create.restype = vp
        L.oracle_xsb_create.argtypes = [C.c_int, C.c_int, pd, pd, C.c_int, pi32, pi32, pd, C.c_int]
        L.oracle_xsb_destroy.argtypes = [vp]
        L.oracle_xsb_grid_index.argtypes = [vp, pi32]
        L.oracle_xsb_lookup.argtypes = [vp, i64, pi32, pd, pd, pi32, C.c_int]
        L.oracle_eigen_begin.restype = C.c_int
        L.oracle_eigen_begin.argtypes = [vp, C.c_int]
        L.oracle_eigen_end.restype = C.c_int
        L.oracle_eigen_end.argtypes = [vp, C.c_int]
        L.oracle_keff.restype = C.c_int
        L.oracle_keff.argtypes = [vp, pd, pd, C.c_int]
        L.oracle_keff_combined.argtypes = [vp, pd]
        L.oracle_source_bank.restype = i64
        L.oracle_source_bank.argtypes = [vp, pd, i64]
        _libs[timing] = L
    return _libs[timing]


def ref_lib():
    """The reference's random_lcg.cpp and random_dist.cpp compiled from
    source, or None."""
    if not REF_PATH.exists():
        return None
    L = C.CDLL(str(REF_PATH))
    L.ref_prn.restype = C.c_double
    L.ref_prn.argtypes = [C.POINTER(C.c_uint64)]
    L.ref_future_seed.restype = C.c_uint64
    L.ref_future_seed.argtypes = [C.c_uint64, C.c_uint64]
    L.ref_init_seed.restype = C.c_uint64
    L.ref_init_seed.argtypes = [C.c_int64, C.c_int, C.c_int64, C.c_uint64]
    pu64 = C.POINTER(C.c_uint64)
    if hasattr(L, "ref_lower_bound_index"):
        L.ref_lower_bound_index.restype = C.c_int64
        L.ref_lower_bound_index.argtypes = [C.POINTER(C.c_double), C.c_int64, C.c_double]
    for name, args in (("ref_uniform", [C.c_double, C.c_double, pu64]), ("ref_maxwell", [C.c_double, pu64]),
                       ("ref_watt", [C.c_double, C.c_double, pu64]),
                       ("ref_normal", [C.c_double, C.c_double, pu64])):
        if hasattr(L, name):  # built from random_dist.cpp as well
            getattr(L, name).restype = C.c_double
            getattr(L, name).argtypes = args
    return L


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


class Oracle:
    """One oracle simulation built from a model.xml."""

    def __init__(self, model_xml, cross_sections=None, timing=False):
        """timing=True runs the timing build (the reference's release
        flags) instead of the parity build."""
        self.L = L = lib(timing)
        self.arrays = flatten.load_model(model_xml, cross_sections)
        blob = flatten.to_blob(self.arrays)
        err = C.create_string_buffer(512)
        self.h = L.oracle_create(blob, len(blob), err, 512)
        if not self.h:
            raise RuntimeError(err.value.decode())
        self.n_particles = int(self.arrays["settings_i"][0])
        self.n_batches = int(self.arrays["settings_i"][1])
        self.eigenvalue = bool(self.arrays["eig_i"][0])
        self._trace = None

    def __del__(self):
        if getattr(self, "h", None):
            self.L.oracle_destroy(self.h)
            self.h = None

    def set_trace(self, n_hist, cap=256, batch=1):
        self.L.oracle_set_trace(self.h, n_hist, cap, batch)
        self._trace = (n_hist, cap)

    def transport(self, batch, first=1, count=None, mode=0, threads=1, in_flight=0):
        count = self.n_particles if count is None else count
        rc = self.L.oracle_transport(self.h, batch, first, count, mode, threads, in_flight)
        if rc != 0:
            raise RuntimeError(self.L.oracle_error(self.h).decode())

    def accumulate(self):
        self.L.oracle_accumulate(self.h)

    def run(self, batches=None, threads=1, mode=0, count=None):
        """Transport and accumulate each batch; an eigenvalue run also starts
        each generation from its source bank and ends it with the fission
        bank's sort and comb and the k-effective bookkeeping."""
        for b in range(1, (batches or self.n_batches) + 1):
            if self.eigenvalue:
                if self.L.oracle_eigen_begin(self.h, b) != 0:
                    raise RuntimeError(self.L.oracle_error(self.h).decode())
            self.transport(b, count=count, threads=threads, mode=mode)
            if self.eigenvalue:
                if self.L.oracle_eigen_end(self.h, b) != 0:
                    raise RuntimeError(self.L.oracle_error(self.h).decode())
            else:
                self.accumulate()

    def keff(self):
        """Eigenvalue run: dict of keff, keff_std (of the average over active
        generations), n_realizations, the last generation's fission sites,
        the k estimators' SUM/SUM_SQ and cross sums, and every generation's
        k (track-length estimate / n_particles)."""
        out = np.zeros(13)
        kg = np.zeros(100000)
        n = self.L.oracle_keff(self.h, _p(out, C.c_double), _p(kg, C.c_double), len(kg))
        names = ("keff", "keff_std", "n_realizations", "fission_sites", "k_col_sum", "k_col_sq", "k_abs_sum",
                 "k_abs_sq", "k_tra_sum", "k_tra_sq", "k_col_abs", "k_col_tra", "k_abs_tra")
        d = dict(zip(names, out.tolist()))
        d["k_generation"] = kg[:n].copy()
        kc = np.zeros(2)
        self.L.oracle_keff_combined(self.h, _p(kc, C.c_double))
        d["k_combined"] = (float(kc[0]), float(kc[1]))
        return d

    def source_bank(self, n=None):
        """The coming generation's source sites: (n, 8) [r, u, E, wgt]."""
        n = self.n_particles if n is None else n
        out = np.zeros((n, 8))
        m = self.L.oracle_source_bank(self.h, _p(out, C.c_double), n)
        return out[:m]

    def tally(self, t):
        L = self.L
        n = L.oracle_tally_size(self.h, t)
        ptr = L.oracle_tally_results(self.h, t)
        return np.ctypeslib.as_array(ptr, shape=(n,)).reshape(-1, 3).copy()

    @property
    def n_tallies(self):
        return self.L.oracle_n_tallies(self.h)

    def globals(self):
        out = np.zeros(8)
        self.L.oracle_globals(self.h, _p(out, C.c_double))
        return out

    def traces(self):
        n_hist, cap = self._trace
        L = self.L
        raw = L.oracle_trace_data(self.h)
        buf = (C.c_char * (n_hist * cap * TRACE_DTYPE.itemsize)).from_address(raw)
        rec = np.frombuffer(buf, TRACE_DTYPE).reshape(n_hist, cap).copy()
        cnt = np.ctypeslib.as_array(L.oracle_trace_counts(self.h), shape=(n_hist,)).copy()
        return rec, cnt

    def macro_xs(self, mats, energies):
        mats = np.ascontiguousarray(mats, np.int32)
        e = np.ascontiguousarray(energies, np.float64)
        n = len(e)
        tot, ab = np.empty(n), np.empty(n)
        gh = np.empty(n, np.int32)
        self.L.oracle_macro_xs(self.h, n, _p(mats, C.c_int32), _p(e, C.c_double),
                              _p(tot, C.c_double), _p(ab, C.c_double), _p(gh, C.c_int32))
        return tot, ab, gh

    def grid_index(self, nuc):
        n = self.L.oracle_grid_index(self.h, nuc, None, 0)
        out = np.empty(n, np.int32)
        self.L.oracle_grid_index(self.h, nuc, _p(out, C.c_int32), n)
        return out


class XSBenchOracle:
    """CPU restatement of the macroscopic lookup on flat 5-channel tables."""

    def __init__(self, data, n_log_bins=8000):
        L = lib()
        n_nuc, G = data.energy.shape
        self._keep = [np.ascontiguousarray(data.energy), np.ascontiguousarray(data.xs),
                      np.ascontiguousarray(data.mat_off, np.int32),
                      np.ascontiguousarray(data.mat_nuc, np.int32),
                      np.ascontiguousarray(data.mat_dens)]
        e, x, mo, mn, md = self._keep
        self.n_nuc, self.G, self.M = n_nuc, G, n_log_bins
        self.h = L.oracle_xsb_create(n_nuc, G, _p(e, C.c_double), _p(x, C.c_double),
                                     len(mo) - 1, _p(mo, C.c_int32), _p(mn, C.c_int32),
                                     _p(md, C.c_double), n_log_bins)

    def __del__(self):
        if getattr(self, "h", None):
            lib().oracle_xsb_destroy(self.h)
            self.h = None

    def grid_index(self):
        out = np.empty((self.n_nuc, self.M + 1), np.int32)
        lib().oracle_xsb_grid_index(self.h, _p(out, C.c_int32))
        return out

    def lookup(self, mats, energies, threads=1):
        mats = np.ascontiguousarray(mats, np.int32)
        e = np.ascontiguousarray(energies, np.float64)
        out = np.empty((len(e), 5))
        gh = np.empty(len(e), np.int32)
        lib().oracle_xsb_lookup(self.h, len(e), _p(mats, C.c_int32), _p(e, C.c_double),
                                _p(out, C.c_double), _p(gh, C.c_int32), threads)
        return out, gh


# ---- functions pinned against the reference's test_math.cpp golden values
def prn(seed: int):
    s = C.c_uint64(seed)
    v = lib().oracle_prn(C.byref(s))
    return v, s.value


def maxwell_spectrum(T, seed):
    s = C.c_uint64(seed)
    return lib().oracle_maxwell_spectrum(T, C.byref(s))


def watt_spectrum(a, b, seed):
    s = C.c_uint64(seed)
    return lib().oracle_watt_spectrum(a, b, C.byref(s))


def rotate_angle(uvw, mu, phi, seed):
    u = np.ascontiguousarray(uvw, np.float64).copy()
    s = C.c_uint64(seed)
    ph = None if phi is None else C.byref(C.c_double(phi))
    lib().oracle_rotate_angle(_p(u, C.c_double), mu, ph, C.byref(s))
    return u, s.value


def future_seed(n, seed):
    return lib().oracle_future_seed(n, seed)


def init_seed(id_, offset, master=1, stride=152917):
    return lib().oracle_init_seed(id_, offset, master, stride)
