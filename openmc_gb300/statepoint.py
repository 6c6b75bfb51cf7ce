"""Reader of the statepoint files the library writes (statepoint format
18.1, docs/source/io_formats/statepoint.rst), with the part of
``openmc.StatePoint`` (openmc/statepoint.py) a tally user reads: run
parameters, k-effective, global tallies and each tally's sums, means and
standard deviations.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import h5

_GLOBAL_NAMES = ("k-collision", "k-absorption", "k-tracklength", "leakage")


def _str(v):
    v = np.asarray(v).reshape(-1)[0] if np.asarray(v).ndim else np.asarray(v).item()
    return v.decode().rstrip("\0") if isinstance(v, (bytes, np.bytes_)) else str(v)


def _strs(v):
    return [x.decode().rstrip("\0") if isinstance(x, (bytes, np.bytes_)) else str(x)
            for x in np.asarray(v).reshape(-1)]


def _int(v):
    return int(np.asarray(v).reshape(-1)[0])


@dataclass
class Filter:
    id: int
    type: str
    bins: np.ndarray
    num_bins: int


@dataclass
class Mesh:
    id: int
    dimension: tuple
    lower_left: np.ndarray
    upper_right: np.ndarray
    width: np.ndarray


@dataclass
class Tally:
    """``openmc.Tally`` as read from a statepoint (openmc/tallies.py:
    sum, sum_sq, mean, std_dev over [filter bins][nuclides][scores])."""
    id: int
    estimator: str
    filters: list
    scores: list
    nuclides: list
    num_realizations: int
    sum: np.ndarray = field(repr=False)
    sum_sq: np.ndarray = field(repr=False)

    @property
    def mean(self):
        n = self.num_realizations
        return self.sum / n if n > 0 else np.zeros_like(self.sum)

    @property
    def std_dev(self):
        n = self.num_realizations
        if n <= 1:
            return np.zeros_like(self.sum)
        mean = self.sum / n
        with np.errstate(invalid="ignore"):
            return np.sqrt(np.maximum((self.sum_sq / n - mean * mean) / (n - 1), 0.0))


class StatePoint:
    """Statepoint file contents (openmc/statepoint.py: StatePoint)."""

    def __init__(self, path):
        self.path = Path(path)
        f = h5.read(self.path)
        if _str(f.attrs["filetype"]) != "statepoint":
            raise ValueError(f"{path} is not a statepoint file")
        self.version = tuple(int(v) for v in np.asarray(f.attrs["version"]).reshape(-1))
        if self.version[0] != 18:
            raise ValueError(f"statepoint version {self.version} is not supported")
        self.seed = _int(f["seed"])
        self.stride = _int(f["stride"])
        self.run_mode = _str(f["run_mode"])
        self.n_particles = _int(f["n_particles"])
        self.n_batches = _int(f["n_batches"])
        self.current_batch = _int(f["current_batch"])
        self.n_realizations = _int(f["n_realizations"])
        self.tallies_present = bool(_int(f.attrs["tallies_present"]))
        self.source_present = bool(_int(f.attrs["source_present"]))
        gt = np.asarray(f["global_tallies"], dtype=np.float64).reshape(4, 2)
        n = self.n_realizations
        mean = gt[:, 0] / n if n > 0 else np.zeros(4)
        std = np.zeros(4)
        if n > 1:
            std = np.sqrt(np.maximum((gt[:, 1] / n - mean * mean) / (n - 1), 0.0))
        self.global_tallies = np.zeros(4, dtype=[("name", "U16"), ("sum", "f8"), ("sum_sq", "f8"),
                                                 ("mean", "f8"), ("std_dev", "f8")])
        for k in range(4):
            self.global_tallies[k] = (_GLOBAL_NAMES[k], gt[k, 0], gt[k, 1], mean[k], std[k])
        if self.run_mode == "eigenvalue":
            self.n_inactive = _int(f["n_inactive"])
            self.k_generation = np.asarray(f["k_generation"], dtype=np.float64).reshape(-1)
            kc = np.asarray(f["k_combined"], dtype=np.float64).reshape(-1)
            self.k_combined = (float(kc[0]), float(kc[1]))
        t = f["tallies"]
        self.meshes = {}
        for name, g in t["meshes"].items():
            if isinstance(g, dict):
                self.meshes[_int(g.attrs["id"])] = Mesh(
                    _int(g.attrs["id"]), tuple(int(v) for v in np.asarray(g["dimension"]).reshape(-1)),
                    np.asarray(g["lower_left"], dtype=np.float64), np.asarray(g["upper_right"], dtype=np.float64),
                    np.asarray(g["width"], dtype=np.float64))
        self.filters = {}
        for name, g in t["filters"].items():
            if isinstance(g, dict):
                fid = int(name.split()[1])
                ftype = _str(g["type"])
                bins = np.asarray(g["bins"])
                if ftype == "particle":
                    bins = np.array(_strs(bins))
                self.filters[fid] = Filter(fid, ftype, bins, _int(g["n_bins"]))
        self.tallies = {}
        for name, g in t.items():
            if not name.startswith("tally "):
                continue
            tid = int(name.split()[1])
            res = np.asarray(g["results"], dtype=np.float64)
            fids = [int(v) for v in np.asarray(g["filters"]).reshape(-1)] if _int(g["n_filters"]) else []
            self.tallies[tid] = Tally(
                tid, _str(g["estimator"]), [self.filters[i] for i in fids], _strs(g["score_bins"]),
                _strs(g["nuclides"]), _int(g["n_realizations"]),
                res[..., 0].reshape(res.shape[0], 1, res.shape[1]).copy(),
                res[..., 1].reshape(res.shape[0], 1, res.shape[1]).copy())

    def get_tally(self, id=None):
        """The tally with this id (openmc/statepoint.py: get_tally, by id only)."""
        if id is None:
            if len(self.tallies) != 1:
                raise LookupError("more than one tally: give an id")
            return next(iter(self.tallies.values()))
        try:
            return self.tallies[int(id)]
        except KeyError:
            raise LookupError(f"no tally with id {id}") from None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        return False
