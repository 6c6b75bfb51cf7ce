"""Learned weight windows: an importance network fitted to pilot mesh-flux
tallies sets the bounds that the unchanged splitting / roulette logic reads.

No reference counterpart.  It stands where OpenMC's MAGIC generator stands
(``WeightWindows::update_weights``, src/weight_windows.cpp:502-755): the
same inputs (a flux tally on the weight-window mesh and energy groups), the
same normalisation of the output (per energy group, lower bound = flux /
(2 max flux), upper = ratio x lower, weight_windows.cpp:690-725), and the
same consumer (``apply_weight_windows``, :56-146).  MAGIC leaves a bin
without a window where the pilot flux is zero or noisier than the threshold;
the network instead predicts log flux everywhere from the (x, y, z, log E)
of the bin centre, so windows reach into regions the pilot never scored.
Splitting and roulette preserve the expected weight, so any positive bounds
keep the estimator unbiased.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np

from . import lib


@dataclass
class MeshGeometry:
    """Regular mesh and energy groups of a weight-window set."""
    lower_left: np.ndarray
    upper_right: np.ndarray
    dimension: tuple
    energy_bounds: np.ndarray

    @property
    def n_mesh(self):
        return int(np.prod(self.dimension))

    @property
    def n_groups(self):
        return len(self.energy_bounds) - 1

    def centres(self):
        """Bin centres [n_mesh][3], x index fastest (mesh.cpp:888-900)."""
        nx, ny, nz = (list(self.dimension) + [1, 1])[:3]
        w = (self.upper_right - self.lower_left) / np.array([nx, ny, nz], dtype=float)
        ix = np.arange(self.n_mesh) % nx
        iy = (np.arange(self.n_mesh) // nx) % ny
        iz = np.arange(self.n_mesh) // (nx * ny)
        return self.lower_left + (np.stack([ix, iy, iz], 1) + 0.5) * w


@dataclass
class Features:
    """Affine maps of the network's inputs and target."""
    e_lo: float
    e_hi: float
    mu: float = 0.0
    sigma: float = 1.0
    geom: MeshGeometry = None

    def inputs(self):
        """[n_groups * n_mesh][4] features, group-major like the bound arrays."""
        g = self.geom
        c = g.centres()
        xyz = 2.0 * (c - g.lower_left) / (g.upper_right - g.lower_left) - 1.0
        eb = np.maximum(np.asarray(g.energy_bounds, float), 1.0e-5)
        le = 0.5 * (np.log(eb[:-1]) + np.log(eb[1:]))
        le = 2.0 * (le - self.e_lo) / (self.e_hi - self.e_lo) - 1.0
        x4 = np.empty((g.n_groups, g.n_mesh, 4))
        x4[:, :, :3] = xyz[None]
        x4[:, :, 3] = le[:, None]
        return x4.reshape(-1, 4)


@dataclass
class Result:
    lower: np.ndarray
    upper: np.ndarray
    loss: np.ndarray
    train_ms: float
    n_pairs: int
    info: dict = field(default_factory=dict)


def scored_bins(mean, std, geom, rel_max=1.0):
    """Bins [n_groups * n_mesh, group-major] that enter the training set."""
    m = np.asarray(mean, float).reshape(geom.n_mesh, geom.n_groups).T
    s = np.asarray(std, float).reshape(geom.n_mesh, geom.n_groups).T
    rel = np.where(m > 0, s / np.where(m > 0, m, 1.0), np.inf)
    return ((m > 0) & (rel < rel_max)).ravel()


def training_pairs(mean, std, geom, rel_max=1.0, rel_floor=0.05):
    """(features, target, weight) from a pilot flux tally.

    mean, std: [n_mesh][n_groups] flux means and standard deviations of the
    mean.  Pairs are the bins scored with relative error below rel_max; the
    target is the standardised log flux, the weight 1 / (rel^2 + rel_floor^2)
    normalised to mean 1 (inverse variance of log flux, capped)."""
    eb = np.maximum(np.asarray(geom.energy_bounds, float), 1.0e-5)
    f = Features(float(np.log(eb[0])), float(np.log(eb[-1])), geom=geom)
    if f.e_hi <= f.e_lo:
        f.e_hi = f.e_lo + 1.0
    x_all = f.inputs().reshape(geom.n_groups, geom.n_mesh, 4)
    m = np.asarray(mean, float).reshape(geom.n_mesh, geom.n_groups).T
    s = np.asarray(std, float).reshape(geom.n_mesh, geom.n_groups).T
    rel = np.where(m > 0, s / np.where(m > 0, m, 1.0), np.inf)
    ok = (m > 0) & (rel < rel_max)
    if ok.sum() < 8:
        raise ValueError("too few scored bins in the pilot tally to fit an importance network")
    logf = np.log(m[ok])
    f.mu = float(logf.mean())
    f.sigma = float(max(logf.std(), 1e-6))
    target = (logf - f.mu) / f.sigma
    w = 1.0 / (rel[ok] ** 2 + rel_floor ** 2)
    w = w / w.mean()
    return x_all[ok], target, w, f


def bounds_from_log_flux(log_flux, geom, ratio=5.0, scored=None, max_extrapolation=1.0e3):
    """MAGIC's normalisation applied to a predicted flux [n_groups * n_mesh]:
    per group lower = flux / (2 max), upper = ratio * lower.

    scored (bool [n_groups * n_mesh], optional): bins the pilot scored.  In
    the other bins the prediction is an extrapolation; there the lower bound
    is kept at or above the group's lowest scored bound / max_extrapolation,
    so that an extrapolation far below the true flux cannot split a particle
    into an unbounded number of copies (a bound above the true flux only
    rouletted particles, which costs efficiency, not correctness)."""
    lf = np.asarray(log_flux, float).reshape(geom.n_groups, geom.n_mesh)
    lf = lf - lf.max(axis=1, keepdims=True)
    lower = 0.5 * np.exp(lf)
    if scored is not None:
        sc = np.asarray(scored, bool).reshape(geom.n_groups, geom.n_mesh)
        for g in range(geom.n_groups):
            if sc[g].any():
                floor = lower[g][sc[g]].min() / max_extrapolation
                lower[g] = np.where(sc[g], lower[g], np.maximum(lower[g], floor))
    return lower.ravel(), ratio * lower.ravel()


def fit(mean, std, geom, steps=2000, lr=2e-3, seed=1, ratio=5.0, rel_max=1.0):
    """Trains the importance network on the GPU and returns the bounds."""
    x4, target, weight, feats = training_pairs(mean, std, geom, rel_max=rel_max)
    net = lib.ImportanceNetwork(max_rows=max(len(target), geom.n_mesh * geom.n_groups), seed=seed)
    try:
        net.set_data(x4, target, weight)
        t0 = time.perf_counter()
        loss = net.train(steps, lr=lr)
        wall = time.perf_counter() - t0
        ms = net.last_train_ms()
        pred = net.predict(feats.inputs()).astype(np.float64) * feats.sigma + feats.mu
    finally:
        net.close()
    lower, upper = bounds_from_log_flux(pred, geom, ratio, scored=scored_bins(mean, std, geom, rel_max))
    return Result(lower, upper, loss, ms, len(target),
                  {"train_wall_s": wall, "mu": feats.mu, "sigma": feats.sigma, "log_flux": pred})


def geometry_of(mesh, energy_bounds):
    """MeshGeometry of an ``openmc_gb300.model.RegularMesh``."""
    return MeshGeometry(np.asarray(mesh.lower_left, float), np.asarray(mesh.upper_right, float),
                        tuple(mesh.dimension), np.asarray(energy_bounds, float))
