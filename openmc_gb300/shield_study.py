"""Figure of merit on the deep-penetration shield: no weight windows, MAGIC
windows, and learned windows from the importance network.

Workload: 200 x 50 x 50 cm stack of alternating 10 cm light-scatterer /
heavy-absorber layers, 1 MeV monodirectional plane source at x = 0, flux on a
200 x 10 x 10 mesh x energy groups, back-face flux over the last 10 cm and
the flux of every layer (for the figure of merit against depth).
Pilot: 5 batches of 10^6 histories without windows.  MAGIC windows come from
``openmc_weight_windows_update_magic`` on the pilot flux tally (threshold 1,
ratio 5: the defaults of WeightWindowsGenerator, weight_windows.h:205-208);
learned windows from ``learned_ww.fit`` on the same tally (2,000 Adam
steps).  Each method then runs the same number of batches; its figure of
merit is 1 / (R^2 T) with R the back-face tally's relative error and T the
device time of the measured batches (docs variance_reduction.rst:132-134).
Split particles run in free slots of their own (split-to-slots mode) unless
--serial-splits keeps the reference's per-history stack.

``python -m openmc_gb300.shield_study`` prints one JSON object.
"""
from __future__ import annotations

import argparse
import json
import sys
import time
from pathlib import Path

import numpy as np

from . import configs, learned_ww, lib
from . import model as om

GROUPS = [0.0, 1.0, 1.0e2, 1.0e4, 1.0e5, 1.0e6, 2.0e7 * 1.000001]


# Atom densities relative to the shield materials' base densities (0.1 and
# 0.085 atom/b-cm).  At the base densities the flux falls about 100x per
# 10 cm layer, so the back face of a 200 cm stack sees ~1e-40 of the source
# flux and no method scores there; at 0.1 it falls ~2x per layer (~1e-6 over
# 200 cm), where plain transport still scores a little at the back face.
DENSITY_SCALE = 0.1


def build(directory, length=200.0, mesh_dim=(200, 10, 10), n_points=11303, groups=GROUPS,
          density_scale=DENSITY_SCALE):
    m, path = configs.shield(directory, particles=1_000_000, batches=100_000, n_points=n_points,
                             length=length, mesh_dim=mesh_dim, energy_groups=groups,
                             tally_mesh_windows=True, density_scale=density_scale)
    m.export_to_model_xml(path)
    flux_mesh = m.tallies[0].filters[0].mesh
    return path, learned_ww.geometry_of(flux_mesh, groups)


def _run(particles, batches, windows_on, log=None):
    lib.settings.particles = int(particles)
    lib.settings.weight_windows_on = bool(windows_on)
    lib.simulation_init()
    dev_ms, wall = 0.0, time.perf_counter()
    events = secondaries = 0
    for b in range(batches):
        lib.next_batch()
        lb = lib.last_batch()
        dev_ms += lb["ms"]
        events += lb.get("events", 0)
        secondaries += lb.get("secondaries", 0)
        if log:
            print(f"{log} batch {b + 1}: {lb['ms']:.1f} ms, {lb['events']:.0f} events, "
                  f"longest history {lb['longest_events']:.0f} events", file=sys.stderr, flush=True)
    wall = time.perf_counter() - wall
    ids = lib.tally_ids()
    flux = lib.tally_mean_std(ids[0])
    back = lib.tally_mean_std(ids[1])
    layers = lib.tally_mean_std(ids[2])
    lib.simulation_finalize()
    return {"device_s": dev_ms * 1e-3, "wall_s": wall, "flux": flux, "back": back, "layers": layers,
            "events": events, "secondaries": secondaries}


def _fom(m, s, t):
    return 1.0 / ((s / m) ** 2 * t) if m > 0 and s > 0 else 0.0


def _fom_rel_unc(batches):
    """Relative standard uncertainty of a figure of merit 1/(R^2 T) whose R
    comes from `batches` batch means: R^2 is a sample variance over
    batches - 1 degrees of freedom, whose relative standard deviation is
    sqrt(2 / (batches - 1)) for normal batch means (heavier-tailed batch
    sums make it larger)."""
    return float(np.sqrt(2.0 / (batches - 1))) if batches > 1 else float("inf")


def _summary(r, batches, setup_s=0.0):
    m, s = float(r["back"][0].ravel()[0]), float(r["back"][1].ravel()[0])
    rel = s / m if m > 0 else float("inf")
    lm, ls = r["layers"][0].ravel(), r["layers"][1].ravel()
    return {"back_mean": m, "back_std": s, "rel_err": rel, "batches": batches, "device_s": r["device_s"],
            "wall_s": r["wall_s"], "fom": _fom(m, s, r["device_s"]), "fom_rel_unc": _fom_rel_unc(batches),
            "setup_s": setup_s, "fom_with_setup": _fom(m, s, r["device_s"] + setup_s),
            "events": r["events"], "secondaries": r["secondaries"],
            "layer_mean": lm.tolist(), "layer_std": ls.tolist(),
            "layer_fom": [_fom(a, b, r["device_s"]) for a, b in zip(lm, ls)]}


def run(directory, length=200.0, mesh_dim=(200, 10, 10), n_points=11303, pilot_particles=1_000_000,
        pilot_batches=5, particles=1_000_000, batches=10, steps=2000, lr=2e-3, ratio=5.0, fp32=True,
        methods=("plain", "magic", "learned"), density_scale=DENSITY_SCALE, verbose=False,
        split_to_slots=True, plain_batches=None):
    """plain_batches: batches of the plain arm (default `batches`); its back-
    face estimate needs many more histories than the windowed arms' for a
    comparable relative error, and the figure of merit does not depend on
    the run length.  Each method's figure of merit is reported with its
    relative uncertainty, and also with T including the setup the method
    needs (the pilot run for MAGIC and learned windows, plus the network's
    training for the learned ones)."""
    plain_batches = plain_batches or batches
    path, geom = build(directory, length, mesh_dim, n_points, density_scale=density_scale)
    out = {"workload": f"shield {length:g} cm, mesh {mesh_dim}, {geom.n_groups} energy groups, "
                       f"densities x {density_scale:g}",
           "split_to_slots": bool(split_to_slots),
           "pilot": f"{pilot_batches} x {pilot_particles}", "measure": f"{batches} x {particles}",
           "measure_plain": f"{plain_batches} x {particles}"}
    lib.init(directory=path)
    saved = (lib.settings.xs_fp32, lib.settings.split_to_slots)
    try:
        lib.settings.xs_fp32 = 1 if fp32 else 0
        lib.settings.split_to_slots = 1 if split_to_slots else 0
        ww = lib.WeightWindows(0)
        off = -np.ones(geom.n_mesh * geom.n_groups)
        pilot = _run(pilot_particles, pilot_batches, windows_on=False, log="pilot" if verbose else None)
        mean, std = pilot["flux"][0][:, 0], pilot["flux"][1][:, 0]
        out["pilot_scored_bins"] = int((mean > 0).sum())
        bounds = {"plain": (off, off)}
        if "magic" in methods:
            ww.update_magic(lib.tally_index(lib.tally_ids()[0]), "mean", 1.0, ratio)
            bounds["magic"] = ww.bounds
            out["magic_window_bins"] = int((bounds["magic"][0] > 0).sum())
        if "learned" in methods:
            fit = learned_ww.fit(mean, std, geom, steps=steps, lr=lr, ratio=ratio)
            bounds["learned"] = (fit.lower, fit.upper)
            out["learned"] = {"pairs": fit.n_pairs, "loss_first": float(fit.loss[0]),
                              "loss_last": float(fit.loss[-1]), "train_ms": fit.train_ms,
                              "steps": steps}
        setup = {"plain": 0.0, "magic": pilot["device_s"],
                 "learned": pilot["device_s"] + (out["learned"]["train_ms"] * 1e-3 if "learned" in out else 0.0)}
        out["pilot_device_s"] = pilot["device_s"]
        res = {}
        for name in methods:
            ww.bounds = bounds[name]
            nb = plain_batches if name == "plain" else batches
            r = _run(particles, nb, windows_on=(name != "plain"), log=name if verbose else None)
            res[name] = r
            out[name] = {**out.get(name, {}), **_summary(r, nb, setup[name])}
    finally:
        lib.settings.xs_fp32, lib.settings.split_to_slots = saved
        lib.finalize()
    base = out["plain"]["fom"] if "plain" in out else 0.0
    for name in methods:
        if name != "plain" and base > 0:
            out[name]["fom_gain"] = out[name]["fom"] / base
            out[name]["fom_gain_rel_unc"] = float(np.hypot(out[name]["fom_rel_unc"], out["plain"]["fom_rel_unc"]))
            out[name]["fom_gain_with_setup"] = out[name]["fom_with_setup"] / base
        if name != "plain" and "plain" in out:
            out[name]["layer_fom_gain"] = [a / b if b > 0 else None
                                           for a, b in zip(out[name]["layer_fom"], out["plain"]["layer_fom"])]
    # agreement of the back-face means (combined sigma)
    for a in methods:
        for b in methods:
            if a < b:
                sa, sb = out[a], out[b]
                sig = np.hypot(sa["back_std"], sb["back_std"])
                out[f"z_{a}_{b}"] = abs(sa["back_mean"] - sb["back_mean"]) / sig if sig > 0 else None
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--dir", default="_models/shield_study")
    ap.add_argument("--length", type=float, default=200.0)
    ap.add_argument("--pilot-particles", type=int, default=1_000_000)
    ap.add_argument("--pilot-batches", type=int, default=5)
    ap.add_argument("--particles", type=int, default=1_000_000)
    ap.add_argument("--batches", type=int, default=10)
    ap.add_argument("--plain-batches", type=int, default=0, help="batches of the plain arm (default: --batches)")
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--fp64", action="store_true")
    ap.add_argument("--density-scale", type=float, default=DENSITY_SCALE)
    ap.add_argument("--methods", default="plain,magic,learned")
    ap.add_argument("-v", "--verbose", action="store_true")
    ap.add_argument("--serial-splits", action="store_true",
                    help="bank split particles on the parent's stack (the reference's order)")
    a = ap.parse_args()
    out = run(Path(a.dir), length=a.length, mesh_dim=(int(a.length), 10, 10),
              pilot_particles=a.pilot_particles, pilot_batches=a.pilot_batches, particles=a.particles,
              batches=a.batches, steps=a.steps, fp32=not a.fp64, density_scale=a.density_scale,
              methods=tuple(a.methods.split(",")), verbose=a.verbose, split_to_slots=not a.serial_splits,
              plain_batches=a.plain_batches or None)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
