"""Full-scale case: the 17x17 lattice inside a 100 cm layered shield, 68
synthetic nuclides, a 100 x 100 x 60 mesh x 50 energy-bin flux tally (3e7
FP64 bins), FP32 tables with learned weight windows, judged against plain
transport with FP64 tables on the same GPU.

By default plain transport with FP32 tables runs against plain transport
with FP64 tables.  With --learned-particles, a plain FP32 pilot fills a
coarse window-mesh flux tally, the importance network is fitted to it
(``learned_ww.fit``; with --magic, OpenMC's MAGIC generator runs on it
instead), and a run with those windows (FP32 tables, split-to-slots)
replaces the plain FP32 run; the windowed run may use fewer
histories per batch, the figures of merit being per unit device time.
Windows normalised like MAGIC's ask for the same particle density in every
bin, which around a 100 cm shield (100x the core's volume, flux falling
~100x per layer) multiplies the tracked population beyond the split ring;
a detector-targeted importance is the next step for this case.
Reported: particles/s of both, the agreement of
the 3e7-bin tally (share of bins scored by both within 3 combined sigma, and
the same over the bins both runs converged to 10 % relative error), and the
flux, figure of merit 1/(R^2 T) and |z| (where both runs score) of every
shell along the x slab through the lattice.

``python -m openmc_gb300.full_scale_study`` prints one JSON object.
"""
from __future__ import annotations

import argparse
import json
import sys
import time
from pathlib import Path

import numpy as np

from . import configs, learned_ww, lib

GROUPS = [0.0, 1.0, 1.0e3, 1.0e5, 2.0e7 * 1.000001]


def _run(particles, batches, windows_on, fp32, log):
    lib.settings.particles = int(particles)
    lib.settings.weight_windows_on = bool(windows_on)
    lib.settings.xs_fp32 = 1 if fp32 else 0
    lib.simulation_init()
    dev_ms = 0.0
    events = 0
    for b in range(batches):
        lib.next_batch()
        lb = lib.last_batch()
        dev_ms += lb["ms"]
        events += lb["events"]
        print(f"{log} batch {b + 1}: {lb['ms']:.0f} ms, {lb['events']:.3g} events", file=sys.stderr, flush=True)
    ids = lib.tally_ids()
    res = [lib.tally_mean_std(t) for t in ids]
    lib.simulation_finalize()
    return {"device_s": dev_ms * 1e-3, "events": events, "tallies": res}


def agreement(a, b, converged_rel=0.1):
    """Bin-by-bin agreement of tally a with tally b, each (mean, std of the
    mean): share of the bins scored by both within 3 combined sigma and the
    largest |z|; the same over the bins both converged to converged_rel
    relative error (where the batch estimates of sigma are themselves
    reliable), with the mean signed z and the shares beyond +3 and -3 sigma
    (a bias of a shows as a shifted mean and a one-sided excess)."""
    ma, sa = (np.asarray(x, float).ravel() for x in a)
    mb, sb = (np.asarray(x, float).ravel() for x in b)
    both = (sa > 0) & (sb > 0)
    z = np.abs(ma - mb)[both] / np.hypot(sa, sb)[both]
    conv = both & (sa < converged_rel * np.abs(ma)) & (sb < converged_rel * np.abs(mb))
    zs = (ma - mb)[conv] / np.hypot(sa, sb)[conv]
    zc = np.abs(zs)
    return {"bins": int(ma.size), "scored_by_both": int(both.sum()),
            "share_within_3_sigma": float((z <= 3).mean()) if z.size else None,
            "max_z": float(z.max()) if z.size else None,
            "converged_by_both": int(conv.sum()),
            "converged_share_within_3_sigma": float((zc <= 3).mean()) if zc.size else None,
            "converged_max_z": float(zc.max()) if zc.size else None,
            "converged_mean_signed_z": float(zs.mean()) if zs.size else None,
            "converged_share_above_3_sigma": float((zs > 3).mean()) if zs.size else None,
            "converged_share_below_3_sigma": float((zs < -3).mean()) if zs.size else None}


def run(directory, particles=100_000_000, batches=3, pilot_particles=10_000_000, pilot_batches=2,
        steps=2000, n_points=11303, ww_mesh_dim=(44, 44, 10), learned_particles=0, magic=False):
    m, path = configs.full_scale(directory, particles=particles, batches=100_000, n_points=n_points,
                                 ww_mesh_dim=ww_mesh_dim, ww_groups=GROUPS)
    m.export_to_model_xml(path)
    wmesh = m.tallies[2].filters[0].mesh
    geom = learned_ww.geometry_of(wmesh, GROUPS)
    out = {"workload": "17x17 lattice in a 100 cm layered shield, 68 nuclides, "
                       "flux 100x100x60 mesh x 50 E bins (3e7 bins)",
           "batches": batches, "particles_per_batch": particles}
    lib.init(directory=path)
    saved = (lib.settings.xs_fp32, lib.settings.split_to_slots, lib.settings.secondary_capacity)
    try:
        lib.settings.split_to_slots = 1
        if learned_particles:
            # uniform particle density over the shells: give the split ring room
            lib.settings.secondary_capacity = 1 << 26
        if learned_particles:
            pilot = _run(pilot_particles, pilot_batches, False, True, "pilot")
            if magic:
                # OpenMC's own generator on the same pilot tally
                lib.WeightWindows(0).update_magic(lib.tally_index(lib.tally_ids()[2]), "mean", 1.0, 5.0)
                out["magic_window_bins"] = int((lib.WeightWindows(0).bounds[0] > 0).sum())
                first_name = "magic_fp32"
            else:
                mean, std = pilot["tallies"][2][0][:, 0], pilot["tallies"][2][1][:, 0]
                fit = learned_ww.fit(mean, std, geom, steps=steps)
                out["learned_fit"] = {"pairs": fit.n_pairs, "loss_first": float(fit.loss[0]),
                                      "loss_last": float(fit.loss[-1]), "train_ms": fit.train_ms}
                lib.WeightWindows(0).bounds = (fit.lower, fit.upper)
                first_name = "learned_fp32"
            lp = learned_particles
            first = _run(lp, batches, True, True, first_name.replace("_", " "))
        else:
            lp = particles
            first = _run(lp, batches, False, True, "plain fp32")
            first_name = "plain_fp32"
        plain = _run(particles, batches, False, False, "plain fp64")
    finally:
        lib.settings.xs_fp32, lib.settings.split_to_slots, lib.settings.secondary_capacity = saved
        lib.finalize()
    learned = first
    out["compared"] = f"{first_name} against plain_fp64"
    for name, r, n in ((first_name, first, lp), ("plain_fp64", plain, particles)):
        out[name] = {"particles_per_batch": n, "device_s": r["device_s"], "events": r["events"],
                     "particles_per_s": n * batches / r["device_s"]}
    # agreement of the 3e7-bin assembly tally
    out["assembly_tally"] = agreement(learned["tallies"][0], plain["tallies"][0])
    # flux and FOM per shell along the x slab
    (la, lsa), (lb_, lsb) = learned["tallies"][1], plain["tallies"][1]
    la, lsa, lb_, lsb = la.ravel(), lsa.ravel(), lb_.ravel(), lsb.ravel()

    def fom(mv, sv, t):
        return [1.0 / ((s / v) ** 2 * t) if v > 0 and s > 0 else 0.0 for v, s in zip(mv, sv)]

    fa, fb = fom(la, lsa, learned["device_s"]), fom(lb_, lsb, plain["device_s"])
    out["slab"] = {"learned_mean": la.tolist(), "plain_mean": lb_.tolist(),
                   "learned_fom": fa, "plain_fom": fb,
                   "fom_gain": [a / b if b > 0 else None for a, b in zip(fa, fb)],
                   "z": [abs(a - b) / np.hypot(c, d) if c > 0 and d > 0 else None
                         for a, b, c, d in zip(la, lb_, lsa, lsb)]}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--dir", default="_models/full_scale")
    ap.add_argument("--particles", type=int, default=100_000_000)
    ap.add_argument("--batches", type=int, default=3)
    ap.add_argument("--pilot-particles", type=int, default=10_000_000)
    ap.add_argument("--pilot-batches", type=int, default=2)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--learned-particles", type=int, default=0,
                    help="run learned windows (FP32) with this many histories per batch against plain FP64; "
                         "default: plain FP32 against plain FP64")
    ap.add_argument("--magic", action="store_true",
                    help="with --learned-particles: MAGIC windows from the same pilot instead of learned ones")
    a = ap.parse_args()
    out = run(Path(a.dir), particles=a.particles, batches=a.batches, pilot_particles=a.pilot_particles,
              pilot_batches=a.pilot_batches, steps=a.steps, learned_particles=a.learned_particles or None,
              magic=a.magic)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
