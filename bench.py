"""Benchmark of the event-based transport path on one GB300.

Workload: the full-size 17x17 pin lattice (pitch 1.26 cm, pin r=0.41 cm,
clad r=0.475 cm, 200 cm tall, reflective radial / vacuum axial boundaries;
3 materials from 12 synthetic nuclides of 11,303 grid points; Maxwellian
1.3 MeV source uniform in the pins; track-length flux on a 17x17x50 mesh x
100 log-energy bins).  One step = one batch of 10^7 histories with FP32
cross-section tables (FP64 geometry, stored energies and directions, search
keys and tally sums; the elastic-scatter kinematics and the track-length
tally's mesh walk in FP32).
Seeded synthetic nuclides stand in for evaluated data (none exists here).

Metric: particles/s = histories per batch / batch time (the reference's
"Calculation Rate (active)", src/output.cpp:460-490).  `value` is timed on
the device (CUDA events around the batch graph), with L2 flushed between
steps; `e2e` is the same metric through the C API (openmc_next_batch +
openmc_tally_results copying the tally arrays to host) on the host clock.

--impl reference times the reference algorithm's CPU implementation (the
oracle's restatement of OpenMC's event-based loop, OpenMP over all host
cores) on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "particles/s (event-based transport, 17x17 lattice, FP32 XS tables)"
WORKLOAD = "17x17 pin lattice, 12 nuclides x 11303 pts, flux 17x17x50 mesh x 100 E bins"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--particles", type=int, default=10_000_000)
    ap.add_argument("--in-flight", type=int, default=0,
                    help="particle slots held on the device (0: the library's default, 3 x 2^20)")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64-table extra measurement")
    ap.add_argument("--fp64-batches", type=int, default=20,
                    help="batches of the FP64-table run whose tally the FP32 tally is compared with")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-sample", type=int, default=0,
                    help="histories in the CPU baseline sample (default 3,000,000: about 10 s on 16 cores)")
    ap.add_argument("--no-xs-bench", action="store_true", help="skip the XS-lookup microbenchmark extra")
    ap.add_argument("--no-network-bench", action="store_true", help="skip the importance-network extra")
    ap.add_argument("--no-shield", action="store_true",
                    help="skip the shield figure-of-merit extra (plain, MAGIC and learned windows)")
    ap.add_argument("--network-only", action="store_true",
                    help="only time the importance network's training kernels (for kernel profilers)")
    ap.add_argument("--precision-only", type=int, default=0, metavar="BATCHES",
                    help="only compare FP32 with FP64 tables on the lattice: BATCHES batches each on "
                         "independent seeds, beside two FP64 runs on independent seeds as the control")
    ap.add_argument("--no-contract", action="store_true",
                    help="FP32-table mode on the transport build with separately rounded FP64 multiplies "
                         "and adds (default: the build with fused multiply-adds)")
    ap.add_argument("--no-defer", action="store_true",
                    help="score track-length tallies inside the advance kernel instead of from track records")
    ap.add_argument("--fuse", type=int, default=-1,
                    help="events run inside the advance kernel: 1 cross sections, 3 cross sections and "
                         "surface crossings (default: the library's choice)")
    ap.add_argument("--no-graph", action="store_true",
                    help="launch every batch kernel by kernel instead of as one CUDA graph "
                         "(for kernel profilers, which cannot see inside conditional graphs)")
    return ap.parse_args()


def mapped_libraries():
    """Shared libraries of this repository mapped into the process (Linux
    /proc/self/maps), relative to the repository root."""
    out = set()
    try:
        with open("/proc/self/maps") as f:
            for line in f:
                path = line.split()[-1] if line.strip() else ""
                if path.endswith(".so") and path.startswith(str(ROOT)):
                    out.add(str(Path(path).relative_to(ROOT)))
    except OSError:
        return None
    return sorted(out)


def config_of(args):
    """The workload, identical in both arms (each arm states its histories
    per step beside it)."""
    return {"workload": WORKLOAD, "xs_tables": "fp32 (reference arm: fp64)",
            "parallelism": f"{args.gpus} ranks, histories sharded by seed" if args.gpus > 1 else "single GPU"}


def model_dir(particles):
    from openmc_gb300 import configs
    d = ROOT / "_models" / f"lattice17_{particles}"
    xml = d / "model.xml"
    if not xml.exists():
        m, _ = configs.lattice17(d, particles=particles, batches=1000)
        m.export_to_model_xml(d)
    return d


class ClockSampler:
    """nvidia-smi samples during the timed region (clocks, throttle reasons)."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu=0):
        self.gpu = gpu
        self.samples = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except FileNotFoundError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([v.strip() for v in line.split(",")])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in self.samples:
            try:
                sm.append(float(s[0]))
                mx = float(s[1])
                for k, n in enumerate(names):
                    if s[3 + k].lower().startswith("active"):
                        reasons.add(n)
            except (ValueError, IndexError):
                pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def flush_l2(buf):
    import torch
    buf.add_(1)  # writes 512 MB (> 129 MB L2)
    torch.cuda.synchronize()


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per algorithmic
# byte of each kernel, from an ncu capture of one launch of the same kernel
# (iteration 20 of the 10^7-history lattice batch at the default 3,145,728
# slots, whose bank outgrows the L2; particle bank packed into per-slot
# records), matched with that launch's OPENMC_GB300_LAUNCH_LOG counts; the
# unfused kernels' ratios come from a
# capture of the unfused kernels of the unpacked bank.  Traffic per launch
# scales with the events a launch processes.  The track-length tally kernel
# reads the 96-byte track records, traffic of this design beyond its 16
# algorithmic bytes per mesh segment.
TRAFFIC_PER_ALGORITHMIC_BYTE = {"xs+advance+surface": 1.934, "xs+advance": 1.376, "surface": 1.406,
                                "collision": 2.736, "tally": 5.66}

# What bounds the transport kernels instead of HBM: the FP64 pipe's busy
# fraction in the same captures (a committed profile, not measured by this run).
_CAPTURE = "ncu --metrics, iteration 20 of the 1e7-history lattice batch, 3,145,728 slots"
FP64_PIPE_NOTE = {
    "xs+advance+surface": {"fp64_pipe_busy": 0.598, "dram_busy": 0.303, "source": _CAPTURE},
    "collision": {"fp64_pipe_busy": 0.524, "dram_busy": 0.288, "source": _CAPTURE},
    "tally": {"fp64_pipe_busy": 0.651, "dram_busy": 0.122, "source": _CAPTURE},
}


def algorithmic_bytes(detail, levels, fp32, deferred=True):
    """Bytes each kernel must move per batch: the particle-state fields
    an event reads and writes, the table bytes of each nuclide lookup (two
    hash-window bounds, two bracketing energies, two table rows, nuclide
    index, atom density) and 16 B of tally read-modify-write per mesh
    segment (in the track-length tally kernel when scoring is deferred, else
    in the advance kernel; the track records that carry a flight from one
    kernel to the other are traffic of this design, not algorithmic bytes).
    The tail kernel moves the bytes of every event it runs."""
    row = 16 if fp32 else 32
    dens = 4 if fp32 else 8
    per_nuc = 8 + 16 + 2 * row + 4 + dens

    def parts(st):
        return {
            "xs": st["xs_events"] * 36 + st["xs_calc"] * 16 + st["xs_nuclide_lookups"] * per_nuc,
            "advance": st["xs_events"] * (136 + 72 * levels),
            "tally": st["mesh_segments"] * 16,
            "surface": st["surface"] * (120 + 96 * levels),
            "collision": st["collision"] * 128 + st["collision_nuclide_lookups"] * per_nuc,
        }
    q = parts(detail["queue"])
    q["tail"] = sum(parts(detail["tail"]).values())
    if not deferred:
        # scored inside the advance kernel
        q["advance"] += q.pop("tally")
    q["xs+advance"] = q["xs"] + q["advance"]
    q["xs+advance+surface"] = q["xs"] + q["advance"] + q["surface"]
    return q


def run_gb300(args, barrier=lambda: None, rank=0):
    import torch
    from openmc_gb300 import lib
    path = model_dir(args.particles)
    n = args.particles
    out = {}
    lib.init(directory=path)
    try:
        # ranks shard the histories: each rank runs its own random streams
        lib.settings.seed = 1 + rank
        lib.settings.xs_fp32 = 1
        lib.settings.contract = 0 if args.no_contract else 1
        lib.settings.defer_tally = 0 if args.no_defer else 1
        lib.settings.particles_in_flight = args.in_flight
        if args.fuse >= 0:
            lib.settings.fuse_xs = args.fuse
        fused = int(lib.settings.fuse_xs)
        sort = int(lib.settings.sort_queue)
        if args.no_graph:
            lib.settings.profile_next = 2
        lib.simulation_init()
        tid = lib.tally_ids()[0]
        flush = torch.zeros(64 * 1024 * 1024, dtype=torch.float64, device="cuda")
        for _ in range(args.warmup):
            lib.next_batch()
        clocks = ClockSampler()
        dev_ms, wall, iters = [], [], []
        d2h = 0
        torch.cuda.synchronize()
        barrier()
        clocks.start()
        for _ in range(args.steps):
            flush_l2(flush)
            t0 = time.perf_counter()
            lib.next_batch()
            res = lib.tally_results(tid)
            t1 = time.perf_counter()
            d2h = res.nbytes + 256
            lb = lib.last_batch()
            dev_ms.append(lb["ms"])
            iters.append(lb["iterations"])
            wall.append(t1 - t0)
        torch.cuda.synchronize()
        barrier()
        clk = clocks.stop()
        detail_timed = lib.last_batch_detail()
        # profiled batch (kernel by kernel, CUDA events) for the roofline
        flush_l2(flush)
        if not args.no_graph:
            lib.settings.profile_next = 1
        lib.next_batch()
        prof = lib.last_batch_detail()
        levels = 2
        lib.simulation_finalize()
        fp32_tally = lib.tally_mean_std(tid)
        fp32_n = lib.tally_n_realizations(tid)
    finally:
        lib.finalize()
    total_ms = sum(dev_ms)
    value = args.steps * n / (total_ms / 1000.0)
    e2e = args.steps * n / sum(wall)
    kms = prof["kernel_ms"]
    byts = algorithmic_bytes(prof, levels, True, deferred=not args.no_defer)
    kms = dict(kms)
    # fused events run inside the advance kernel; their own spans only time event records
    if fused & 2:
        kms["xs+advance+surface"] = kms.pop("advance")
        kms.pop("xs")
        kms.pop("surface")
    elif fused & 1:
        kms["xs+advance"] = kms.pop("advance")
        kms.pop("xs")
    dom = max((k for k in ("xs", "advance", "xs+advance", "xs+advance+surface", "surface", "collision", "tail")
               if k in kms),
              key=lambda k: kms[k])
    peak, peak_kind = peaks()
    achieved = byts[dom] / (kms[dom] * 1e-3) / 1e9
    # kernels per event iteration: advance, [xs], [surface], collision, tail,
    # refill plan, refill, sort (3) or queue copy (1), finish; plus batch init
    # and accumulate
    per_iter = 1 + (0 if fused & 1 else 1) + (0 if fused & 2 else 1) + 1 + 1 + 2 + (3 if sort else 1) + 1
    launches = sum(2 + per_iter * int(i) for i in iters)
    dom_launches = int(prof["iterations"]) if "iterations" in prof else int(iters[-1])
    alg_per_launch = byts[dom] / max(dom_launches, 1)
    ratio = TRAFFIC_PER_ALGORITHMIC_BYTE.get(dom)
    traffic = ratio * alg_per_launch if ratio else None
    table = {}
    for k, ms in kms.items():
        if k in byts and ms > 0:
            gbs = byts[k] / (ms * 1e-3) / 1e9
            table[k] = {"ms": ms, "alg_bytes": byts[k], "GB/s": gbs, "frac": gbs / peak}
        else:
            table[k] = {"ms": ms}
    out.update(value=value, ms_per_step=total_ms / args.steps, e2e=e2e, e2e_d2h=d2h, clocks=clk,
               launches=launches, dominant=dom, achieved=achieved, peak=peak, peak_kind=peak_kind,
               traffic=traffic, alg_per_launch=alg_per_launch, dom_launches=dom_launches, kernel_table=table,
               kernel_ms=kms, bytes=byts, detail=detail_timed, profile=prof, iterations=iters)
    if not args.no_fp64:
        lib.init(directory=path)
        try:
            lib.settings.xs_fp32 = 0
            # its own random streams: the two tallies are then independent
            # estimates, so that each bin's z follows the t law the
            # comparison's expected shares assume (with shared seeds the
            # runs are correlated and the z values come out smaller)
            lib.settings.seed = 1001 + rank
            lib.settings.particles_in_flight = args.in_flight
            lib.simulation_init()
            # as many batches as the FP32 tally holds at least (warm-up +
            # timed + profiled), so that both sigmas have the same degrees
            # of freedom
            n64 = max(args.fp64_batches, 2)
            for _ in range(n64 - 1):
                lib.next_batch()
            flush_l2(flush)
            lib.next_batch()
            out["fp64_value"] = n / (lib.last_batch()["ms"] / 1000.0)
            lib.simulation_finalize()
            t64 = lib.tally_ids()[0]
            tally64, n64r = lib.tally_mean_std(t64), lib.tally_n_realizations(t64)
            out["fp32_vs_fp64"] = compare_tallies(fp32_tally, tally64, fp32_n, n64r)
            out["fp32_vs_fp64"]["seeds"] = {"fp32": 1 + rank, "fp64": 1001 + rank}
        finally:
            lib.finalize()
        # control: an FP64 run on a third seed with the FP32 run's batch count,
        # compared with the same FP64 tally.  Neighbouring bins share
        # histories, so statistics that treat bins as independent (the
        # converged-bin mean z and its 1/sqrt(count) error, the summed-flux z)
        # are read against this control, not against their nominal errors.
        lib.init(directory=path)
        try:
            lib.settings.xs_fp32 = 0
            lib.settings.seed = 2001 + rank
            lib.settings.particles_in_flight = args.in_flight
            lib.simulation_init()
            for _ in range(max(fp32_n, 2)):
                lib.next_batch()
            lib.simulation_finalize()
            tc = lib.tally_ids()[0]
            out["fp32_vs_fp64"]["control_fp64_vs_fp64"] = compare_tallies(
                lib.tally_mean_std(tc), tally64, lib.tally_n_realizations(tc), n64r)
            out["fp32_vs_fp64"]["control_fp64_vs_fp64"]["seeds"] = {"fp64_a": 2001 + rank, "fp64_b": 1001 + rank}
        finally:
            lib.finalize()
        # the same batch through the history-based kernel (settings.event_based = False)
        lib.init(directory=path)
        try:
            lib.settings.xs_fp32 = 1
            lib.settings.event_based = False
            lib.settings.particles_in_flight = args.in_flight
            lib.simulation_init()
            lib.next_batch()
            flush_l2(flush)
            lib.next_batch()
            out["history_value"] = n / (lib.last_batch()["ms"] / 1000.0)
            lib.simulation_finalize()
        finally:
            lib.settings.event_based = True
            lib.finalize()
    return out


def shield_fom():
    """The metric's second half: figure of merit 1/(R^2 T) of the back-face
    flux of the 200 cm deep-penetration shield (densities x 0.1, 200 x 10 x 10
    mesh x 6 energy groups) for plain transport (200 x 10^6 histories),
    MAGIC windows and learned windows from the same 5 x 10^6-history pilot
    (40 x 10^6 histories each), FP32 tables; T is the device time of the
    measured batches (and, in fom_with_setup, also of the pilot and the
    network's training).  Each figure of merit carries its relative
    uncertainty.  A failure here is reported in the line instead of ending
    the bench."""
    from openmc_gb300 import shield_study
    try:
        # the plain arm runs 200 batches, so that its back-face relative
        # error (0.43 after 10 batches) comes down to ~0.1; 40 batches of
        # each windowed arm bound its figure of merit to ~23 %
        r = shield_study.run(ROOT / "_models" / "shield_bench", batches=40, plain_batches=200)
    except Exception as e:  # the transport line above stands on its own
        return {"error": f"{type(e).__name__}: {e}"}
    out = {"workload": r["workload"], "pilot": r["pilot"], "measure": r["measure"],
           "measure_plain": r["measure_plain"], "pilot_device_s": r["pilot_device_s"]}
    keys = ("fom", "fom_rel_unc", "rel_err", "back_mean", "batches", "device_s", "setup_s", "fom_with_setup",
            "fom_gain", "fom_gain_rel_unc", "fom_gain_with_setup")
    for k in ("plain", "magic", "learned"):
        out[k] = {key: r[k][key] for key in keys if key in r[k]}
    out["z"] = {k: r[k] for k in ("z_magic_plain", "z_learned_plain", "z_learned_magic") if k in r}
    return out


def network_bench(rows=1 << 20, steps=20):
    """Training throughput of the importance network: full-batch Adam steps
    over `rows` random rows, with the fused per-tile kernel (the default) and
    with the layer-by-layer kernels.  FLOPs per step count the network's
    matrix products, independent of either kernel set's padding: forward
    2R(4x128 + 2x128x128 + 128), backward 2R(2x128x128 + 2x128x128 + 4x128
    + 128)."""
    from openmc_gb300 import lib
    rng = np.random.default_rng(3)
    x = rng.uniform(-1, 1, size=(rows, 4)).astype(np.float32)
    t = (x[:, 0] - 0.5 * x[:, 3]).astype(np.float32)
    flops = 2.0 * rows * ((4 * 128 + 2 * 128 * 128 + 128) + (4 * 128 * 128 + 4 * 128 + 128))
    peak, peak_src = 1900.0, "fallback"  # dense BF16 burst, one earlier GB300 measurement
    pk = ROOT / "MEASURED_PEAKS.json"
    if pk.exists() and json.loads(pk.read_text()).get("bf16_tflops"):
        peak, peak_src = float(json.loads(pk.read_text())["bf16_tflops"]), "measured"
    old = lib.settings.mlp_fused
    ms = {}
    try:
        for mode in (1, 0):
            lib.settings.mlp_fused = mode
            net = lib.ImportanceNetwork(max_rows=rows, seed=1)
            try:
                net.set_data(x, t)
                net.train(3, lr=1e-3)
                net.train(steps, lr=1e-3)
                ms[mode] = net.last_train_ms() / steps
            finally:
                net.close()
    finally:
        lib.settings.mlp_fused = old
    tflops = flops / (ms[1] * 1e-3) / 1e12
    return {"rows": rows, "steps": steps, "ms_per_step": ms[1], "tflops": tflops,
            "bf16_peak_tflops": peak, "peak_source": peak_src, "frac_of_bf16_peak": tflops / peak,
            "layer_by_layer_ms_per_step": ms[0], "layer_by_layer_tflops": flops / (ms[0] * 1e-3) / 1e12,
            "note": "fused: one persistent kernel per step keeps each 128-row tile's activations in shared "
                    "and tensor memory (one CTA per SM); layer-by-layer: one kernel per product, "
                    "activations through device memory"}


def compare_tallies(a, b, n_a, n_b):
    """FP32-table tally (a) against the FP64-table tally (b), both
    (mean, std of the mean) over n_a and n_b batches.

    Per bin scored by both runs, z = (mean_a - mean_b) / hypot(s_a, s_b).
    Each sigma is estimated from its batches, so z follows Student's t with
    the Welch-Satterthwaite degrees of freedom of the bin, not a normal law:
    the expected share beyond 3 (and the expected count beyond 5) is the
    mean over bins of that t law's two-sided tail, which the observed share
    is reported beside, with the equal-variance (pooled) t law's share as
    the lower bound of the expectation.  A bias of the FP32 tables would show as a signed-z
    mean away from 0 among the well-converged bins (nominal standard error
    1/sqrt(count), which holds for independent bins only: neighbouring mesh
    bins share histories, so the figure is read against an FP64-vs-FP64
    control of the same batch counts).  Per tally: the relative difference of the summed flux
    with its z, and the largest relative difference among bins both runs
    converged to 1 % relative error, with the largest combined relative
    error of those bins beside it."""
    ma, sa = (np.asarray(x, float).ravel() for x in a)
    mb, sb = (np.asarray(x, float).ravel() for x in b)
    both = (sa > 0) & (sb > 0)
    va, vb = sa[both] ** 2, sb[both] ** 2
    zs = (ma - mb)[both] / np.sqrt(va + vb)
    z = np.abs(zs)
    dof = (va + vb) ** 2 / (va ** 2 / max(n_a - 1, 1) + vb ** 2 / max(n_b - 1, 1))
    try:
        from scipy.stats import t as student_t
        exp3 = float(np.mean(2 * student_t.sf(3.0, dof)))
        # equal-variance bound: the pooled t law with n_a + n_b - 2 degrees of
        # freedom (lighter tails than the per-bin Welch estimate, which
        # over-predicts the tail when each sigma has few batches)
        exp3_pooled = float(2 * student_t.sf(3.0, n_a + n_b - 2))
        exp5 = float(np.sum(2 * student_t.sf(5.0, dof)))
        pval = 2 * student_t.sf(z, dof)
        # share of bins whose two-sided p-value is below 0.27 % (the 3-sigma
        # level of a normal law): uniform p-values give 0.0027
        p_share = float(np.mean(pval < 0.0027))
    except ImportError:
        exp3 = exp5 = p_share = exp3_pooled = None
    ta, tb = ma.sum(), mb.sum()
    st = np.sqrt((sa ** 2).sum() + (sb ** 2).sum())
    conv = both & (sa < 0.01 * np.abs(ma)) & (sb < 0.01 * np.abs(mb))
    rel = np.abs(ma - mb)[conv] / np.abs(mb)[conv]
    crel = np.hypot(sa, sb)[conv] / np.abs(mb)[conv]
    zc = (ma - mb)[conv] / np.hypot(sa, sb)[conv]
    return {"batches": [int(n_a), int(n_b)], "bins_scored_by_both": int(both.sum()),
            "share_within_3_sigma": float((z <= 3).mean()),
            "share_beyond_3_sigma": float((z > 3).mean()),
            "expected_share_beyond_3_sigma_t": exp3,
            "expected_share_beyond_3_sigma_pooled_t": exp3_pooled,
            "share_p_below_0.0027_t": p_share,
            "beyond_5_sigma": int((z > 5).sum()), "expected_beyond_5_sigma_t": exp5,
            "median_dof": float(np.median(dof)), "max_abs_z": float(z.max()),
            "mean_signed_z_all": float(zs.mean()),
            "converged_bins": int(conv.sum()),
            "mean_signed_z_converged": float(zc.mean()) if zc.size else None,
            "mean_signed_z_converged_stderr": float(1 / np.sqrt(zc.size)) if zc.size else None,
            "max_rel_diff_converged": float(rel.max()) if rel.size else None,
            "max_combined_rel_err_converged": float(crel.max()) if crel.size else None,
            "total_rel_diff": float((ta - tb) / tb),
            "total_z": float((ta - tb) / st) if st > 0 else None}


def xs_lookup_bench(fp32, n=17_000_000, reps=5):
    """Macroscopic-XS lookup microbenchmark: 68 nuclides x 11,303 points x 5
    channels, 12 materials, 1.7e7 (material, energy) lookups resident on the
    device, sorted by (material, energy) before the lookup kernel.  Returns
    lookups/s of the lookup kernel and of sort + lookup, and the kernel's
    algorithmic bytes per second: 12 B in + 40 B out per lookup and, per
    nuclide of the material, two hash-window bounds (8 B), two bracketing
    grid energies (16 B), two table rows (2 x 5 x 8 B, or x 4 B in FP32),
    the nuclide index (4 B) and its atom density (8 B, or 4 B)."""
    import torch
    from openmc_gb300 import data, lib
    d = data.make_xsbench()
    mats, e = data.xsbench_lookups(d, n, seed=11)
    counts = np.diff(np.asarray(d.mat_off))
    nuc_per_lookup = float(np.mean(counts[mats]))
    per_nuc = 8 + 16 + 2 * 5 * (4 if fp32 else 8) + 4 + (4 if fp32 else 8)
    alg = 52 + nuc_per_lookup * per_nuc
    t = lib.XSTables(d, fp32=fp32, max_lookups=n)
    dm = torch.from_numpy(mats).cuda()
    de = torch.from_numpy(e).cuda()
    do = torch.empty(n * 5, dtype=torch.float64, device="cuda")
    k_ms, tot_ms = [], []
    for r in range(reps + 2):
        t.lookup_device(n, dm.data_ptr(), de.data_ptr(), do.data_ptr(), None, sort=True)
        torch.cuda.synchronize()
        sort_ms, look_ms = t.last_times()
        if r >= 2:
            k_ms.append(look_ms)
            tot_ms.append(sort_ms + look_ms)
    t.close()
    head = do[:5 * 1_000_000].view(-1, 5).cpu().numpy()
    km, tm = statistics.median(k_ms), statistics.median(tot_ms)
    peak, kind = peaks()
    gbs = alg * n / (km * 1e-3) / 1e9
    return {"lookups_per_s": n / (km * 1e-3), "with_sort_lookups_per_s": n / (tm * 1e-3),
            "kernel_ms": km, "nuclides_per_lookup": nuc_per_lookup, "alg_bytes_per_lookup": alg,
            "GB/s": gbs, "frac_of_hbm_peak": gbs / peak,
            "note": "tables (37 MB FP64) stay in the 129 MB L2; inputs/outputs stream from HBM",
            "_head": head}


def cpu_baseline(path, sample, threads=None, mode=1):
    """Oracle transport of `sample` histories of batch 1 on the host cores,
    timing build (the reference's release flags): mode 1 = event-based loop
    (100,000 particles in flight, the reference's default
    max_particles_in_flight), mode 0 = history-based loop (the reference's
    default mode)."""
    import oracle
    o = oracle.Oracle(path / "model.xml", timing=True)
    threads = threads or os.cpu_count()
    t0 = time.perf_counter()
    o.transport(1, 1, sample, mode=mode, threads=threads, in_flight=100000 if mode == 1 else 0)
    dt = time.perf_counter() - t0
    return sample / dt, threads, dt


def precision_study(particles, batches):
    """FP32 against FP64 tables on the lattice flux tally, each run with
    `batches` batches on its own seeds, and two FP64 runs on independent
    seeds compared the same way: the FP32 comparison's statistics (share
    beyond 3 sigma, count beyond 5, mean signed z of converged bins, summed
    flux) are judged against what the control shows with no FP32 involved."""
    from openmc_gb300 import lib
    path = model_dir(particles)

    def run(fp32, seed):
        lib.init(directory=path)
        try:
            lib.settings.xs_fp32 = 1 if fp32 else 0
            lib.settings.seed = seed
            lib.simulation_init()
            for _ in range(batches):
                lib.next_batch()
            lib.simulation_finalize()
            t = lib.tally_ids()[0]
            return lib.tally_mean_std(t), lib.tally_n_realizations(t)
        finally:
            lib.finalize()

    a, na = run(True, 1)
    b, nb = run(False, 1001)
    c, nc = run(False, 2001)
    return {"workload": WORKLOAD, "histories_per_batch": particles, "batches": batches,
            "seeds": {"fp32": 1, "fp64": 1001, "fp64_control": 2001},
            "fp32_vs_fp64": compare_tallies(a, b, na, nb),
            "fp64_vs_fp64_control": compare_tallies(c, b, nc, nb)}


def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if rank == 0:
        if args.impl == "reference":
            # the CPU implementation only: the oracle's libraries, not this
            # package's CUDA library
            import oracle
            oracle.build()
        else:
            import __graft_entry__
            __graft_entry__.build()
        model_dir(args.particles)  # written once, before the other ranks read it
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        dist.barrier()
    if args.impl == "reference":
        if rank != 0:
            return
        path = model_dir(args.particles)
        sample = args.cpu_sample or 2_000_000
        cores = os.cpu_count()
        for _ in range(args.warmup):
            cpu_baseline(path, max(sample // 10, 1000), cores)
        t_all = 0.0
        for _ in range(args.steps):
            _, cores, dt = cpu_baseline(path, sample, cores)
            t_all += dt
        value = args.steps * sample / t_all
        # the reference's default mode, beside the event-based rate the ratio uses
        hist_sample = max(sample // 2, 1000)
        vh, _, dth = cpu_baseline(path, hist_sample, cores, mode=0)
        line = {"metric": METRIC, "value": value, "unit": "particles/s", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * t_all / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded nuclides, full-size model)", "impl": "reference",
                "config": config_of(args),
                "histories_per_step": sample,
                "sample_note": (f"each step transports {sample} of the workload's 10^7-history batch: "
                                f"a full batch takes ~30 s on the host cores, and the run must end "
                                f"within a few minutes; particles/s does not depend on the batch size here"),
                "ratio_mode": "event-based (the metric's loop); history-based beside it",
                "cpu_baseline": {"value": value, "unit": "particles/s", "cores": cores, "kind": "port",
                                 "build": "timing (reference release flags: -O2 -g -DNDEBUG, default FP contraction)",
                                 "sample": f"{sample} histories of batch 1 per step, event-based OpenMP loop",
                                 "history_based": {"value": vh, "unit": "particles/s",
                                                   "sample": f"{hist_sample} histories ({dth:.1f} s)"}},
                "e2e": {"value": value, "unit": "particles/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        line["libraries_mapped"] = mapped_libraries()
        print(json.dumps(line))
        return
    import torch
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    if args.network_only:
        print(json.dumps({"importance_network": network_bench(rows=args.particles, steps=args.steps)}))
        return
    if args.precision_only:
        print(json.dumps(precision_study(args.particles, args.precision_only)))
        return
    barrier = (lambda: None)
    if world > 1:
        import torch.distributed as dist
        barrier = dist.barrier
    r = run_gb300(args, barrier=barrier, rank=rank)
    if not args.no_network_bench and rank == 0:
        r["network"] = network_bench()
    if not args.no_shield and rank == 0:
        r["shield"] = shield_fom()
    if not args.no_xs_bench and rank == 0:
        x64, x32 = xs_lookup_bench(False), xs_lookup_bench(True)
        h64, h32 = x64.pop("_head"), x32.pop("_head")
        rel = np.abs(h32 - h64) / np.maximum(np.abs(h64), 1e-300)
        x32["max_rel_err_vs_fp64"] = {c: float(rel[:, k].max()) for k, c in
                                      enumerate(("total", "elastic", "absorption", "aux1", "aux2"))}
        r["xs_lookup"] = {"fp64": x64, "fp32": x32}
    if world > 1:
        import torch.distributed as dist
        # whole-job throughput over the slowest rank (device time and e2e wall time)
        t = torch.tensor([r["ms_per_step"], args.steps * args.particles / r["e2e"]], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        r["ms_per_step"] = float(t[0].item())
        r["value"] = world * args.particles / (r["ms_per_step"] / 1000.0)
        r["e2e"] = world * args.steps * args.particles / float(t[1].item())
    if rank != 0:
        return
    cpu = None
    if not args.no_cpu_baseline:
        path = model_dir(args.particles)
        sample = args.cpu_sample or 3_000_000
        v, cores, dt = cpu_baseline(path, sample)
        vh, _, dth = cpu_baseline(path, max(sample // 3, 1000), mode=0)
        cpu = {"value": v, "unit": "particles/s", "cores": cores, "kind": "port",
               "sample": f"{sample} histories of the same model, event-based loop, OpenMP ({dt:.1f} s)",
               "history_based": {"value": vh, "sample": f"{max(sample // 3, 1000)} histories ({dth:.1f} s)"}}
    line = {
        "metric": METRIC, "value": r["value"], "unit": "particles/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms_per_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32-xs/f64-geometry",
        "data": "synthetic (seeded nuclides, full-size model)",
        "config": config_of(args),
        "histories_per_step": args.particles,
        "l2": "flushed between steps (512 MB write)",
        "e2e": {"value": r["e2e"], "unit": "particles/s", "h2d_bytes_per_step": 256,
                "d2h_bytes_per_step": r["e2e_d2h"]},
        "gpu_launches": r["launches"],
        "clocks": r["clocks"],
        "roofline": {"bound": "hbm", "kernel": r["dominant"], "achieved": r["achieved"], "peak": r["peak"],
                     "unit": "GB/s", "frac": r["achieved"] / r["peak"], "peak_source": r["peak_kind"],
                     "traffic": r["traffic"], "alg_bytes_per_launch": r["alg_per_launch"],
                     "launches": r["dom_launches"],
                     "limiter": FP64_PIPE_NOTE.get(r["dominant"])},
        "kernels": r["kernel_table"],
        "cpu_baseline": cpu,
        "kernel_ms_profiled_batch": r["kernel_ms"],
        "fp64_xs_particles_per_s": r.get("fp64_value"),
        "fp32_vs_fp64_tally": r.get("fp32_vs_fp64"),
        "history_based_gpu_particles_per_s": r.get("history_value"),
        "events_per_step": r["detail"]["queue"]["xs_events"] + r["detail"]["tail"]["xs_events"],
        "iterations_per_step": r["iterations"],
        "xs_lookup_microbench": r.get("xs_lookup"),
        "importance_network_training": r.get("network"),
        "shield_fom": r.get("shield"),
    }
    print(json.dumps(line))


if __name__ == "__main__":
    main()
