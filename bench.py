#!/usr/bin/env python
"""Throughput of the FIB_MD hot path on GB300: atom-steps/s.

Workload (the single-cascade configuration): a diamond-cubic Si slab of
40 x 40 x 20 unit cells (256,000 Si, eight atoms per cubic unit cell) plus
one Ga ion at 5 keV, 7 degrees off normal, seeded azimuth and impact point
10 A above the surface; Maxwell-Boltzmann velocities at 300 K (seeded);
bottom 2 atomic layers fixed, next 4 Berendsen-thermostatted at 300 K;
variable dt = min(1 fs, 0.05 A / max|v|); lists rebuilt once the two largest
displacements since the last build add up to the skin.
Synthetic data, seeded (spec_slab, seed 2001).

One bench step = MD steps 1..`--md-steps` (default 5000) of that cascade,
from a fresh upload of the seeded initial state, through fibmd_gpu_steps.
`value` is the mixed-precision path (binary32 force arithmetic, binary64
accumulation/integration) with the upload, list build and first force
outside the timed region; `fp64` is the plain binary64 path on the same
window. L2 (129 MB) is flushed before every timed step. `e2e` times what a
host does per cascade through the C-ABI with pinned host buffers: upload of
the initial state -> tags -> si_nlist -> si_force -> steps -> download.

--impl reference times the CPU oracle (the binary64 restatement of the
reference's si_nlist/si_force with the spec-mode step, its force OpenMP over
all host cores) on a bounded sample of the same window of the same cascade,
set up from the oracle's restatements alone.
"""
from __future__ import annotations

import argparse
import csv
import io
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

KB = 1.381e-23
A_LAT = 5.431073e-10
METRIC = "atom-steps/s (256k-atom Si slab, 5 keV Ga cascade from the ion's start)"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--md-steps", type=int, default=5000,
                    help="MD steps of the cascade per bench step, from the ion's start")
    ap.add_argument("--cells", default="40,40,20")
    ap.add_argument("--fp64-steps", type=int, default=2,
                    help="timed bench steps of the binary64 arm (after one untimed)")
    ap.add_argument("--cpu-sample-steps", type=int, default=12,
                    help="spec-mode oracle steps of the CPU baseline's timed sample")
    ap.add_argument("--no-small-slab", action="store_true",
                    help="skip the 8x8x8-cell (4097-atom) slab's binary64 line beside the oracle")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--list-skin", type=float, default=-1.0,
                    help="spec-mode list skin in Angstrom; negative (the default): the "
                         "library's run-time tuning, which starts from 0.6 A and re-times "
                         "0.45, 0.6 and 0.81 A on the current state; 0: the reference's "
                         "list radii; positive: that start value (still tuned unless the "
                         "context's skin_tune option is 0). The oracle runs take the start "
                         "value (0.6 A for a negative one)")
    ap.add_argument("--reactions", type=int, default=0,
                    help="1: the mixed context's binary32 force path stores the 3-body "
                         "reactions and gathers them per atom instead of adding them by "
                         "binary64 atomics (the option 'reactions'; slower on GB300, for "
                         "comparison)")
    ap.add_argument("--no-graph", action="store_true",
                    help="run the step loop launch by launch (for a profiler's launch list)")
    ap.add_argument("--ensemble-replicas", type=int, default=256)
    ap.add_argument("--ensemble-steps", type=int, default=3000)
    ap.add_argument("--ensemble-plain-sample", type=int, default=3,
                    help="impacts run one by one in plain binary64 to time that form")
    ap.add_argument("--no-ensemble", action="store_true")
    ap.add_argument("--dose-impacts", type=int, default=10,
                    help="impacts of the cumulative-dose run (0: skip)")
    ap.add_argument("--dose-fp64-impacts", type=int, default=-1,
                    help="impacts of its binary64 counterpart (default: as many)")
    ap.add_argument("--dose-study", action="store_true",
                    help="run only the config-4 dose study (--dose-impacts mixed impacts on the "
                         "first seed, --dose-compare mixed and binary64 impacts on each of "
                         "--dose-seeds seeds) and print its JSON")
    ap.add_argument("--dose-compare", type=int, default=100)
    ap.add_argument("--dose-seeds", type=int, default=3)
    ap.add_argument("--dose-chunk", type=int, default=50)
    ap.add_argument("--large-steps", type=int, default=20000,
                    help="MD steps of the 1,048,577-atom 30 keV cascade (0: skip)")
    ap.add_argument("--profile", choices=["mixed", "fp64", "build", "step", "ensemble", "dose"],
                    default=None,
                    help="set up the workload, evaluate the force 3 times (mixed, fp64), "
                         "rebuild the lists 5 times (build), run the window's first "
                         "min(md-steps, 300) mixed steps launch by launch (step), run the 256-impact ensemble 1000 steps as "
                         "graphs and 20 launch by launch (ensemble), or run the dose slab's "
                         "first impact 300 steps as graphs and 20 launch by launch on the "
                         "8-lanes-per-centre force path (dose), exit (for ncu)")
    ap.add_argument("--profile-graph-steps", type=int, default=-1,
                    help="CUDA-graph steps before the launch-by-launch segment of the "
                         "ensemble and dose profiles (default 1000 and 300)")
    return ap.parse_args()


# ---------------------------------------------------------------------------
# workload
def _impact_xy(cells, centre):
    return (0.5 * A_LAT * cells[0], 0.5 * A_LAT * cells[1]) if centre else None


def _as_workload(params, X, V, Xi, mass, atype, tags):
    N = params.Natm
    return dict(params=params, X=X, V=V, Xi=Xi, mass=mass, atype=atype,
                xsides=np.zeros(N, dtype=np.int32), tags=tags)


def make_workload(cells, seed=2001, energy_eV=5000.0, polar_deg=7.0, list_skin_A=0.0,
                  centre=False):
    """The spec-mode cascade slab (fib_md_gb300.spec_slab): 300 K
    Maxwell-Boltzmann velocities, bottom 2 planes fixed, next 4
    thermostatted, the ion 10 A above the surface (at a seeded point, or the
    slab centre), atoms 35 A above the surface removed."""
    import fib_md_gb300 as fm

    p = fm.params_default()
    p.list_skin = list_skin_A * 1e-10
    s = fm.spec_slab(cells, seed, energy_eV, polar_deg, ion_height=10e-10,
                     remove_above=35e-10, params=p, impact_xy=_impact_xy(cells, centre))
    return _as_workload(s.params, s.X, s.V, s.Xi, s.mass, s.atype, s.tags)


def oracle_workload(cells, seed=2001, energy_eV=5000.0, polar_deg=7.0, list_skin_A=0.0,
                    centre=False):
    """The same slab from the oracle's restatements alone (oracle_ffi.spec_slab
    draws the same numbers in the same order): the reference arm and the CPU
    baseline load nothing of the GPU package."""
    sys.path.insert(0, str(ROOT / "tests"))
    import oracle_ffi as of

    p = of.params_default()
    p.list_skin = list_skin_A * 1e-10
    s = of.spec_slab(cells, seed, energy_eV, polar_deg, ion_height=10e-10,
                     remove_above=35e-10, params=p, impact_xy=_impact_xy(cells, centre))
    return _as_workload(s["params"], s["X"], s["V"], s["Xi"], s["mass"], s["atype"], s["tags"])


def fresh_state(g, w):
    """A cascade's start on context g: upload of the seeded initial state,
    tags, the ion fired, lists built, the first force."""
    g.upload(w["X"], w["V"], None, w["Xi"], w["mass"], w["atype"], w["xsides"])
    g.set_tags(w["tags"])
    g.set_impact(1)
    g.si_nlist()
    g.si_force()


def make_ctx(w, precision):
    import fib_md_gb300 as fm

    p = w["params"].copy()
    p.precision = precision
    g = fm.FibMD(p)
    fresh_state(g, w)
    return g


def skin_text(skin_A):
    if skin_A < 0:
        return "tuned at run time (start 0.6 A, candidates 0.45, 0.6, 0.81 A)"
    if skin_A == 0:
        return "reference radii"
    return f"tuned at run time (start {skin_A} A)"


def oracle_skin(skin_A):
    """The oracle's list skin (A): the start of the GPU run's tuning."""
    return 0.6 if skin_A < 0 else skin_A


def workload_config(args, cells, N):
    """The `config` object of both arms' JSON lines (static: what is run)."""
    return {
        "workload": f"Si slab {cells[0]}x{cells[1]}x{cells[2]} unit cells ({N - 1} Si + 1 Ga), "
                    "5 keV Ga at 7 deg, 10 A above the surface, 300 K, spec mode",
        "atoms": N,
        "window": f"MD steps 1-{args.md_steps} of the cascade from the ion's start; every "
                  "bench step starts from the seeded initial state",
        "md_steps_per_step": args.md_steps, "mode": "spec",
        "list_skin": skin_text(args.list_skin),
        "seed": 2001,
        "parallelism": "replicas (one cascade per GPU)",
        "l2": "flushed before every timed step",
    }


# ---------------------------------------------------------------------------
# clocks during the timed region
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.proc:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        rows = list(csv.reader(io.StringIO(getattr(self, "out", "") or "")))
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                mx = max(mx, float(r[2]))
            except ValueError:
                continue
            for k, name in enumerate(names):
                if r[5 + k].lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
def run_windows(g, w, torch, stream, steps, md_steps, flush):
    """`steps` bench steps on the device: each a fresh start of the cascade
    (untimed: upload, tags, lists, first force), an L2 flush, then MD steps
    1..md_steps timed with CUDA events on the library's stream. Returns the
    per-step seconds and the list rebuilds inside the timed steps."""
    times, rebuilds = [], 0
    for _ in range(steps):
        fresh_state(g, w)
        rb0 = g.work_counters()[4]
        flush.zero_()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        g.steps(2, md_steps, 0, 0.0, 300.0)
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1) * 1e-3)
        rebuilds += g.work_counters()[4] - rb0
    return times, rebuilds


def flops_per_force(counts):
    """Algorithmic flop model (+ - * / sqrt and exp count 1): 40 per active
    SW pair, 100 per non-zero angle term, 60 per Moliere pair, 100 per
    stale-list angle term."""
    pairs, angles, mol, stale = counts[:4]
    return 40 * pairs + 100 * angles + 60 * mol + 100 * stale


def tuning_chunks(md_steps):
    """Graph chunks of one call of md_steps steps right after an upload: the
    force path is re-timed 1000 steps after the upload and then after twice
    the last interval, up to 8000 steps, while its choice stands."""
    pairs, interval, n = md_steps // 2, 500, 0
    while pairs > 0:
        pairs -= min(pairs, interval)
        interval = min(2 * interval, 4000)
        n += 1
    return n


def replica_rate(dist, units, seconds, device):
    """Whole-job rate of independent replicas (one per rank, no data-path
    collective): the units all ranks processed over the slowest rank's
    time. Returns (rate, slowest time, total units)."""
    if dist is None:
        return units / seconds, seconds, units
    import torch

    t = torch.tensor([seconds], dtype=torch.float64, device=device)
    u = torch.tensor([units], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(u.item()) / float(t.item()), float(t.item()), float(u.item())


def bench_ours(args, rank, world, dist):
    import torch

    import fib_md_gb300 as fm

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    cells = tuple(int(x) for x in args.cells.split(","))
    w = make_workload(cells, list_skin_A=args.list_skin)
    N = w["params"].Natm
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    fp64_peak, fp32_peak = fm.md.pipe_peaks()

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    # ---- mixed precision (the headline); the step loop runs as CUDA graphs
    g = make_ctx(w, fm.PREC_MIXED)
    g.set_option("timers", 0)
    g.set_option("graph", 0 if args.no_graph else 1)
    g.set_option("reactions", args.reactions)
    stream = torch.cuda.ExternalStream(g.stream_ptr)
    run_windows(g, w, torch, stream, args.warmup, args.md_steps, flush)
    barrier()
    with ClockSampler(dev) as clk:
        w0 = time.perf_counter()
        times, rebuilds = run_windows(g, w, torch, stream, args.steps, args.md_steps, flush)
        barrier()
        wall = time.perf_counter() - w0
    stage_end = int(g.get_option("stage"))
    skin_end = g.get_option("skin")
    pdl_end = g.get_option("pdl") == 1.0
    blocks_end = {"force_block": int(g.get_option("force_block")),
                  "build_block": int(g.get_option("build_block"))}
    X_end, _, _ = g.download()
    value, t_dev, atom_steps = replica_rate(dist, float(N) * args.md_steps * args.steps,
                                            sum(times), "cuda")
    # the main force kernel, timed live with CUDA events on the library's
    # stream over the window's first steps run launch by launch (events
    # cannot sit inside the graph's conditional bodies), from a fresh start
    g.set_option("graph", 0)
    g.set_option("kernel_timing", 1)
    fresh_state(g, w)
    g.kernel_time(reset=True)
    g.steps(2, min(args.md_steps, 1000), 0, 0.0, 300.0)
    fk_total, fk_n = g.kernel_time(reset=True)
    g.set_option("kernel_timing", 0)
    g.set_option("graph", 0 if args.no_graph else 1)
    g.si_force()
    counts = g.work_counters()
    flops = flops_per_force(counts)
    fk_avg = fk_total / max(fk_n, 1)
    achieved = flops / fk_avg / 1e12

    # ---- end to end through the C-ABI with pinned host buffers: per step
    # the initial state goes up, the cascade runs, the final state comes down
    e2e = None
    if not args.no_e2e:
        import ctypes as C

        def pinned(shape, dtype=torch.float64):
            n = int(np.prod(shape))
            a = torch.empty(n, dtype=dtype, pin_memory=True).numpy()
            return a.reshape(shape[::-1]).T if len(shape) > 1 else a

        hX, hV, hXi = (pinned((N, 3)) for _ in range(3))
        hX[:], hV[:], hXi[:] = w["X"], w["V"], w["Xi"]
        hm = pinned((N,))
        hm[:] = w["mass"]
        ha = pinned((N,), torch.int32)
        ha[:] = w["atype"]
        hs = pinned((N,), torch.int32)
        hs[:] = w["xsides"]
        ht = pinned((N,), torch.int32)
        ht[:] = w["tags"].astype(np.int32)
        oX, oV, oF = (pinned((N, 3)) for _ in range(3))
        lib, h = g.lib, g.h
        dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
        ip = lambda a: a.ctypes.data_as(C.POINTER(C.c_int))
        tp = ht.ctypes.data_as(C.POINTER(C.c_uint32))

        def cascade():
            for rc in (lib.fibmd_gpu_upload(h, dp(hX), dp(hV), None, dp(hXi), dp(hm), ip(ha),
                                            ip(hs)),
                       lib.fibmd_gpu_set_tags(h, tp),
                       lib.fibmd_gpu_set_impact(h, 1),
                       lib.fibmd_gpu_nlist(h),
                       lib.fibmd_gpu_force(h, None, None, None)):
                g._check(rc, "e2e set-up")
            g.steps(2, args.md_steps, 0, 0.0, 300.0)
            g._check(lib.fibmd_gpu_download(h, dp(oX), dp(oV), dp(oF)), "e2e download")

        cascade()
        barrier()
        w0 = time.perf_counter()
        for _ in range(args.steps):
            cascade()
        barrier()
        t_e2e = time.perf_counter() - w0
        e2e_value, _, _ = replica_rate(dist, float(N) * args.md_steps * args.steps, t_e2e, "cuda")
        e2e = {"value": e2e_value, "unit": "atom-steps/s",
               "h2d_bytes_per_step": N * (3 * 24 + 8 + 4 + 4 + 4),
               "d2h_bytes_per_step": N * 3 * 24,
               "what": "per step: upload of the initial state (X, V, Xi, mass, atype, xsides) "
                       "and the tags from pinned host memory, si_nlist, si_force, the "
                       f"{args.md_steps} MD steps, download of X, V, F to pinned host memory"}
    g.close()

    # ---- plain binary64 on the same window
    g64 = make_ctx(w, fm.PREC_FP64)
    g64.set_option("timers", 0)
    s64 = torch.cuda.ExternalStream(g64.stream_ptr)
    n64 = max(1, args.fp64_steps)
    run_windows(g64, w, torch, s64, 1, args.md_steps, flush)
    barrier()
    t64, rb64 = run_windows(g64, w, torch, s64, n64, args.md_steps, flush)
    g64.set_option("graph", 0)
    g64.set_option("kernel_timing", 1)
    fresh_state(g64, w)
    g64.kernel_time(reset=True)
    g64.steps(2, min(args.md_steps, 200), 0, 0.0, 300.0)
    f64_total, f64_n = g64.kernel_time(reset=True)
    g64.si_force()
    c64 = g64.work_counters()
    g64.close()
    value64, _, _ = replica_rate(dist, float(N) * args.md_steps * n64, sum(t64), "cuda")
    f64_avg = f64_total / max(f64_n, 1)

    # HBM view of the whole step: 150 algorithmic bytes per atom-step
    step_bytes = 150.0 * N
    md_step_s = t_dev / (args.md_steps * args.steps)
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) \
        if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    traffic = None
    tr_file = ROOT / "profiles" / "force_kernel_traffic.txt"
    if tr_file.exists():
        # "key = value" lines written from an ncu capture of the same kernel
        kv = {}
        for line in tr_file.read_text().splitlines():
            if "=" in line and not line.lstrip().startswith("#"):
                k, v = line.split("=", 1)
                kv[k.strip()] = v.strip()
        bpa = float(kv.get("mixed_dram_bytes_per_atom", "0") or 0)
        if bpa > 0:
            traffic = bpa * N
        bpl = float(kv.get("mixed_dram_bytes_per_atom_in_loop", "0") or 0)
        traffic_loop = bpl * N if bpl > 0 else None
    else:
        traffic_loop = None
    out = {
        "metric": METRIC,
        "value": value,
        "unit": "atom-steps/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * t_dev / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 force arithmetic, f64 accumulation/positions/VV",
        "data": "synthetic (seeded)",
        "config": workload_config(args, cells, N),
        "step_loop": "launch by launch" if args.no_graph else
                     ("CUDA graph, kernels as programmatic dependents" if pdl_end else "CUDA graph"),
        "autotune": {"force_path": "1000 steps after the upload, then after doubling "
                                   "intervals, among 6 or 10 staged legs per thread (in blocks of 128 or 64) and 8 lanes per centre (1)",
                     "force_path_at_end": stage_end,
                     "force_reactions": "stored and gathered per atom" if args.reactions
                                        else "binary64 atomics",
                     "list_skin": skin_text(args.list_skin),
                     "list_skin_at_end_A": skin_end,
                     "atoms_per_block_at_end": blocks_end},
        "fp64": {"value": value64, "unit": "atom-steps/s", "steps": n64,
                 "window": "the same", "mixed_over_fp64": value / value64,
                 "ms_per_step": 1e3 * sum(t64) / n64,
                 "force_kernel_ms": 1e3 * f64_avg,
                 "rebuild_fraction": rb64 / float(args.md_steps * n64),
                 "roofline": {"bound": "fp64", "achieved": flops_per_force(c64) / f64_avg / 1e12,
                              "peak": fp64_peak, "unit": "TFLOP/s",
                              "frac": flops_per_force(c64) / f64_avg / 1e12 / fp64_peak,
                              "peak_source": "measured in this run (DFMA loop)"}},
        "roofline": {"bound": "fp32", "kernel": "k_force<mixed>", "achieved": achieved,
                     "peak": fp32_peak, "unit": "TFLOP/s", "frac": achieved / fp32_peak,
                     "traffic": traffic,
                     "traffic_in_loop": traffic_loop,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum per "
                                       "launch of this kernel on this slab "
                                       "(profiles/force_kernel_traffic.txt): 'traffic' with "
                                       "ncu's cache flush before the launch, 'traffic_in_loop' "
                                       "with the caches the step loop leaves",
                     "flops_per_launch": flops,
                     "bytes_per_launch_algorithmic": 56 * N,
                     "force_kernel_ms": 1e3 * fk_avg, "launches": fk_n,
                     "timed_over": f"the window's first {min(args.md_steps, 1000)} steps, "
                                   "launch by launch",
                     "peak_source": "measured in this run (FFMA loop)"},
        "roofline_hbm": {"bound": "hbm", "achieved": step_bytes / md_step_s / 1e9,
                         "peak": hbm_peak, "unit": "GB/s",
                         "frac": step_bytes / md_step_s / 1e9 / hbm_peak,
                         "bytes_per_atom_step": 150,
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs"},
        "mixed_error_vs_fp64": {
            **force_error(w, X_end),
            "nve_drift_eV_per_atom_per_ps": {"mixed": nve_drift(w, fm.PREC_MIXED),
                                             "fp64": nve_drift(w, fm.PREC_FP64)},
            "nve_segment": "1 ps (1000 steps at the 1 fs cap) of the same slab at 300 K, "
                           "ion held outside, thermostat off, fixed layers kept; drift = "
                           "slope of a line fitted to 11 samples of the total energy",
        },
        "work_counters": {"sw_pairs": counts[0], "angle_terms": counts[1],
                          "moliere_pairs": counts[2], "stale_terms": counts[3],
                          "many_leg_centres": counts[5]},
        # per MD step: drift, rebuild condition, force (main with the Moliere
        # blocks, many-leg; one kernel on the 8-lanes-per-centre path), kick,
        # kick reduction = 6; per step pair the loop control; 9 kernels per
        # list rebuild; the loop set-up per chunk between force-path tunings
        # (1000 steps after the upload, then doubling). Launch by launch:
        # the 9 list kernels every step (they return at once when no rebuild
        # is due), no condition or loop kernels
        "gpu_launches": int((14 if stage_end != 1 else 13) * args.md_steps * args.steps
                            if args.no_graph else
                            (6.5 if stage_end != 1 else 5.5) * args.md_steps * args.steps +
                            9 * rebuilds + args.steps * tuning_chunks(args.md_steps)),
        "rebuild_fraction": rebuilds / float(args.md_steps * args.steps),
        "wall_s_timed": wall,
        "clocks": clk.summary(),
    }
    if e2e:
        out["e2e"] = e2e
    return out


# ---------------------------------------------------------------------------
# binary64 flops of one spec-mode integration step per atom: the drift's
# c = dt^2/2m (1), x + v dt + c f (3 x 2 FMA = 12) and fixed-point shadow (3
# FMA = 6) and removal test (2); the kick's c = dt/2m (1), f + f' (3),
# v + c (f + f') (3 FMA = 6) and |v|^2 (5)
INTEGRATOR_FP64_FLOPS = 36


def bench_large(args):
    """The large single cascade: 64x64x32 unit cells (1,048,576 Si; diamond
    has 8 atoms per cell) and one 30 keV Ga at normal incidence on the slab
    centre, args.large_steps variable-dt steps in mixed precision through the
    CUDA-graph step loop, timed whole (cascade and all) with CUDA events."""
    import torch

    import fib_md_gb300 as fm

    w = make_workload((64, 64, 32), seed=5001, energy_eV=30000.0, polar_deg=0.0,
                      list_skin_A=args.list_skin, centre=True)
    N = w["params"].Natm
    fp64_peak, fp32_peak = fm.md.pipe_peaks()
    g = make_ctx(w, fm.PREC_MIXED)
    g.set_option("timers", 0)
    stream = torch.cuda.ExternalStream(g.stream_ptr)
    rb0 = g.work_counters()[4]
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        a.record(stream)
        _, t_sim, _, _ = g.steps(2, args.large_steps, 0, 0.0, 300.0)
        b.record(stream)
        torch.cuda.synchronize()
    secs = a.elapsed_time(b) / 1e3
    rebuilds = g.work_counters()[4] - rb0
    stage_end = int(g.get_option("stage"))
    skin_end = g.get_option("skin")
    # the main force kernel timed live over a launch-by-launch segment
    g.set_option("graph", 0)
    g.set_option("kernel_timing", 1)
    g.kernel_time(reset=True)
    g.steps(2, 100, 0, t_sim, 300.0)
    fk_total, fk_n = g.kernel_time(reset=True)
    g.si_force()
    counts = g.work_counters()
    g.close()
    fk = fk_total / max(fk_n, 1)
    f32 = flops_per_force(counts) / fk / 1e12
    rate = N * args.large_steps / secs
    f64 = INTEGRATOR_FP64_FLOPS * rate / 1e12
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) \
        if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    return {
        "config": "Si slab 64x64x32 unit cells (1,048,576 Si + 1 Ga), 30 keV Ga at normal "
                  f"incidence on the slab centre, {args.large_steps} variable-dt steps, "
                  "mixed precision, CUDA-graph step loop, list skin "
                  f"{skin_text(args.list_skin)}",
        "atoms": N, "md_steps": args.large_steps,
        "atom_steps_per_s": rate, "us_per_md_step": 1e6 * secs / args.large_steps,
        "simulated_ps": t_sim * 1e12,
        "rebuild_fraction": rebuilds / float(args.large_steps),
        "force_stage": "autotuned at doubling intervals from 1000 steps among 6 or 10 "
                       "staged legs per thread "
                       "and 8 lanes per centre (1); "
                       f"{stage_end} at the end",
        "list_skin_at_end_A": skin_end,
        "fp32_pipe": {"kernel": "k_force<mixed>", "achieved_tflops": f32, "peak_tflops": fp32_peak,
                      "frac": f32 / fp32_peak, "force_kernel_us": 1e6 * fk,
                      "peak_source": "measured in this run (FFMA loop)"},
        "fp64_pipe": {"what": "integration (drift + kick), INTEGRATOR_FP64_FLOPS per atom-step "
                              "over the whole step time",
                      "achieved_tflops": f64, "peak_tflops": fp64_peak, "frac": f64 / fp64_peak,
                      "peak_source": "measured in this run (DFMA loop)"},
        "hbm": {"achieved_gbs": 150.0 * rate / 1e9, "peak_gbs": hbm_peak,
                "frac": 150.0 * rate / 1e9 / hbm_peak, "bytes_per_atom_step": 150,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs"},
        "work_counters": {"sw_pairs": counts[0], "angle_terms": counts[1],
                          "moliere_pairs": counts[2], "many_leg_centres": counts[5]},
        "clocks": clk.summary(),
    }


# ---------------------------------------------------------------------------
def force_error(w, X):
    """Mixed against binary64 forces on one configuration (the slab after the
    timed cascade: thermal disorder plus the damaged region)."""
    import fib_md_gb300 as fm

    F = {}
    for prec in (fm.PREC_MIXED, fm.PREC_FP64):
        p = w["params"].copy()
        p.precision = prec
        g = fm.FibMD(p)
        g.upload(X, w["V"], None, w["Xi"], w["mass"], w["atype"], w["xsides"])
        g.set_tags(w["tags"])
        g.set_impact(1)
        g.si_nlist()
        F[prec] = g.si_force()
        g.close()
    dF = F[fm.PREC_MIXED] - F[fm.PREC_FP64]
    rms_d = float(np.sqrt(np.mean(np.sum(dF * dF, axis=1))))
    rms_f = float(np.sqrt(np.mean(np.sum(F[fm.PREC_FP64] ** 2, axis=1))))
    ev_a = w["params"].ec * 1e10
    return {"force_rms_rel": rms_d / rms_f, "force_rms_abs_eV_per_A": rms_d / ev_a,
            "force_max_abs_eV_per_A": float(np.abs(dF).max()) / ev_a,
            "force_config": "the slab after the timed mixed run (300 K plus the cascade)"}


def nve_drift(w, precision, steps=1000):
    """Total-energy drift (eV per mobile atom per ps) of an unthermostatted
    segment of the workload's slab with the ion parked far above it."""
    import fib_md_gb300 as fm

    p = w["params"].copy()
    p.precision = precision
    N, nsg = p.Natm, p.Nsg
    X = w["X"].copy(order="F")
    V = w["V"].copy(order="F")
    X[nsg:, 2] = p.remove_z - 1e-10
    V[nsg:] = 0.0
    tags = (w["tags"] & fm.TAG_FROZEN).astype(np.uint32)
    g = fm.FibMD(p)
    g.upload(X, V, None, w["Xi"], w["mass"], w["atype"], w["xsides"])
    g.set_tags(tags)
    g.set_impact(1)
    g.si_nlist()
    g.si_force()

    def energy():
        _, Vd, _ = g.download()
        _, _, U = g.si_force_energy()
        return U + 0.5 * float(np.sum(w["mass"][:, None] * Vd * Vd))

    # the slope of a least-squares line through E(t), sampled every tenth of
    # the segment: velocity Verlet's bounded energy fluctuation is not drift
    ts, Es = [0.0], [energy()]
    lt, t = 0, 0.0
    for k in range(10):
        lt, t, _, _ = g.steps(2, steps // 10, lt, t, 300.0)
        ts.append(t)
        Es.append(energy())
    g.close()
    mobile = int(np.count_nonzero(tags[:nsg] == 0))
    slope = np.polyfit(np.array(ts) * 1e12, np.array(Es), 1)[0]
    return float(slope / p.ec / mobile)


# ---------------------------------------------------------------------------
# batched ensemble: independent impacts on uneven slabs
def make_ensemble(nrep, precision, seed0=3000, list_skin_A=0.0):
    """Slabs of U{6..12} x U{6..12} x 10 unit cells, one Ga each at
    U(0.5, 5) keV and U(0, 30) degrees off normal, seeded azimuth and impact
    point (seed 3000 + r); atoms more than 15 A above the surface leave."""
    import fib_md_gb300 as fm

    p = fm.params_default()
    p.precision = precision
    p.list_skin = list_skin_A * 1e-10
    rs = np.random.default_rng(seed0)
    slabs = []
    for r in range(nrep):
        lx, ly = (int(v) for v in rs.integers(6, 13, size=2))
        eV = float(rs.uniform(500.0, 5000.0))
        th = float(rs.uniform(0.0, 30.0))
        slabs.append(fm.spec_slab((lx, ly, 10), seed=seed0 + r, ion_eV=eV, polar_deg=th,
                                  remove_above=15e-10, params=p))
    return slabs


def run_ensemble_batch(slabs, precision, steps):
    """Every impact in one batch context: wall time from upload to the
    downloaded final state, and each impact's outcome."""
    import torch
    import fib_md_gb300 as fm

    p = slabs[0].params.copy()
    p.precision = precision
    reps = [(s.params.Natm, s.params.Nsg, list(s.params.Lb), s.params.remove_z) for s in slabs]
    b = fm.FibMDBatch(p, reps)
    X = b.pad([s.X for s in slabs])
    V = b.pad([s.V for s in slabs])
    Xi = b.pad([s.Xi for s in slabs])
    mass = b.pad([s.mass for s in slabs], fill=1.0)
    atype = b.pad([s.atype for s in slabs], fill=1, dtype=np.int32)
    tags = b.pad([s.tags for s in slabs], fill=0, dtype=np.uint32)
    xs = np.zeros(b.N, np.int32)
    torch.cuda.synchronize()
    rb0 = 0
    w0 = time.perf_counter()
    b.upload(X, V, None, Xi, mass, atype, xs)
    b.set_tags(tags)
    b.si_nlist()
    b.si_force()
    rb0 = b.work_counters()[4]
    b.steps(2, steps, 0, 0.0, 300.0)
    Xf, _, _ = b.download()
    t_sim, _, removed = b.scalars()
    wall = time.perf_counter() - w0
    rebuilds = b.work_counters()[4] - rb0
    # each impact's outcome, computed on the device (the same quantities as
    # impact_statistics on the downloaded states)
    sp, dc, dp = b.impact_stats([s.surface_z for s in slabs])
    stats = [(int(sp[r]), float(dp[r]), int(dc[r])) for r in range(len(slabs))]
    atoms = int(b.natm.sum())
    stage = int(b.get_option("stage"))
    skin = b.get_option("skin")
    b.close()
    return {"wall_s": wall, "atoms": atoms, "padded_atoms": int(b.N), "rebuilds": int(rebuilds),
            "removed": removed.tolist(), "sim_time_s": t_sim.tolist(), "stats": stats,
            "force_stage": stage, "list_skin_A": skin}


def run_plain(slab, steps):
    """One impact alone in a plain binary64 context (no batching)."""
    import torch
    import fib_md_gb300 as fm

    p = slab.params.copy()
    p.precision = fm.PREC_FP64
    torch.cuda.synchronize()
    w0 = time.perf_counter()
    g = fm.FibMD(p)
    g.upload(slab.X, slab.V, None, slab.Xi, slab.mass, slab.atype, np.zeros(p.Natm, np.int32))
    g.set_tags(slab.tags)
    g.set_impact(1)
    g.si_nlist()
    g.si_force()
    g.steps(2, steps, 0, 0.0, 300.0)
    g.download()
    wall = time.perf_counter() - w0
    g.close()
    return wall


def two_sample(a, b):
    """Mann-Whitney U and Kolmogorov-Smirnov p-values of two samples."""
    from scipy import stats

    a = np.asarray([x for x in a if np.isfinite(x)], dtype=float)
    b = np.asarray([x for x in b if np.isfinite(x)], dtype=float)
    if len(a) < 2 or len(b) < 2:
        return {"n": [len(a), len(b)], "p_mannwhitney": None, "p_ks": None}
    if np.all(a == a[0]) and np.all(b == a[0]):
        pm = pk = 1.0
    else:
        pm = float(stats.mannwhitneyu(a, b, alternative="two-sided").pvalue)
        pk = float(stats.ks_2samp(a, b).pvalue)
    return {"n": [len(a), len(b)], "mean": [float(a.mean()), float(b.mean())],
            "p_mannwhitney": pm, "p_ks": pk}


def bench_ensemble(args):
    import fib_md_gb300 as fm

    nrep, steps = args.ensemble_replicas, args.ensemble_steps
    slabs = make_ensemble(nrep, fm.PREC_MIXED, list_skin_A=args.list_skin)
    # a short warm-up batch (context set-up, graph capture, first-touch)
    run_ensemble_batch(slabs[:4], fm.PREC_MIXED, 20)
    mixed = run_ensemble_batch(slabs, fm.PREC_MIXED, steps)
    fp64 = run_ensemble_batch(slabs, fm.PREC_FP64, steps)
    k = max(1, min(args.ensemble_plain_sample, nrep))
    run_plain(slabs[0], 20)
    plain = [run_plain(slabs[r], steps) for r in range(k)]
    plain_s = float(np.mean(plain))
    ih = lambda res: 3600.0 * nrep / res["wall_s"]
    cmp = {}
    for q, name in enumerate(["sputter_yield", "implant_depth_m", "displaced_atoms"]):
        cmp[name] = two_sample([s[q] for s in mixed["stats"]], [s[q] for s in fp64["stats"]])
    ok = all(v["p_mannwhitney"] is None or v["p_mannwhitney"] > 0.05 for v in cmp.values())
    return {
        "config": f"{nrep} impacts, U{{6..12}}^2 x 10 unit-cell slabs, U(0.5,5) keV Ga, "
                  f"U(0,30) deg, {steps} variable-dt steps each, one batch context, list skin "
                  f"{skin_text(args.list_skin)}",
        "impacts_per_hour": {"mixed_batched": ih(mixed), "fp64_batched": ih(fp64),
                             "fp64_plain": 3600.0 / plain_s},
        "mixed_batched_over_fp64_plain": ih(mixed) * plain_s / 3600.0,
        "mixed_batched_over_fp64_batched": fp64["wall_s"] / mixed["wall_s"],
        "atom_steps_per_s": {"mixed_batched": mixed["atoms"] * steps / mixed["wall_s"],
                             "fp64_batched": fp64["atoms"] * steps / fp64["wall_s"]},
        "wall_s": {"mixed_batched": mixed["wall_s"], "fp64_batched": fp64["wall_s"],
                   "fp64_plain_per_impact": plain_s, "fp64_plain_sample": k},
        "atoms": mixed["atoms"], "padded_atoms": mixed["padded_atoms"],
        "rebuild_fraction": {"mixed": mixed["rebuilds"] / steps, "fp64": fp64["rebuilds"] / steps},
        "mixed_force_stage_at_end": mixed["force_stage"],
        "list_skin_at_end_A": {"mixed": mixed["list_skin_A"], "fp64": fp64["list_skin_A"]},
        "mixed_vs_fp64_two_sample": cmp,
        "statistically_consistent_95": ok,
        "timing": "wall clock from upload of the initial states to the downloaded final states",
    }


# ---------------------------------------------------------------------------
# cumulative dose: successive impacts on one slab, run on the device
def run_dose(d, precision, nimp, steps=3000, relax=2e-12):
    import torch
    import fib_md_gb300 as fm

    sl = d.slab
    p = sl.params.copy()
    p.precision = precision
    g = fm.FibMD(p)
    torch.cuda.synchronize()
    w0 = time.perf_counter()
    g.upload(sl.X, sl.V, None, sl.Xi, sl.mass, sl.atype, np.zeros(p.Natm, np.int32))
    g.set_tags(sl.tags)
    g.set_impact(len(d.ion_atoms))
    g.si_nlist()
    g.si_force()
    stream = torch.cuda.ExternalStream(g.stream_ptr)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    rm, ir, t, st = g.dose(d.ion_atoms[:nimp], d.X0[:nimp], d.V0[:nimp], steps, relax)
    e1.record(stream)
    X, _, _ = g.download()
    wall = time.perf_counter() - w0
    dose_s = e0.elapsed_time(e1) * 1e-3
    g.close()
    crater = fm.crater_depth(X, sl.atype, list(p.Lb), sl.surface_z, p.remove_z,
                             (0.5 * p.Lb[0], 0.5 * p.Lb[1]), 30e-10)
    return {"wall_s": wall, "dose_call_s": dose_s, "removed": rm.tolist(), "ions_removed": ir.tolist(),
            "sim_time_s": t.tolist(), "md_steps": int(st[-1]), "atoms": int(sl.params.Natm),
            "crater_depth_m": crater}


def bench_dose(args):
    import fib_md_gb300 as fm

    n = args.dose_impacts
    n64 = n if args.dose_fp64_impacts < 0 else min(n, args.dose_fp64_impacts)
    p = fm.params_default()
    p.list_skin = args.list_skin * 1e-10
    d = fm.dose_slab((20, 20, 12), n, seed=4001, ion_eV=2000.0, window=30e-10,
                     remove_above=15e-10, params=p)
    mixed = run_dose(d, fm.PREC_MIXED, n)
    fp64 = run_dose(d, fm.PREC_FP64, n64) if n64 > 0 else None
    per = lambda r: np.diff(np.concatenate([[0], r["removed"]])).tolist()
    out = {
        "config": f"20x20x12 unit-cell slab ({d.slab.params.Nsg} Si), {n} successive 2 keV Ga "
                  "impacts at normal incidence in a 30x30 A window (seed 4001), 3000 steps "
                  "then 2 ps relaxation each, atoms 15 A above the surface removed, one "
                  "device-side dose call, list skin "
                  f"{skin_text(args.list_skin)}",
        "impacts": n,
        "impacts_per_hour": {"mixed": 3600.0 * n / mixed["wall_s"]},
        "wall_s": {"mixed": mixed["wall_s"]},
        "md_steps": {"mixed": mixed["md_steps"]},
        "us_per_md_step_in_dose_call": {
            "mixed": 1e6 * mixed["dose_call_s"] / max(mixed["md_steps"], 1)},
        "atom_steps_per_s": {"mixed": mixed["atoms"] * mixed["md_steps"] / mixed["wall_s"]},
        "yield_vs_dose": {"mixed": mixed["removed"]},
        "reflected_ions": {"mixed": mixed["ions_removed"][-1]},
        "crater_depth_m": {"mixed": mixed["crater_depth_m"]},
        "timing": "impacts_per_hour: wall clock from upload to the downloaded final state; "
                  "us_per_md_step_in_dose_call: CUDA events around the dose call alone",
    }
    if fp64:
        out["impacts_per_hour"]["fp64"] = 3600.0 * n64 / fp64["wall_s"]
        out["wall_s"]["fp64"] = fp64["wall_s"]
        out["md_steps"]["fp64"] = fp64["md_steps"]
        out["us_per_md_step_in_dose_call"]["fp64"] = (
            1e6 * fp64["dose_call_s"] / max(fp64["md_steps"], 1))
        out["atom_steps_per_s"]["fp64"] = fp64["atoms"] * fp64["md_steps"] / fp64["wall_s"]
        out["yield_vs_dose"]["fp64"] = fp64["removed"]
        out["reflected_ions"]["fp64"] = fp64["ions_removed"][-1]
        out["crater_depth_m"]["fp64"] = fp64["crater_depth_m"]
        out["mixed_vs_fp64_per_impact_yield"] = two_sample(per(mixed)[:n64], per(fp64))
    return out


# ---------------------------------------------------------------------------
# the cumulative-dose study at its full size (1000 impacts)
def dose_run_chunked(d, precision, nimp, chunk, steps=3000, relax=2e-12):
    """One dose of nimp successive impacts on the device, run in calls of
    `chunk` impacts with the positions downloaded after each call: the
    sputtered atoms after every impact and the crater depth after every
    chunk."""
    import fib_md_gb300 as fm

    sl = d.slab
    p = sl.params.copy()
    p.precision = precision
    g = fm.FibMD(p)
    g.upload(sl.X, sl.V, None, sl.Xi, sl.mass, sl.atype, np.zeros(p.Natm, np.int32))
    g.set_tags(sl.tags)
    g.set_impact(len(d.ion_atoms))
    g.si_nlist()
    g.si_force()
    removed, reflected, crater, steps_run = [], [], [], 0
    w0 = time.perf_counter()
    for k0 in range(0, nimp, chunk):
        k1 = min(nimp, k0 + chunk)
        rm, ir, _, st = g.dose(d.ion_atoms[k0:k1], d.X0[k0:k1], d.V0[k0:k1], steps, relax)
        removed += rm.tolist()
        reflected += ir.tolist()
        steps_run += int(st[-1])
        X, _, _ = g.download()
        crater.append((k1, fm.crater_depth(X, sl.atype, list(p.Lb), sl.surface_z, p.remove_z,
                                           (0.5 * p.Lb[0], 0.5 * p.Lb[1]), 30e-10)))
    wall = time.perf_counter() - w0
    g.close()
    per = np.diff(np.concatenate([[0], removed])).tolist()
    return {"impacts": nimp, "wall_s": wall, "md_steps": steps_run,
            "impacts_per_hour": 3600.0 * nimp / wall,
            "sputtered_per_impact": per, "sputtered_total": removed[-1],
            "reflected_ions": reflected[-1], "crater_depth_A": [[k, 1e10 * c] for k, c in crater]}


def dose_study(args):
    """Config 4: a 20x20x12 unit-cell slab (38,400 Si) receiving 2 keV Ga at
    normal incidence at seeded points of a 30x30 A window, 3000 steps plus
    2 ps of relaxation per impact, atoms 15 A above the surface removed.
    The first seed runs args.dose_impacts mixed-precision impacts (the full
    dose); every seed runs args.dose_compare mixed and binary64 impacts,
    whose per-impact yields and crater depths are compared by two-sample
    tests."""
    import fib_md_gb300 as fm

    seeds = [4001 + k for k in range(args.dose_seeds)]
    nfull, ncmp = args.dose_impacts, args.dose_compare
    p = fm.params_default()
    p.list_skin = args.list_skin * 1e-10
    runs = {}
    for k, seed in enumerate(seeds):
        n_mixed = max(ncmp, nfull) if k == 0 else ncmp
        d = fm.dose_slab((20, 20, 12), n_mixed, seed=seed, ion_eV=2000.0, window=30e-10,
                         remove_above=15e-10, params=p)
        runs[seed] = {"mixed": dose_run_chunked(d, fm.PREC_MIXED, n_mixed, args.dose_chunk),
                      "fp64": dose_run_chunked(d, fm.PREC_FP64, ncmp, args.dose_chunk)}
        print(json.dumps({"seed": seed, "mixed_impacts": n_mixed,
                          "mixed_wall_s": runs[seed]["mixed"]["wall_s"],
                          "fp64_wall_s": runs[seed]["fp64"]["wall_s"]}), file=sys.stderr,
              flush=True)
    ym = [y for sd in seeds for y in runs[sd]["mixed"]["sputtered_per_impact"][:ncmp]]
    yf = [y for sd in seeds for y in runs[sd]["fp64"]["sputtered_per_impact"][:ncmp]]

    def crater_at(r, n):
        return dict((kk, c) for kk, c in r["crater_depth_A"]).get(n)

    cm = [crater_at(runs[sd]["mixed"], ncmp) for sd in seeds]
    cf = [crater_at(runs[sd]["fp64"], ncmp) for sd in seeds]
    from scipy import stats

    out = {
        "config": "20x20x12 unit cells (38,400 Si), 2 keV Ga at normal incidence at seeded "
                  "uniform points of a 30x30 A window, 3000 steps then 2 ps of relaxation per "
                  "impact, atoms 15 A above the surface removed, spec mode, list skin "
                  f"{skin_text(args.list_skin)}, device-side dose calls of {args.dose_chunk} impacts",
        "seeds": seeds,
        "full_dose": {"seed": seeds[0], "precision": "mixed", **runs[seeds[0]]["mixed"]},
        "comparison": {
            "impacts_per_seed": ncmp,
            "per_impact_yield": two_sample(ym, yf),
            "per_impact_yield_t_test_p": float(stats.ttest_ind(ym, yf, equal_var=False).pvalue),
            "crater_depth_A_after": ncmp,
            "crater_depth_A": {"mixed": cm, "fp64": cf},
            "yield_per_seed": {str(sd): {"mixed": float(np.mean(
                runs[sd]["mixed"]["sputtered_per_impact"][:ncmp])), "fp64": float(np.mean(
                    runs[sd]["fp64"]["sputtered_per_impact"]))} for sd in seeds},
            "impacts_per_hour": {"mixed": [runs[sd]["mixed"]["impacts_per_hour"] for sd in seeds],
                                 "fp64": [runs[sd]["fp64"]["impacts_per_hour"] for sd in seeds]},
        },
    }
    if len(seeds) >= 2:
        out["comparison"]["crater_depth_two_sample"] = two_sample(cm, cf)
    return out


# ---------------------------------------------------------------------------
# the 8x8x8-cell slab (4097 atoms) in plain binary64 on the GPU beside the oracle
def bench_small_slab(args, repeats=3, cpu_sample=200):
    """8x8x8 unit cells (4096 Si + 1 Ga), 500 eV Ga at normal incidence 10 A
    above the surface (seed 1001), 300 K, the 2000 variable-dt steps from the
    ion's start on the GPU in binary64 (and in mixed precision), each run
    from a fresh upload, timed with CUDA events (median of `repeats`); the
    oracle's spec-mode step on the same slab over all host cores, a sample
    of `cpu_sample` steps after an untimed tenth."""
    import torch

    import fib_md_gb300 as fm

    cells, steps = (8, 8, 8), 2000
    w = make_workload(cells, seed=1001, energy_eV=500.0, polar_deg=0.0,
                      list_skin_A=args.list_skin)
    N = w["params"].Natm
    res = {}
    for name, prec in (("gpu_fp64", fm.PREC_FP64), ("gpu_mixed", fm.PREC_MIXED)):
        g = make_ctx(w, prec)
        g.set_option("timers", 0)
        stream = torch.cuda.ExternalStream(g.stream_ptr)
        ts = []
        for r in range(repeats + 1):
            fresh_state(g, w)
            torch.cuda.synchronize()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            _, t_sim, _, _ = g.steps(2, steps, 0, 0.0, 300.0)
            b.record(stream)
            b.synchronize()
            if r > 0:
                ts.append(a.elapsed_time(b) / 1e3)
        g.close()
        sec = statistics.median(ts)
        res[name] = {"atom_steps_per_s": N * steps / sec, "ms_per_run": 1e3 * sec,
                     "simulated_ps": t_sim * 1e12}
    nthreads = os.cpu_count() or 1
    sys.path.insert(0, str(ROOT / "tests"))
    import oracle_ffi as of

    ow = oracle_workload(cells, seed=1001, energy_eV=500.0, polar_deg=0.0,
                         list_skin_A=oracle_skin(args.list_skin))
    p = ow["params"].copy()
    o = of.Oracle(p)
    o.load(ow["X"], ow["V"], ow["Xi"], ow["mass"], ow["atype"], ow["xsides"])
    o.set_impact(1)
    o.spec_init(ow["tags"], 0.0)
    o.si_nlist()
    o.F[:] = o.si_force(nthreads=nthreads)
    _oracle_sample(o, cpu_sample // 10, nthreads)
    cpu = _oracle_sample(o, cpu_sample, nthreads)
    o.close()
    return {
        "config": f"8x8x8 unit cells ({N - 1} Si + 1 Ga), 500 eV Ga at normal incidence 10 A "
                  f"above the surface, seed 1001, 300 K, {steps} variable-dt steps from the "
                  "ion's start, spec mode, list skin "
                  f"{skin_text(args.list_skin)}",
        **res,
        "cpu_oracle": {"atom_steps_per_s": cpu, "cores": nthreads, "kind": "port",
                       "algorithm": CPU_ALGORITHM,
                       "sample": f"MD steps {cpu_sample // 10 + 1}-{cpu_sample // 10 + cpu_sample}"
                                 f" of the same cascade after {cpu_sample // 10} untimed"},
        "gpu_fp64_over_cpu": res["gpu_fp64"]["atom_steps_per_s"] / cpu,
    }


# ---------------------------------------------------------------------------
# the CPU side: the oracle (binary64, the reference's si_nlist/si_force with
# the spec-mode step) on the same cascade, set up without the GPU package
def _oracle_cascade(cells, list_skin_A, nthreads):
    """The oracle at the cascade's start: the seeded slab, spec-mode lists
    built, the first force evaluated (all host threads for the force)."""
    sys.path.insert(0, str(ROOT / "tests"))
    import oracle_ffi as of

    w = oracle_workload(cells, list_skin_A=oracle_skin(list_skin_A))
    p = w["params"].copy()
    p.mode = 1
    o = of.Oracle(p)
    o.load(w["X"], w["V"], w["Xi"], w["mass"], w["atype"], w["xsides"])
    o.set_impact(1)
    o.spec_init(w["tags"], 0.0)
    o.si_nlist()
    o.F[:] = o.si_force(nthreads=nthreads)
    return o


def _oracle_sample(o, sample_steps, nthreads):
    """Atom-steps/s of the next sample_steps spec-mode steps (rebuilds
    included as they fall due)."""
    t0 = time.perf_counter()
    for _ in range(sample_steps):
        o.spec_step(nthreads)
    return o.N * sample_steps / (time.perf_counter() - t0)


CPU_ALGORITHM = ("the oracle: binary64 restatement of the reference's si_nlist (cell lists) "
                 "and si_force (table SW 2-body, Moliere, connected-triplet SW 3-body) with "
                 "the spec-mode step; its force OpenMP over all host threads")


def cpu_baseline(cells, list_skin_A, sample_steps, nthreads=None):
    """The oracle on the cascade's first steps over all host cores: an
    untimed sample of a third of the steps, then sample_steps timed."""
    nthreads = nthreads or os.cpu_count() or 1
    o = _oracle_cascade(cells, list_skin_A, nthreads)
    _oracle_sample(o, max(1, sample_steps // 3), nthreads)
    value = _oracle_sample(o, sample_steps, nthreads)
    first = max(1, sample_steps // 3) + 1
    N = o.N
    o.close()
    return {"value": value, "unit": "atom-steps/s", "cores": nthreads, "kind": "port",
            "algorithm": CPU_ALGORITHM,
            "sample": f"MD steps {first}-{first + sample_steps - 1} of the {N}-atom cascade "
                      f"(after {first - 1} untimed), {nthreads} threads"}


def cpu_reference_run(cells, list_skin_A, warmup, steps, sample_steps, nthreads=None):
    """The reference arm: the oracle's cascade set up once, `warmup` untimed
    samples, then `steps` timed samples of sample_steps spec-mode steps each
    (the cascade goes on from sample to sample); the median rate."""
    nthreads = nthreads or os.cpu_count() or 1
    o = _oracle_cascade(cells, list_skin_A, nthreads)
    vals = []
    for n in range(warmup + steps):
        v = _oracle_sample(o, sample_steps, nthreads)
        if n >= warmup:
            vals.append(v)
    N = o.N
    o.close()
    return statistics.median(vals), {
        "value": statistics.median(vals), "unit": "atom-steps/s", "cores": nthreads,
        "kind": "port", "algorithm": CPU_ALGORITHM,
        "sample": f"per step {sample_steps} MD steps of the {N}-atom cascade, continuing from "
                  f"step to step over steps 1-{(warmup + steps) * sample_steps} of the window "
                  f"({warmup} untimed samples first), {nthreads} threads; median of {steps}"}


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    cells = tuple(int(x) for x in args.cells.split(","))
    if args.impl == "reference":
        if rank != 0:
            return 0
        steps, warmup = max(1, args.steps), max(0, args.warmup)
        v, cb = cpu_reference_run(cells, args.list_skin, warmup, steps,
                                  max(2, args.cpu_sample_steps // 4))
        N = 8 * cells[0] * cells[1] * cells[2] + 1
        out = {"impl": "reference", "metric": METRIC,
               "value": v, "unit": "atom-steps/s", "n_gpus": 0, "steps": steps,
               "warmup": warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
               "dtype": "f64", "data": "synthetic (seeded)",
               "config": workload_config(args, cells, N),
               "cpu_algorithm": CPU_ALGORITHM,
               "cpu_baseline": cb,
               "e2e": {"value": v, "unit": "atom-steps/s", "h2d_bytes_per_step": 0,
                       "d2h_bytes_per_step": 0}}
        print(json.dumps(out))
        return 0

    if args.dose_study:
        print(json.dumps(dose_study(args)))
        return 0

    if args.profile == "ensemble":
        import fib_md_gb300 as fm

        slabs = make_ensemble(256, fm.PREC_MIXED, list_skin_A=args.list_skin)
        p = slabs[0].params.copy()
        reps = [(s.params.Natm, s.params.Nsg, list(s.params.Lb), s.params.remove_z) for s in slabs]
        b = fm.FibMDBatch(p, reps)
        b.upload(b.pad([s.X for s in slabs]), b.pad([s.V for s in slabs]), None,
                 b.pad([s.Xi for s in slabs]), b.pad([s.mass for s in slabs], fill=1.0),
                 b.pad([s.atype for s in slabs], fill=1, dtype=np.int32), np.zeros(b.N, np.int32))
        b.set_tags(b.pad([s.tags for s in slabs], fill=0, dtype=np.uint32))
        b.si_nlist()
        b.si_force()
        ng = args.profile_graph_steps if args.profile_graph_steps >= 0 else 1000
        lt, t, _, _ = b.steps(2, ng, 0, 0.0, 300.0)
        b.set_option("graph", 0)
        b.steps(2, 20, lt, t, 300.0)
        b.close()
        return 0

    if args.profile == "dose":
        import fib_md_gb300 as fm

        p = fm.params_default()
        p.list_skin = args.list_skin * 1e-10
        d = fm.dose_slab((20, 20, 12), 1, seed=4001, ion_eV=2000.0, window=30e-10,
                         remove_above=15e-10, params=p)
        sl = d.slab
        q = sl.params.copy()
        q.precision = fm.PREC_MIXED
        g = fm.FibMD(q)
        g.upload(sl.X, sl.V, None, sl.Xi, sl.mass, sl.atype, np.zeros(q.Natm, np.int32))
        g.set_tags(sl.tags)
        g.set_impact(len(d.ion_atoms))
        g.si_nlist()
        g.si_force()
        g.set_option("stage", 1)
        g.set_atom(int(d.ion_atoms[0]), d.X0[0], d.V0[0])
        ng = args.profile_graph_steps if args.profile_graph_steps >= 0 else 300
        lt, t, _, _ = g.steps(2, ng, 0, 0.0, 300.0)
        g.set_option("graph", 0)
        g.steps(2, 20, lt, t, 300.0)
        g.close()
        return 0

    if args.profile:
        import fib_md_gb300 as fm

        w = make_workload(cells, list_skin_A=args.list_skin)
        g = make_ctx(w, fm.PREC_FP64 if args.profile == "fp64" else fm.PREC_MIXED)
        if args.reactions and args.profile != "fp64":
            g.set_option("reactions", 1)
        if args.profile == "step":
            # the window's first min(md_steps, 300) mixed spec-mode steps
            # launch by launch (every kernel of the step loop)
            g.set_option("graph", 0)
            g.steps(2, min(args.md_steps, 300), 0, 0.0, 300.0)
            g.close()
            return 0
        for _ in range(5 if args.profile == "build" else 3):
            if args.profile == "build":
                g.si_nlist()
            else:
                g.si_force()
        g.close()
        return 0

    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    out = bench_ours(args, rank, world, dist)
    if not args.no_ensemble:
        out["ensemble"] = bench_ensemble(args)
    if args.dose_impacts > 0:
        out["dose"] = bench_dose(args)
    if args.large_steps > 0 and rank == 0:
        out["large"] = bench_large(args)
    if not args.no_small_slab and rank == 0:
        out["small_slab"] = bench_small_slab(args)
    if rank == 0:
        if not args.no_cpu_baseline:
            out["cpu_baseline"] = cpu_baseline(cells, args.list_skin, args.cpu_sample_steps)
        print(json.dumps(out))
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
