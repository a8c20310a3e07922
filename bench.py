#!/usr/bin/env python3
"""Benchmark of the GB300 photon-history transport path.

Workload (one "step"): the heterogeneous cone-beam dose configuration - 256x256x128 voxels
at 0.5 mm, 40 seeded ellipsoids (soft tissue / adipose / cortical bone) in air, 80 kVp
Kramers spectrum filtered by 2.5 mm Al, point source 50 cm from the phantom with a 20 degree
cone, per-voxel dose and variance tally - 1e8 histories through the mixed-precision kernel
(FP32 transport, 64-bit fixed-point tallies).  Seeded synthetic inputs; nothing is read
from a dataset.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One JSON line on rank 0.  --impl reference times the CPU restatement of the reference
transport (oracle/, all host threads) on bounded samples of the same workload.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "histories/s per GB300, mixed-precision vs plain at matched dose error; p99 latency"
UNIT = "histories/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--histories", type=float, default=1e8)
    p.add_argument("--cpu-sample", type=float, default=1e6, help="histories of the CPU baseline sample")
    p.add_argument("--quick", action="store_true", help="skip the FP64, e2e, CPU, batched and serving legs")
    p.add_argument("--batched", type=int, default=1, help="run the 64-job batched leg (1/0)")
    p.add_argument("--batch-scale", type=float, default=1.0, help="history scale of the batched jobs")
    p.add_argument("--batch-fp64-scale", type=float, default=0.1,
                   help="further history scale of the jobs of the batched FP64/mixed pair")
    p.add_argument("--batch-jobs", type=int, default=64, help="jobs of the batched leg")
    p.add_argument("--batch-autotune", type=int, default=1,
                   help="autotune the batched launch shape (1) or take the default shape (0)")
    p.add_argument("--batch-pair", type=int, default=1, help="run the batched FP64/mixed pair (1/0)")
    p.add_argument("--batched-only", action="store_true",
                   help="run the batched leg alone and print its JSON (profiling)")
    p.add_argument("--precision", default="mixed", choices=["mixed", "fp64"],
                   help="precision of the timed transport steps (fp64: the plain drop-in form, for profiling)")
    p.add_argument("--serving", type=int, default=1, help="run the serving leg (1/0)")
    p.add_argument("--serving-requests", type=int, default=120, help="requests at 200/s in the serving leg")
    p.add_argument("--radiography", type=int, default=1, help="run the radiography precision-ablation leg (1/0)")
    p.add_argument("--radiography-histories", type=float, default=1e6,
                   help="histories per precision (radiography, reference tracking)")
    p.add_argument("--radiography-macro-histories", type=float, default=1e8,
                   help="histories per precision (radiography, macro-cell tracking)")
    p.add_argument("--radiography-only", action="store_true",
                   help="run the radiography precision-ablation leg alone and print its JSON (profiling)")
    return p.parse_args()


def log(*a):
    print(*a, file=sys.stderr, flush=True)


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.index)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm, smax, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
                power.append(float(f[3]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "power_w_max": max(power) if power else None, "samples": len(sm), "reasons": sorted(reasons)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        backend = "nccl"
        try:
            import torch
            if not torch.cuda.is_available():
                backend = "gloo"
        except ImportError:
            backend = "gloo"
        dist.init_process_group(backend=backend)
    return world, rank, local, dist


def replica_first(rank, i, n):
    """First history id of step i on rank `rank`: replicas take disjoint history ranges of
    the same Philox key (rank r owns ids [r * 2^40, (r + 1) * 2^40))."""
    return (rank << 40) + i * n


def job_rate(dist, world, steps, n_hist, total_s, device="cuda"):
    """(whole-job histories/s, the slowest rank's time): every rank ran `steps` steps of
    n_hist histories in total_s seconds; the job's time is the maximum over ranks."""
    if dist:
        import torch
        t = torch.tensor([total_s], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_s = float(t.item())
    return world * steps * n_hist / total_s, total_s


def rel_diff_stats(np, a, b, frac=0.01):
    """|a - b| / b over the entries of b above frac x its maximum: p50, p99, max and the
    count - the per-voxel (or per-bin) error of one precision against the other."""
    a, b = np.asarray(a, dtype=np.float64).ravel(), np.asarray(b, dtype=np.float64).ravel()
    sel = b > frac * b.max()
    r = np.abs(a[sel] - b[sel]) / b[sel]
    return {"entries": int(sel.sum()), "p50": float(np.percentile(r, 50)), "p99": float(np.percentile(r, 99)),
            "max": float(r.max()), "total_rel_diff": float(abs(a.sum() - b.sum()) / b.sum())}


def reference_arm(args, world, rank):
    """CPU restatement of the reference transport, all host threads, bounded samples."""
    if rank != 0:
        return
    import oracle
    from midsx_gb300 import build as B, scenes
    B.build()  # compiles the oracle library (nothing of the product is loaded in this arm)
    al = oracle.tables.tables((scenes.ALUMINIUM,), 150e3)
    sc = scenes.cone_beam_dose(n_histories=int(args.histories), al=al)
    blob = oracle.tables_for(sc)  # the oracle's own table build
    threads = os.cpu_count() or 1
    n = int(min(args.cpu_sample, 4e5))
    times = []
    for i in range(args.warmup + args.steps):
        r = oracle.run(blob, n=n, seed=1, first=i * n, rng=oracle.RNG_MT19937, threads=threads, dose=True,
                       **sc.oracle_kwargs())
        if i >= args.warmup:
            times.append(r["run_time"])
    value = n * len(times) / sum(times)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded ellipsoid phantom, Kramers spectrum)",
            "config": {"workload": sc.name, "histories_per_step": n, "note": "bounded sample of the 1e8-history step"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": "%d histories per step of %s, mt19937 streams" % (n, sc.name)},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    world, rank, local, dist = dist_setup()
    if args.impl == "reference":
        reference_arm(args, world, rank)
        return
    import numpy as np
    import torch
    if args.radiography_only or args.batched_only:
        from midsx_gb300 import build as B
        B.build()
        torch.cuda.set_device(local)
        if rank == 0:
            out = radiography_leg(args, np, torch) if args.radiography_only else batched_leg(args, torch)
            print(json.dumps(out), flush=True)
        return

    import midsx_gb300 as M
    from midsx_gb300 import build as B, native as N, scenes

    torch.cuda.set_device(local)
    # one rank per node compiles (in-tree objects and libraries); the others wait for it
    if local == 0:
        B.build()
    if dist:
        dist.barrier()
    N_hist = int(args.histories)
    t0 = time.time()
    sc = scenes.cone_beam_dose(n_histories=N_hist)
    tables, ph, src, tl = sc.build()
    log("setup %.1fs (tables %d materials, %d voxels)" % (time.time() - t0, len(sc.materials), ph.n_voxels))
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")  # > 129 MB L2
    base = replica_first(rank, 0, 0)

    def step(i, precision=args.precision, n=N_hist, events=None):
        flush.zero_()
        if events:
            events[0].record(stream)
        tl.reset(sptr)
        if events:
            events[1].record(stream)
        M.run(tables, ph, src, tl, n, seed=1, first=replica_first(rank, i, n), precision=precision, stream=sptr)
        if events:
            events[2].record(stream)

    for i in range(args.warmup):
        step(i)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    for i in range(args.steps):
        step(args.warmup + i, events=evs[i])
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clk = clocks.stop()
    step_ms = [e[0].elapsed_time(e[2]) for e in evs]
    kern_ms = [e[1].elapsed_time(e[2]) for e in evs]
    value, total_s = job_rate(dist, world, args.steps, N_hist, sum(step_ms) / 1e3)
    st = tl.stats()  # raises MidsxError(STEP_CAP) if any history reached the step cap
    result = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
              "warmup": args.warmup, "ms_per_step": 1e3 * total_s / args.steps, "higher_is_better": True,
              "scaling": "weak", "vs_baseline": None,
              "dtype": "f32 transport / int64 fixed-point tallies" if args.precision == "mixed" else "f64",
              "data": "synthetic (seeded ellipsoid phantom, Kramers spectrum)",
              "config": {"workload": sc.name, "histories_per_step": N_hist, "precision": args.precision,
                         "voxels": ph.n_voxels, "dose_tally": "count/sum/sumsq per voxel (268 MB)",
                         "l2": "flushed between steps (256 MB write) and tally > L2",
                         "launch": "photon pool, 128-thread blocks, 2 Woodcock steps per pass (defaults)",
                         "parallelism": "replicas over history ranges" if world > 1 else "single GPU"},
              "clocks": clk, "gpu_launches": args.steps,
              "step_latency_ms": {"p50": statistics.median(step_ms), "p99": float(np.percentile(step_ms, 99))},
              "steps_per_history": st["steps"] / st["histories"],
              "voxel_fetches_per_history": st["voxel_fetches"] / st["histories"],
              "step_cap_hits": st["step_cap_hits"]}
    if rank != 0:
        return
    if not args.quick:
        # plain FP64 form on the same workload and the same Philox streams
        n64 = max(N_hist // 10, 1000)
        ev64 = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(2)]
        step(0, "fp64", n64)
        for i in range(2):
            step(1 + i, "fp64", n64, ev64[i])
        torch.cuda.synchronize()
        t64 = sum(e[1].elapsed_time(e[2]) for e in ev64) / 1e3
        plain = 2 * n64 / t64
        # error of the mixed form against the FP64 form on identical Philox streams: the
        # per-voxel relative difference of the dose sums (voxels above 1 % of the maximum)
        ncmp = min(N_hist, 4_000_000)
        doses = {}
        for p in ("fp64", "mixed"):
            tl.reset(sptr)
            M.run(tables, ph, src, tl, ncmp, seed=77, precision=p, stream=sptr)
            doses[p] = tl.dose(sptr)["sum"]
        result["plain_fp64"] = {"value": plain, "unit": UNIT, "histories_per_step": n64,
                                "mixed_over_plain": value / world / plain}
        result["mixed_vs_fp64_identical_streams"] = dict(
            histories=ncmp, **rel_diff_stats(np, doses["mixed"], doses["fp64"]))
        result["batch_variance"] = batch_variance_leg(M, np, torch, sc, tables, ph, src, sptr, flush, N_hist)
        # end to end through the C ABI with host buffers (pinned), copies inside the timing
        ids_pinned = torch.from_numpy(sc.ids.ravel()).pin_memory()
        dose_pinned = torch.empty(ph.n_voxels, dtype=torch.float64).pin_memory()
        e2e_t = []
        for i in range(1 + args.steps):
            cfg = M.run_config(N_hist, 1, first=base + (100 + i) * N_hist, precision="mixed")
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            _run_host(M, N, tables, ph.spec, ids_pinned, src.spec, sc, cfg, dose_pinned)
            t2 = time.perf_counter()
            if i:
                e2e_t.append(t2 - t1)
        result["e2e"] = {"value": N_hist / statistics.mean(e2e_t), "unit": UNIT,
                         "h2d_bytes_per_step": int(sc.ids.nbytes + 2 * 8 * len(sc.source["spectrum"][0])),
                         "d2h_bytes_per_step": int(ph.n_voxels * 8 + 128),
                         "latency_ms": {"p50": 1e3 * statistics.median(e2e_t),
                                        "p99": 1e3 * float(np.percentile(e2e_t, 99))}}
        # CPU baseline: the oracle on a bounded sample, all host threads
        import oracle
        threads = os.cpu_count() or 1
        ncpu = int(args.cpu_sample)
        r = oracle.run(oracle.tables_for(sc), n=ncpu, seed=1, rng=oracle.RNG_MT19937, threads=threads, dose=True,
                       **sc.oracle_kwargs())
        so = r["stats"]
        result["cpu_baseline"] = {"value": ncpu / r["run_time"], "unit": UNIT, "cores": threads, "kind": "port",
                                  "sample": "%d histories of %s (oracle, mt19937 streams)" % (ncpu, sc.name)}
        F = so["voxel_fetches"] / so["histories"]
        W = so["tally_words"] / so["histories"]
    else:
        F = st["voxel_fetches"] / st["histories"]
        W = st["tally_words"] / st["histories"]
    # roofline of the transport kernel: algorithmic bytes = 32 B x (voxel fetches + tally
    # records) per history, F and W counted by the CPU oracle on this workload
    b_hist = 32.0 * (F + W)
    kernel_s = statistics.mean(kern_ms) / 1e3
    achieved = N_hist * b_hist / kernel_s / 1e9
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    peak, peak_src = 6800.0, "fallback"
    if os.path.exists(peaks_path):
        peak, peak_src = float(json.load(open(peaks_path))["hbm_gbs"]), "measured"
    traffic = None
    profile = {}
    tpath = os.path.join(ROOT, "profiles", "transport_traffic.txt")
    if os.path.exists(tpath):
        for line in open(tpath):
            if line and not line.startswith("#") and len(line.split()) == 2:
                profile[line.split()[0]] = float(line.split()[1])
    if "dram_bytes_per_history" in profile:
        traffic = profile["dram_bytes_per_history"] * N_hist
    result["roofline"] = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                          "frac": achieved / peak, "traffic": traffic, "peak_source": peak_src,
                          "bytes_per_history": b_hist, "F": F, "W": W,
                          "kernel_ms": 1e3 * kernel_s}
    if "issue_active_pct" in profile:
        # neither HBM nor a tensor pipe limits this kernel: dependent-latency chains per warp
        result["roofline"]["limiter"] = {
            "kind": "latency (dependent chains per warp), not bandwidth",
            "issue_active_pct": profile["issue_active_pct"],
            "warps_active_per_sm": profile.get("warps_active_per_sm"),
            "lanes_per_instruction": profile.get("lanes_per_instruction"),
            "l2_sectors_per_history": profile.get("l2_sectors_per_history"),
            "l2_gbs_in_capture": profile.get("l2_gbs"),
            "source": "ncu capture of 4e6 histories (profiles/transport_traffic.txt)"}
    rs = random_sector_leg(torch)
    result["roofline"]["random_sector"] = rs
    # the same histories against the random-sector ceilings: voxel fetches from the L2 (the
    # 8 MB phantom stays resident), tally records as atomics to HBM (the 268 MB tally does not)
    bound = sector_bound_rate(F, W, rs["l2_load_gbs"], rs["hbm_red_gbs"])
    result["roofline"]["random_sector_bound"] = {
        "fetches_from": "L2", "tally_records_to": "HBM", "histories_per_s": bound,
        "frac": value / world / bound}
    if "e2e" not in result:
        result["e2e"] = None
    if not args.quick:
        for mode in ("background_fast", "macro_cell"):
            result[mode + "_tracking"] = fast_tracking_leg(M, np, torch, tables, ph, src, tl, sptr, flush, N_hist,
                                                           mode)
    if not args.quick:
        result["water_cube_plain"] = water_cube_leg(args, np, torch)
    if not args.quick and args.radiography:
        result["radiography_precision_ablation"] = radiography_leg(args, np, torch)
    # configurations whose phantom and tallies fit the L2: frac of the L2 random-sector bound,
    # with F and W frozen from the oracle's counters on their seeded inputs
    wc = result.get("water_cube_plain")
    if wc:
        F1, W1 = FROZEN_FW["water_cube"]
        b1 = sector_bound_rate(F1, W1, rs["l2_load_gbs"], rs["l2_red_gbs"])
        wc["l2_random_sector_bound"] = {"F": F1, "W": W1, "histories_per_s": b1, "frac": wc["mixed"]["value"] / b1}
    ra = result.get("radiography_precision_ablation")
    if ra:
        F3, W3 = FROZEN_FW["radiography"]
        b3 = sector_bound_rate(F3, W3, rs["l2_load_gbs"], rs["l2_red_gbs"])
        ra["l2_random_sector_bound"] = {"F": F3, "W": W3, "histories_per_s": b3,
                                        "frac": ra["reference_tracking"]["mixed"]["value"] / b3,
                                        "tracking": "reference (F counts its Woodcock steps in the grid)"}
    if not args.quick and args.batched:
        result["batched"] = batched_leg(args, torch)
    if not args.quick and args.serving:
        result["serving"] = serving_leg(args)
    print(json.dumps(result), flush=True)


def fast_tracking_leg(M, np, torch, tables, ph, src, tl, sptr, flush, n_hist, mode):
    """The same workload with MIDSX_TRACK_BACKGROUND_FAST (flights in the background air use
    the air's own attenuation and stop at the grid) or MIDSX_TRACK_MACRO_CELL (also local
    majorants of 8^3-voxel cells inside the grid): not the reference's algorithm, so it is
    reported beside the headline, with its dose checked statistically against the reference
    algorithm on 2e6 histories."""
    stream = torch.cuda.current_stream()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    times = []
    for i in range(4):  # one warm-up, three timed
        flush.zero_()
        tl.reset(sptr)
        ev[0].record(stream)
        M.run(tables, ph, src, tl, n_hist, seed=11, first=(50 + i) * n_hist, precision="mixed", stream=sptr,
              tracking=mode)
        ev[1].record(stream)
        torch.cuda.synchronize()
        if i:
            times.append(ev[0].elapsed_time(ev[1]) / 1e3)
    st = tl.stats(allow_cap=True)
    ncmp = 2_000_000
    doses = {}
    for m in ("reference", mode):
        tl.reset(sptr)
        M.run(tables, ph, src, tl, ncmp, seed=91 if m == "reference" else 92, precision="mixed", stream=sptr,
              tracking=m)
        doses[m] = tl.dose(sptr)
    a, b = doses["reference"], doses[mode]
    s1, q1, s2, q2 = (x.ravel() for x in (a["sum"], a["sumsq"], b["sum"], b["sumsq"]))
    sel = (s1 + s2) > 0.01 * max(s1.max(), s2.max())
    z = (s1[sel] - s2[sel]) / np.sqrt(q1[sel] + q2[sel])
    return {"value": n_hist / (sum(times) / len(times)), "unit": UNIT, "histories_per_step": n_hist,
            "steps_timed": len(times), "steps_per_history": st["steps"] / st["histories"],
            "step_cap_hits": st["step_cap_hits"],
            "dose_vs_reference_tracking": {"histories": ncmp, "voxels_compared": int(sel.sum()),
                                           "frac_voxels_beyond_3sigma": float(np.mean(np.abs(z) > 3)),
                                           "total_rel_diff": float(abs(s1.sum() - s2.sum()) / s1.sum())}}


def radiography_leg(args, np, torch):
    """Config 3, the precision ablation: the 512x512x256 radiography phantom at 0.5 mm (40
    ellipsoids and sixteen 2 mm lead spheres), 100 kVp, 512^2 detector of 1 mm bins at 100 cm
    SID, primary and scattered fluence per bin.  The mixed and the FP64 path run on identical
    Philox streams; the error of the mixed form is the per-bin relative difference of its
    images against the FP64 images.  With the reference algorithm (global majorant: ~17.5k
    Woodcock steps per history, lead sets it along the whole 100 cm) on a bounded history
    count; with the opt-in macro-cell majorants on 1e8 histories in both precisions (the
    config's 1e9 would take ~6 s mixed, ~1 min FP64)."""
    import midsx_gb300 as M
    from midsx_gb300 import scenes
    t0 = time.time()
    sc = scenes.radiography(n_histories=1)
    tables, ph, src, tl = sc.build()
    log("radiography setup %.1fs" % (time.time() - t0))
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]

    def timed(n, precision, tracking="reference", seed=5):
        tl.reset(sptr)
        ev[0].record(stream)
        M.run(tables, ph, src, tl, n, seed=seed, precision=precision, stream=sptr, tracking=tracking)
        ev[1].record(stream)
        torch.cuda.synchronize()
        return ev[0].elapsed_time(ev[1]) / 1e3

    def ablation(n, tracking, seed):
        images, out = {}, {}
        for precision in ("mixed", "fp64"):
            dt = timed(n, precision, tracking, seed)
            e, c = tl.binned(0, sptr)
            images[precision] = e
            st = tl.stats(sptr)  # raises if a history reached the step cap
            out[precision] = {"value": n / dt, "unit": UNIT, "steps_per_history": st["steps"] / st["histories"],
                              "step_cap_hits": st["step_cap_hits"]}
        a, b = images["mixed"], images["fp64"]
        err = {}
        for name, cls in (("primary", [0]), ("scatter", [1, 2, 3])):
            ia, ib = a[..., cls].sum(axis=2), b[..., cls].sum(axis=2)
            err[name] = rel_diff_stats(np, ia, ib)
            err[name]["bins_identical"] = float(np.mean(ia[ib > 0] == ib[ib > 0]))
            k = 8  # 64 x 64 image of 8 x 8 bins
            ra = ia.reshape(ia.shape[0] // k, k, ia.shape[1] // k, k).sum(axis=(1, 3))
            rb = ib.reshape(ib.shape[0] // k, k, ib.shape[1] // k, k).sum(axis=(1, 3))
            err[name + "_8x8_rebinned"] = rel_diff_stats(np, ra, rb)
        return {"histories": n, "tracking": tracking, "mixed": out["mixed"], "fp64": out["fp64"],
                "mixed_over_fp64": out["mixed"]["value"] / out["fp64"]["value"],
                "mixed_vs_fp64_identical_streams": err}, images["mixed"]

    n = int(args.radiography_histories)
    timed(n // 10, "mixed")  # warm-up
    ref, ref_img = ablation(n, "reference", 5)
    macro, macro_img = ablation(int(args.radiography_macro_histories), "macro_cell", 7)
    # the opt-in modes against the reference algorithm (different streams: statistical)
    prim_ref, scat_ref = ref_img[..., 0].sum(), ref_img[..., 1:].sum()
    nm = int(args.radiography_macro_histories)
    macro["primary_per_history_rel_diff_vs_reference"] = float(
        abs(macro_img[..., 0].sum() / nm - prim_ref / n) / (prim_ref / n))
    macro["scatter_per_history_rel_diff_vs_reference"] = float(
        abs(macro_img[..., 1:].sum() / nm - scat_ref / n) / (scat_ref / n))
    dt = timed(n, "mixed", tracking="background_fast", seed=6)
    st = tl.stats(sptr)
    e, _ = tl.binned(0, sptr)
    bg = {"histories": n, "value": n / dt, "unit": UNIT, "steps_per_history": st["steps"] / st["histories"],
          "step_cap_hits": st["step_cap_hits"],
          "primary_total_rel_diff_vs_reference": float(abs(e[..., 0].sum() - prim_ref) / prim_ref),
          "scatter_total_rel_diff_vs_reference": float(abs(e[..., 1:].sum() - scat_ref) / scat_ref)}
    return {"workload": sc.name + " (512^2 detector at 100 cm SID, 16 Pb spheres)",
            "reference_tracking": ref, "macro_cell_tracking": macro, "background_fast_tracking": bg}


def water_cube_leg(args, np, torch):
    """Config 1, the plain-method drop-in: 100^3 water voxels at 1 mm in a 20 cm air box, 60 keV
    pencil beam, 100 x 100 exit-plane bins, 1e6 histories per run (seed 1), per-voxel dose.
    The FP64 plain kernel and the mixed kernel (five timed runs each, device events), the
    mixed form's per-voxel and per-bin error against FP64 on identical streams, and the CPU
    oracle on the same 1e6 histories (all host threads)."""
    import midsx_gb300 as M
    import oracle
    from midsx_gb300 import scenes
    sc = scenes.water_cube()
    tables, ph, src, tl = sc.build()
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    n = 1_000_000
    out, dose, bins = {}, {}, {}
    for precision in ("fp64", "mixed"):
        tl.reset(sptr)
        M.run(tables, ph, src, tl, n, seed=1, precision=precision, stream=sptr)  # warm-up, and the error data
        st = tl.stats(sptr)
        dose[precision] = tl.dose(sptr)["sum"]
        bins[precision] = tl.binned(0, sptr)[0].sum(axis=2)
        times = []
        for i in range(5):
            tl.reset(sptr)
            ev[0].record(stream)
            M.run(tables, ph, src, tl, n, seed=1, first=(i + 1) * n, precision=precision, stream=sptr)
            ev[1].record(stream)
            torch.cuda.synchronize()
            times.append(ev[0].elapsed_time(ev[1]) / 1e3)
        out[precision] = {"value": n / statistics.mean(times), "unit": UNIT, "ms_per_run": 1e3 * statistics.mean(times),
                          "steps_per_history": st["steps"] / st["histories"], "step_cap_hits": st["step_cap_hits"]}
    threads = os.cpu_count() or 1
    r = oracle.run(oracle.tables_for(sc), n=n, seed=1, rng=oracle.RNG_MT19937, threads=threads, **sc.oracle_kwargs())
    return {"workload": sc.name + " (100^3 at 1 mm, 100 x 100 exit-plane bins)", "histories": n,
            "fp64": out["fp64"], "mixed": out["mixed"],
            "cpu_oracle": {"value": n / r["run_time"], "unit": UNIT, "cores": threads},
            "mixed_vs_fp64_identical_streams": {"dose_voxels": rel_diff_stats(np, dose["mixed"], dose["fp64"]),
                                                "exit_plane_bins": rel_diff_stats(np, bins["mixed"], bins["fp64"])}}


def batch_variance_leg(M, np, torch, sc, tables, ph, src, sptr, flush, n_hist):
    """The headline workload with the batch-method dose variance (MIDSX_DOSE_BATCHES): one
    step split into 10 and into 100 batches, against the same step without batches - the
    cost of a history-based variance on top of the reference's per-deposit sums."""
    from midsx_gb300 import native as N
    stream = torch.cuda.current_stream()
    tb = M.Tallies(ph, sc.specs, N.DOSE_BATCHES)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    out = {}
    for B in (1, 10, 100):
        times = []
        for i in range(3):
            flush.zero_()
            tb.reset(sptr)
            ev[0].record(stream)
            M.run(tables, ph, src, tb, n_hist, seed=1, first=(200 + i) * n_hist, precision="mixed", stream=sptr,
                  variance_batches=B)
            ev[1].record(stream)
            torch.cuda.synchronize()
            times.append(ev[0].elapsed_time(ev[1]) / 1e3)
        out["batches_%d" % B] = {"value": n_hist / statistics.mean(times), "unit": UNIT}
    tb.close()
    return out


# Voxel fetches (F) and tally records (W) per history counted by the oracle on the seeded
# inputs of the water-cube (100^3, 60 keV pencil) and radiography (512x512x256, 16 Pb spheres,
# reference tracking) workloads, frozen with the CPU baseline.
FROZEN_FW = {"water_cube": (2.06, 2.15), "radiography": (2369.0, 1.23)}


def sector_bound_rate(F, W, load_gbs, red_gbs):
    """Histories/s if every voxel fetch and tally record ran at its random-32 B-sector ceiling."""
    return 1.0 / (32.0 * F / (load_gbs * 1e9) + 32.0 * W / (red_gbs * 1e9))


def random_sector_leg(torch, requests=1 << 27):
    """Ceilings of random 32 B sector traffic (midsx_gpu_probe_sectors): loads cached in L2 only
    and 64-bit atomic adds, over footprints from 16 MiB to 4 GiB; CUDA events around 5 launches
    after 2 warm-up launches, `requests` sectors per launch.  The L2 ceiling is the best of the
    footprints up to a quarter of the L2, the HBM ceiling the 4 GiB footprint."""
    import ctypes as C
    from midsx_gb300 import native as N
    lib = N.load()
    l2 = torch.cuda.get_device_properties(torch.cuda.current_device()).L2_cache_size
    stream = torch.cuda.current_stream()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    out = {"l2_bytes": l2, "requests_per_launch": requests, "load_gbs_by_footprint": {}, "red_gbs_by_footprint": {}}
    for mib in (16, 32, 64, 256, 1024, 4096):
        buf = torch.zeros(mib << 20, dtype=torch.uint8, device="cuda")
        for mode, key in ((0, "load_gbs_by_footprint"), (1, "red_gbs_by_footprint")):
            issued = C.c_uint64()

            def launch(seed):
                N.check(lib.midsx_gpu_probe_sectors(C.c_void_p(buf.data_ptr()), buf.numel(), mode, requests, seed,
                                                    C.byref(issued), C.c_void_p(stream.cuda_stream)),
                        "midsx_gpu_probe_sectors")
            launch(1)
            launch(2)
            ev[0].record(stream)
            for r in range(5):
                launch(100 + r)
            ev[1].record(stream)
            torch.cuda.synchronize()
            t = ev[0].elapsed_time(ev[1]) / 1e3 / 5
            out[key]["%d_MiB" % mib] = issued.value * 32 / t / 1e9
            buf.zero_()
        del buf
    torch.cuda.empty_cache()
    fits = [k for k in out["load_gbs_by_footprint"] if (int(k.split("_")[0]) << 20) <= l2 // 4]
    out["l2_load_gbs"] = max(out["load_gbs_by_footprint"][k] for k in fits)
    out["l2_red_gbs"] = max(out["red_gbs_by_footprint"][k] for k in fits)
    out["hbm_load_gbs"] = out["load_gbs_by_footprint"]["4096_MiB"]
    out["hbm_red_gbs"] = out["red_gbs_by_footprint"]["4096_MiB"]
    return out


def batched_leg(args, torch):
    """64 independent simulations (phantom edge log-uniform 32-256 voxels at 1 mm, 20-120 kVp,
    1e5-1e8 histories each, own dose tallies) in one CUDA-graph replay: the jobs of at least
    the own-launch threshold in single-job launches of their own, the others in one persistent
    launch (shape from the autotuner); beside it the same graph with every job in the
    persistent launch, and the same jobs run one midsx_gpu_run each, back to back on one
    stream."""
    import midsx_gb300 as M
    from midsx_gb300 import scenes
    t0 = time.time()
    jobs = scenes.batch_jobs(n_jobs=args.batch_jobs, seed=1, hist_scale=args.batch_scale)
    tables = M.Tables(jobs[0].materials, e_max=150e3)
    objs = []
    for sc in jobs:
        ph = M.Phantom(tables, sc.domain, sc.spacing, sc.origin, sc.ids, sc.background)
        objs.append((ph, M.Source(**sc.source), M.Tallies(ph, sc.specs, sc.dose_mode)))
    log("batched setup %.1fs" % (time.time() - t0))
    batch = M.Batch(tables, [(ph, src, tl, 1 + j, 0, sc.n_histories)
                             for j, (sc, (ph, src, tl)) in enumerate(zip(jobs, objs))])
    stream = M.Stream()
    launch, tuned_rate = {}, None
    if args.batch_autotune:
        launch, tuned_rate = batch.autotune("mixed", trial=4_000_000, stream=stream.handle)
    batch.capture(stream.handle, "mixed", **launch)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    ts = torch.cuda.ExternalStream(stream.handle.value)
    batch.replay(stream.handle)  # warm-up
    stream.synchronize()
    reps = 2
    ev[0].record(ts)
    for _ in range(reps):
        batch.replay(stream.handle)
    ev[1].record(ts)
    stream.synchronize()
    graph_s = ev[0].elapsed_time(ev[1]) / 1e3 / reps
    # the same graph with every job in the persistent launch (no launches of their own)
    batch.set_own_launch(2**64 - 1)
    batch.capture(stream.handle, "mixed", **launch)
    batch.replay(stream.handle)
    stream.synchronize()
    ev[0].record(ts)
    for _ in range(reps):
        batch.replay(stream.handle)
    ev[1].record(ts)
    stream.synchronize()
    persistent_s = ev[0].elapsed_time(ev[1]) / 1e3 / reps
    batch.set_own_launch(0)
    # the library's default own-launch threshold (batch_split: 16 loads of the resident photon
    # slots, 28,672 histories per SM), to report which jobs took launches of their own
    own_min = 28672 * torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    # the same jobs as separate single-simulation launches
    ev2 = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    ev2[0].record(ts)
    for j, (sc, (ph, src, tl)) in enumerate(zip(jobs, objs)):
        tl.reset(stream.handle)
        # the single-job default launch shape (a batch may tune to blocks a single job cannot take)
        M.run(tables, ph, src, tl, sc.n_histories, seed=1 + j, first=0, precision="mixed", stream=stream.handle)
    ev2[1].record(ts)
    stream.synchronize()
    seq_s = ev2[0].elapsed_time(ev2[1]) / 1e3
    h = batch.histories
    out = {"workload": "%d jobs, edge 32-256 voxels at 1 mm, 20-120 kVp, histories log-uniform 1e5-1e8 x %g"
                       % (args.batch_jobs, args.batch_scale),
           "histories_per_replay": h, "value": h / graph_s, "unit": UNIT, "ms_per_replay": 1e3 * graph_s,
           "separate_launches_value": h / seq_s, "autotuned_launch": launch, "autotune_trial_rate": tuned_rate,
           "own_launch_jobs": sum(1 for sc in jobs if sc.n_histories >= own_min),
           "own_launch_min_histories": own_min,
           "own_launch_histories": sum(sc.n_histories for sc in jobs if sc.n_histories >= own_min),
           "all_jobs_in_the_persistent_launch_value": h / persistent_s,
           "replays_timed": reps}
    batch.close()
    if not args.batch_pair:
        stream.close()
        return out
    # plain FP64 and mixed on the same jobs (histories x fp64_scale, so that the FP64 runs stay
    # short): batched under a graph and as separate launches, each precision with its own tallies
    scale64 = args.batch_fp64_scale
    small = scenes.batch_jobs(n_jobs=args.batch_jobs, seed=1, hist_scale=args.batch_scale * scale64)
    pair = {"histories_scale": args.batch_scale * scale64}
    for prec in ("fp64", "mixed"):
        tls = [M.Tallies(ph, sc.specs, sc.dose_mode) for sc, (ph, _, _) in zip(small, objs)]
        b = M.Batch(tables, [(ph, src, tl, 1 + j, 0, sc.n_histories)
                             for j, (sc, (ph, src, _), tl) in enumerate(zip(small, objs, tls))])
        lp = {}
        if args.batch_autotune:
            lp, _ = b.autotune(prec, trial=1_000_000 if prec == "fp64" else 4_000_000, stream=stream.handle)
        b.capture(stream.handle, prec, **lp)
        b.replay(stream.handle)
        stream.synchronize()
        ev[0].record(ts)
        b.replay(stream.handle)
        ev[1].record(ts)
        stream.synchronize()
        g_s = ev[0].elapsed_time(ev[1]) / 1e3
        ev2[0].record(ts)
        for j, (sc, (ph, src, _), tl) in enumerate(zip(small, objs, tls)):
            tl.reset(stream.handle)
            M.run(tables, ph, src, tl, sc.n_histories, seed=1 + j, first=0, precision=prec, stream=stream.handle)
        ev2[1].record(ts)
        stream.synchronize()
        s_s = ev2[0].elapsed_time(ev2[1]) / 1e3
        pair[prec] = {"histories": b.histories, "batched_value": b.histories / g_s,
                      "separate_launches_value": b.histories / s_s, "autotuned_launch": lp}
        b.close()
        for tl in tls:
            tl.close()
    pair["mixed_batched_over_fp64_separate"] = pair["mixed"]["batched_value"] / pair["fp64"]["separate_launches_value"]
    pair["mixed_batched_over_fp64_batched"] = pair["mixed"]["batched_value"] / pair["fp64"]["batched_value"]
    out["fp64_pair_same_jobs"] = pair
    stream.close()
    return out


def serving_leg(args):
    """The serving mix (70% 64^3 dose 1e6, 25% 128^3 dose 1e7, 5% 256x256x128 radiography with
    a 256^2 detector 1e8) as a seeded Poisson stream at 200 requests/s, then at 80% of the
    request rate the server sustained."""
    from midsx_gb300 import scenes, serving
    t0 = time.time()
    tmpl = scenes.serving_templates(pool=4, seed=1)
    mix = serving.Mix(tmpl)
    log("serving setup %.1fs" % (time.time() - t0))
    # warm-up: one request of each class
    warm = [dict(t=0.0, cls=c[0], template=0, n=200_000, seed=999 + k, first=0)
            for k, c in enumerate(scenes.SERVING_CLASSES)]
    serving.drive(mix, warm)
    # the kernel rate of the mix: one request of each class run alone (midsx_gpu_run, device
    # events), weighted by the classes' histories in the stream
    import torch
    import midsx_gb300 as M
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    class_rate = {}
    for name, _, n in scenes.SERVING_CLASSES:
        sc = tmpl[name][0]
        t = mix.tables[tuple(sc.materials)]
        ph = M.Phantom(t, sc.domain, sc.spacing, sc.origin, sc.ids, sc.background)
        tl = M.Tallies(ph, sc.specs, sc.dose_mode)
        src = M.Source(**sc.source)
        M.run(t, ph, src, tl, min(n, 2_000_000), seed=5, precision="mixed")
        tl.reset()
        ev[0].record()
        M.run(t, ph, src, tl, n, seed=6, precision="mixed")
        ev[1].record()
        torch.cuda.synchronize()
        class_rate[name] = n / (ev[0].elapsed_time(ev[1]) / 1e3)
        tl.close()
        ph.close()
    reqs = scenes.serving_requests(rate=200.0, n_requests=args.serving_requests, seed=1)
    mix_hist = {c: sum(r["n"] for r in reqs if r["cls"] == c) for c in class_rate}
    kernel_rate = sum(mix_hist.values()) / sum(mix_hist[c] / class_rate[c] for c in class_rate)
    hot = serving.drive(mix, reqs)
    mean_h = hot["histories"] / hot["requests"]
    rate = max(1.0, 0.8 * hot["histories_per_s"] / mean_h)
    reqs2 = scenes.serving_requests(rate=rate, n_requests=max(20, args.serving_requests // 2), seed=2)
    calm = serving.drive(mix, reqs2)
    mix.close()

    def brief(d, lam):
        s = d["server"]
        return {"rate_req_per_s": lam, "requests": d["requests"], "failed": d["failed"],
                "step_cap_hits": d["step_cap_hits"], "compton_cap_hits": d["compton_cap_hits"],
                "histories_per_s": d["histories_per_s"], "offered_histories_per_s": d["offered_histories_per_s"],
                "latency_ms": d["latency_ms"], "server_latency_ms": d["server_latency_ms"],
                "by_class": d["by_class"], "launches": s["launches"], "max_active": s["max_active_seen"],
                "peak_hbm_bytes": s["peak_bytes_in_use"], "gpu_busy_s": s["busy_seconds"]}

    return {"workload": "poisson mix: 70% 64^3 dose 1e6, 25% 128^3 dose 1e7, 5% 256x256x128 radiography "
                        "256^2 detector 1e8 (mixed precision)",
            "kernel_rate_of_the_mix": {"value": kernel_rate, "unit": UNIT, "per_class": class_rate,
                                       "how": "one request of each class alone, weighted by the stream's histories"},
            "at_200_req_per_s": brief(hot, 200.0), "at_sustainable_rate": brief(calm, rate)}


def _run_host(M, N, tables, geom, ids_pinned, src_spec, sc, cfg, dose_pinned):
    import ctypes as C
    st = N.RunStats()
    arr = M.tally_specs(sc.specs)
    N.check(N.load().midsx_gpu_run_host(tables.handle, C.byref(geom), C.c_void_p(ids_pinned.data_ptr()),
                                        C.byref(src_spec), arr, len(sc.specs), int(sc.dose_mode), C.byref(cfg),
                                        C.cast(C.c_void_p(dose_pinned.data_ptr()), N.PD), C.byref(st)),
            "midsx_gpu_run_host")
    return st


if __name__ == "__main__":
    main()
