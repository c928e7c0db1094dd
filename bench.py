#!/usr/bin/env python
"""Benchmark: 512^3 all-triangle bispectra per second on GB300.

Workload (one "step" = one full bispectrum of one mesh):
  512^3 float32 lognormal mesh, L = 1000 Mpc/h, shells of width 2 k_f from
  k_f to k_Nyq/2 (63 shells), all 24 305 auto triangle bins; the step runs
  r2c of the mesh -> shell filter + batched c2r of 63 shells -> bf16 split ->
  tcgen05 bf16x3 triple-product contraction -> FP64 normalisation by the
  cached triangle counts.  Grid information (N_tri, k_mean) depends only on
  the binning and is computed once before timing ("warm"); its one-off cost is
  reported under "cold".

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Under torchrun (N > 1) every rank measures its own meshes (replicas, no
collective on the data path); the time is the max over ranks.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "512³ all-tri bispectra/s, bf16x3 vs FP32 at ≤1e-5 rel err; serve p50/p99 ms"
# name -> (Nmesh, BoxSize, kmax in units of k_f, dk in units of k_f, description)
WORKLOADS = {
    "mesh512_all": (512, 1000.0, 128.0, 2,
                    "512^3 all-triangle auto bispectrum: L=1000 Mpc/h, 63 shells dk=2kf from kf "
                    "to kNyq/2, 24305 bins, lognormal float32 mesh (seed 1+rank), grid info "
                    "cached"),
    "mesh256_all": (256, 500.0, 64.0, 2,
                    "256^3 all-triangle auto bispectrum: L=500 Mpc/h, 31 shells dk=2kf from kf "
                    "to kNyq/2, 3321 bins, lognormal float32 mesh (seed 1+rank), grid info "
                    "cached"),
    "mesh1024_all": (1024, 2000.0, 0.3 * 512, 4,
                     "1024^3 all-triangle auto bispectrum: L=2000 Mpc/h, 38 shells dk=4kf from "
                     "kf to 0.3 kNyq, 5833 bins, lognormal float32 mesh (seed 1+rank), grid "
                     "info cached"),
    # the headline's 384-point contraction grid with 15 shells (k from 7 kf in steps of 8 kf):
    # a small case of the same field-synthesis kernels for multi-pass profiler captures
    "mesh512_dk8": (512, 1000.0, 128.0, 8,
                    "512^3 all-triangle auto bispectrum: L=1000 Mpc/h, 15 shells dk=8kf from 7kf "
                    "to kNyq/2, 477 bins, lognormal float32 mesh (seed 1+rank), grid info cached",
                    7.0),
}
NMESH, BOX = 512, 1000.0
WORKLOAD = WORKLOADS["mesh512_all"][4]


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="bf16x3")
    ap.add_argument("--workload", default="mesh512_all", choices=sorted(WORKLOADS),
                    help="mesh512_all is the headline; the others are smaller/larger cases "
                         "of the same estimator (profiling, the 1024^3 grid)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp32", action="store_true")
    ap.add_argument("--no-precision", action="store_true",
                    help="skip the per-bin error study against the FP64 GPU contraction")
    ap.add_argument("--serve-requests", type=int, default=2000,
                    help="requests of the serving leg (0 = skip)")
    ap.add_argument("--serve-rate", type=float, default=SERVE_RATE,
                    help="Poisson arrival rate, req/s")
    ap.add_argument("--serve-small", action="store_true",
                    help="serving mix without N=512 (weights renormalised)")
    ap.add_argument("--serve-sweep", default="20,40,80,160,320,640",
                    help="offered rates of the bf16x3 p99-vs-rate sweep ('' = none)")
    ap.add_argument("--serve-sweep-requests", type=int, default=300)
    ap.add_argument("--serve-only", action="store_true", help="run only the serving leg")
    ap.add_argument("--precision-study", action="store_true",
                    help="run only the 512^3 cross-bispectrum precision study (equilateral, "
                         "isosceles m=2, squeezed bins; fp32/bf16/bf16x3 vs the FP64 contraction)")
    ap.add_argument("--precision-out", default=None,
                    help="with --precision-study: write the per-bin errors to this JSON file")
    ap.add_argument("--shard", action="store_true",
                    help="under torchrun: split every bispectrum's contraction-grid points over "
                         "the ranks (replicated FFTs, one NCCL all-reduce of the T partial "
                         "sums); the line reports strong scaling")
    ap.add_argument("--no-studies", action="store_true",
                    help="skip the 512^3 cross precision study and the 1024^3 resident / "
                         "streamed runs that the headline line carries")
    ap.add_argument("--grid", default="reduced", choices=["reduced", "single", "native"],
                    help="contraction grid of the headline plan: reduced (grid levels), "
                         "single (the reduced grid for every bin) or native")
    ap.add_argument("--no-cold", action="store_true",
                    help="profiling runs only: skip the one-off FP64 grid information and "
                         "normalise by 1 (same kernels and timings in the step)")
    return ap.parse_args()


def guarded_leg(name, fn):
    """Run one extra leg of the bench line; a failure is recorded in the line (and on stderr)
    instead of losing the headline measurement."""
    t0 = time.perf_counter()
    try:
        out = fn()
    except Exception as e:  # the headline line must still be printed
        import traceback
        traceback.print_exc()
        out = {"error": "%s: %s" % (type(e).__name__, e)}
    # release what the leg left behind before the next leg sizes its memory
    import gc
    gc.collect()
    if "torch" in sys.modules:
        import torch
        if torch.cuda.is_available():
            torch.cuda.empty_cache()
    sys.stderr.write("leg %s: %.1f s\n" % (name, time.perf_counter() - t0))
    return out


def shard_step(plan, tset, ntri, precision, group=None):
    """One bispectrum split over the process group's ranks: this rank contracts its range of
    contraction-grid points, the FP64 partial vectors are summed by one all-reduce (bskit's
    slab sums with gather + bcast, main.py:1875-1879), and every rank normalises."""
    from bskit_gb300.sharding import sharded_measure_b
    b = sharded_measure_b(plan, tset, precision=precision, group=group)
    return plan.normalize(b, ntri)


def select_workload(name):
    global NMESH, BOX, WORKLOAD
    NMESH, BOX, WORKLOAD = WORKLOADS[name][0], WORKLOADS[name][1], WORKLOADS[name][4]


def workload_bins(name="mesh512_all"):
    from bskit_gb300 import bins
    n, box, kmax, dk = WORKLOADS[name][:4]
    kmin = WORKLOADS[name][5] if len(WORKLOADS[name]) > 5 else 1.0
    kf = 2 * math.pi / box
    kw = dict(kmin=kmin * kf, kmax=kmax * kf, dk=dk * kf)
    return bins.generate_bin_edge_list(**kw), bins.generate_triangle_bin_list(return_indices=True,
                                                                              **kw)


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return d, "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, \
            "fallback"


class ClockSampler(object):
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region.

    start() launches the sampler and waits (up to 5 s) for its first row, so that the timed
    region that follows is covered from its beginning; mark() records where the timed region
    begins; stop() keeps the rows taken after the mark.  A region shorter than one sampling
    interval has no row of its own: the row just before it is reported, with
    "samples_in_region": 0."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None
        self.mark_rows = 0

    def _rows(self):
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        return rows

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
            return
        t0 = time.time()
        while time.time() - t0 < 5.0 and not self._rows() and self.proc.poll() is None:
            time.sleep(0.05)

    def mark(self):
        self.mark_rows = len(self._rows()) if self.proc is not None else 0

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = self._rows()
        os.unlink(self.path)
        if not rows:
            return None
        inside = rows[self.mark_rows:]
        n_inside = len(inside)
        if not inside:
            inside = rows[-1:]
        sm = sorted(float(r[1]) for r in inside if r[1].replace(".", "").isdigit())
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in inside:
            for nm, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": sm[len(sm) // 2] if sm else None,
                "sm_max_mhz": (float(inside[0][2]) if inside[0][2].replace(".", "").isdigit()
                               else None),
                "reasons": sorted(reasons), "samples_in_region": n_inside}


def kernel_launches_per_step(plan, ts, slots=(0, 0, 0)):
    """Kernels of libbskit_gb300 launched by one step (cuFFT's R2C kernels excluded): the
    spectrum extraction of each painted slot; per grid level the level's spectrum (levels
    below the plan's grid), the field synthesis (X, Y, Z passes per batch of 8 shells, the
    bf16 split written by the Z pass) and one contraction; the normalisation."""
    nslot = len(set(slots))
    levels = ts.levels()
    n = nslot
    if levels:
        for lv in levels:
            if lv["ngrid"] != plan.ngrid:
                n += nslot
            n += 3 * ((lv["shells"] + 7) // 8) * nslot + 1
    else:
        n += 3 * ((plan.n_shells + 7) // 8) * nslot + 1 + 1  # synthesis, contraction, scale
    return n + 1


def run_ours(args):
    import numpy as np
    import torch

    from bskit_gb300 import synthetic
    from bskit_gb300.engine import Plan

    world, rank, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
        sys.stderr.write("rank %d/%d: process group %s on cuda:%d%s\n"
                         % (rank, world, dist.get_backend(), local,
                            ", point-range shards" if args.shard else ", replicas"))
    else:
        dist = None
        torch.cuda.set_device(0)
    dev = torch.device("cuda", torch.cuda.current_device())

    def barrier():
        if dist is not None:
            dist.barrier()

    edges, tri = workload_bins(args.workload)
    plan = Plan(NMESH, BOX, edges, grid=args.grid, device=dev)
    ts = plan.triangles(tri)
    # replicas measure their own meshes; shards split one mesh's bispectrum
    seed = 1 if args.shard else 1 + rank
    delta = synthetic.lognormal_mesh_torch(NMESH, BOX, seed=seed, device=dev).contiguous()
    torch.cuda.synchronize()

    # ---- cold: grid information (FP64), once
    t0 = time.perf_counter()
    if args.no_cold:
        ntri = torch.ones(len(tri), dtype=torch.float64, device=dev)
        cold_gridinfo_s = None
    else:
        ntri, kmean = plan.gridinfo(ts)
        plan.sync_check()
        cold_gridinfo_s = time.perf_counter() - t0

    stream = torch.cuda.current_stream()
    prec = args.precision

    def step(p=prec):
        plan.paint(0, delta)
        if args.shard:  # this rank's point range, then the all-reduce of the T partial sums
            return shard_step(plan, ts, ntri, p)
        b = plan.measure_b(ts, precision=p)
        return plan.normalize(b, ntri)

    def timed(fn, k, w):
        for _ in range(w):
            fn()
        plan.sync_check()
        barrier()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(k):
            out = fn()
        e1.record(stream)
        torch.cuda.synchronize()
        barrier()
        ms = e0.elapsed_time(e1)
        if dist is not None:
            t = torch.tensor([ms], device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms = float(t.item())
        return ms, out

    clocks = ClockSampler(dev.index)
    for _ in range(args.warmup):
        step()
    plan.sync_check()
    clocks.start()
    clocks.mark()
    ms, bn = timed(step, args.steps, 0)
    clk = clocks.stop()
    plan.sync_check()
    ms_step = ms / args.steps
    # replicas: every rank measures its own bispectra; shards: the ranks measure one together
    per_step = 1 if args.shard else world
    value = per_step * args.steps / (ms / 1e3)

    # ---- end to end through the public API: pinned host mesh in, B to host each step.
    # The host->device copy of step k+1 runs on a copy stream while step k computes
    # (double-buffered device meshes); every copy of a timed step is issued after the
    # start event, and the stop event follows the last step's device->host read.
    host = delta.cpu().pin_memory()
    bufs = [torch.empty_like(delta), torch.empty_like(delta)]
    out_host = torch.empty(len(tri), dtype=torch.float64).pin_memory()
    copy_stream = torch.cuda.Stream(device=dev)
    loaded = [torch.cuda.Event(), torch.cuda.Event()]
    free = [torch.cuda.Event(), torch.cuda.Event()]

    def prefetch(k):
        i = k % 2
        copy_stream.wait_event(free[i])  # the paint that last read this buffer is done
        with torch.cuda.stream(copy_stream):
            bufs[i].copy_(host, non_blocking=True)
            loaded[i].record(copy_stream)

    def run_e2e(n):
        copy_stream.wait_stream(stream)
        prefetch(0)
        for k in range(n):
            i = k % 2
            stream.wait_event(loaded[i])
            plan.paint(0, bufs[i])
            free[i].record(stream)
            if k + 1 < n:
                prefetch(k + 1)
            if args.shard:
                out_host.copy_(shard_step(plan, ts, ntri, prec), non_blocking=True)
            else:
                b = plan.measure_b(ts, precision=prec)
                out_host.copy_(plan.normalize(b, ntri), non_blocking=True)

    run_e2e(2)
    plan.sync_check()
    barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    run_e2e(args.steps)
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    e2e_ms = e0.elapsed_time(e1)
    if dist is not None:
        t = torch.tensor([e2e_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_ms = float(t.item())
    e2e_value = per_step * args.steps / (e2e_ms / 1e3)
    host_check = out_host.clone()

    # ---- contraction alone (fields and split cached): the dominant kernel
    plan.paint(0, delta)
    step()
    torch.cuda.synchronize()
    reps = 5
    c_ms, b_tc = timed(lambda: plan.measure_b(ts, precision=prec), reps, 1)
    c_ms /= reps
    ng = plan.ngrid
    # the contraction's work: 2 flops per bin and point of the grid the bin is contracted on
    # (grid levels: bins of small shells on smaller grids); the single reduced grid's work
    # 2 T Ng^3 is reported beside it
    levels = ts.levels()
    single_flops = 2.0 * len(tri) * float(ng) ** 3
    algo_flops = (sum(2.0 * lv["bins"] * float(lv["ngrid"]) ** 3 for lv in levels)
                  if levels else single_flops)
    sched_cols = None
    peaks, peak_kind = measured_peaks()
    peak = float(peaks.get("bf16_tflops_sustained", 1700.0))
    achieved = algo_flops / (c_ms / 1e3) / 1e12
    # MMA work the kernel issues: per grid point, for every tile, 128 rows x (2 nc + nc)
    # (bf16x3: hi x [Bhi; Blo] and lo x Bhi) multiply-adds
    tiles, sum_nc, pair_rows = ts.schedule()
    terms = 3 if prec == "bf16x3" else 1
    if levels:
        issued_flops = sum(2.0 * 128 * terms * lv["sum_nc"] * float(lv["ngrid"]) ** 3
                           for lv in levels)
        tiles = sum(lv["tiles"] for lv in levels)
        sum_nc = sum(lv["sum_nc"] for lv in levels)
        pair_rows = sum(lv["pair_rows"] for lv in levels)
        useful = algo_flops / (2.0 * 128 * sum(lv["sum_nc"] * float(lv["ngrid"]) ** 3
                                               for lv in levels))
    else:
        issued_flops = 2.0 * 128 * terms * sum_nc * float(ng) ** 3
        useful = len(tri) / (128.0 * sum_nc)
    issued = {"flops_per_launch": issued_flops,
              "tflops": issued_flops / (c_ms / 1e3) / 1e12,
              "frac": issued_flops / (c_ms / 1e3) / 1e12 / peak,
              "tiles": tiles, "sum_nc": sum_nc, "pair_rows": pair_rows,
              "useful_fraction": useful}
    traffic = None  # the committed DRAM capture is of a single-grid launch
    if not levels:
        try:
            with open(os.path.join(ROOT, "profiles", "contract_tc_traffic.json")) as f:
                tr = json.load(f)
            traffic = tr.get("bytes_per_launch", {}).get(args.workload)
        except Exception:
            pass

    # ---- plain FP32 path on the same workload, and agreement with it
    fp32 = None
    if not args.no_fp32:
        k32 = max(1, min(args.steps, 3))
        ms32, b32 = timed(lambda: step("fp32"), k32, 1)
        bref = b32.double().cpu().numpy()
        bt = bn.double().cpu().numpy()
        rel = np.abs(bt - bref) / np.abs(bref)
        # the plain FP32 contraction alone (fields cached), against the FP32 SIMT peak
        plan.paint(0, delta)
        step()
        torch.cuda.synchronize()
        c32_ms, _ = timed(lambda: plan.measure_b(ts, precision="fp32"), reps, 1)
        c32_ms /= reps
        props = torch.cuda.get_device_properties(dev)
        fp32_peak = props.multi_processor_count * 128 * 2 * float(peaks.get("sm_max_mhz", 2070.0)) / 1e6
        fp32 = {"value": world * k32 / (ms32 / 1e3), "ms_per_step": ms32 / k32,
                "contraction": {"kernel": "contract_f32_kernel (FP32 SIMT)",
                                "launch_ms": c32_ms,
                                "achieved_tflops": algo_flops / (c32_ms / 1e3) / 1e12,
                                "peak_tflops": fp32_peak,
                                "frac": algo_flops / (c32_ms / 1e3) / 1e12 / fp32_peak,
                                "peak_source": "nominal: SMs x 128 FP32 lanes x 2 x max SM clock",
                                "tensor_kernel_speedup": c32_ms / c_ms},
                "bf16x3_vs_fp32_rel_err": {"max": float(np.nanmax(rel)),
                                           "median": float(np.nanmedian(rel)),
                                           "p99": float(np.nanpercentile(rel, 99))}}

    # ---- per-bin error of bf16x3 / fp32 / bf16 against the FP64 contraction of the same fields
    precision = None
    if not args.no_precision:
        plan.paint(0, delta)
        b64 = plan.measure_b(ts, precision="fp64")
        absf = torch.stack([plan.field(0, s).abs().reshape(-1) for s in range(len(edges))])
        babs = plan.contract(ts, absf, absf, absf, precision="fp64") * (BOX ** 6 / float(ng) ** 3)
        del absf
        torch.cuda.empty_cache()

        live = (babs > 0) & (b64 != 0)  # bins with at least one closed triangle
        over = {}

        def err_stats(name, b):
            err = (b - b64).abs()[live]
            nrm = err / babs[live]
            rel = err / b64[live].abs()
            well = b64[live].abs() >= 0.1 * babs[live]
            over[name] = rel > 1e-5
            ratio = (b64[live].abs() / babs[live])[over[name]]
            return {"max_normalised": float(nrm.max()), "max_rel": float(rel.max()),
                    "max_rel_well_conditioned": float(rel[well].max()) if bool(well.any()) else None,
                    "median_rel": float(rel.median()), "p99_rel": float(rel.quantile(0.99)),
                    "n_bins_rel_gt_1e-5": int(over[name].sum()),
                    "max_abs_over_abs_sum_of_those": float(ratio.max()) if ratio.numel() else None,
                    "well_conditioned_bins": int(well.sum()), "bins": int(live.sum())}

        precision = {"reference": "FP64 SIMT contraction of the same FP32 shell fields "
                                  "(every bin; the oracle comparison of sampled bins is "
                                  "tests/test_gpu_configs.py)",
                     "normalised": "|B - B64| / (L^6/Ng^3 sum |I_i I_j I_l|)",
                     "well_conditioned": "|B64| >= 0.1 * L^6/Ng^3 sum |I_i I_j I_l|"}
        for p_ in ("bf16x3", "fp32", "bf16"):
            precision[p_] = err_stats(p_, plan.measure_b(ts, precision=p_))
        plan.sync_check()
        both = over["bf16x3"] & over["fp32"]
        precision["bf16x3_over_1e-5_also_fp32_over_1e-5"] = int(both.sum())
        precision["bf16x3_over_1e-5_where_fp32_within"] = int((over["bf16x3"] & ~over["fp32"]).sum())

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = guarded_leg("cpu_baseline", lambda: cpu_sampled(delta.cpu().numpy(), edges, tri))
        if args.workload == "mesh512_all" and "error" not in cpu:
            cpu["full_256"] = guarded_leg("cpu_full_256", cpu_full_256)

    line = {
        "metric": METRIC,
        "value": value,
        "unit": "bispectra/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_step,
        "higher_is_better": True,
        "scaling": "strong" if args.shard else "weak",
        "vs_baseline": None,
        "dtype": prec,
        "data": "synthetic lognormal mesh (seeded), no dataset",
        "config": {"workload": WORKLOAD, "workload_name": args.workload, "nmesh": NMESH,
                   "box": BOX, "n_shells": len(edges),
                   "n_bins": int(len(tri)), "precision": prec, "contraction_grid": ng,
                   "grid_mode": args.grid,
                   "grid_levels": [lv["ngrid"] for lv in ts.levels()],
                   "l2": "inputs larger than L2 (mesh %d MiB, shell fields %.1f GiB)"
                         % (NMESH ** 3 * 4 >> 20, len(edges) * ng ** 3 * 4 / 2 ** 30),
                   "parallelism": ("point-range shards of one bispectrum over %d GPUs, NCCL "
                                   "all-reduce of the T partial sums" % world) if args.shard
                   else ("replicas" if world > 1 else "single GPU")},
        "e2e": {"value": e2e_value, "unit": "bispectra/s",
                "h2d_bytes_per_step": int(host.numel() * 4),
                "d2h_bytes_per_step": int(out_host.numel() * 8),
                "ms_per_step": e2e_ms / args.steps,
                "pipelining": "next step's H2D copy overlaps this step's compute (copy stream, "
                              "two device buffers)",
                "result_matches_device_step": bool(torch.allclose(
                    host_check, bn.detach().cpu().double(), rtol=1e-9, atol=0))},
        "gpu_launches": kernel_launches_per_step(plan, ts) * args.steps,
        "roofline": {"kernel": "contract_tc_kernel (tcgen05 bf16x3)", "bound": "tensor",
                     "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "peak_source": "%s bf16_tflops_sustained" % peak_kind,
                     "algorithmic_flops_per_launch": algo_flops,
                     "single_grid_flops_per_launch": single_flops,
                     "grid_levels": levels,
                     "launch_ms": c_ms,
                     "issued": issued},
        "cpu_baseline": cpu,
        "clocks": clk,
        "cold": {"gridinfo_s": cold_gridinfo_s},
        "fp32_plain": fp32,
        "precision_vs_fp64": precision,
    }
    if fp32:
        line["speedup_vs_fp32_plain"] = value / fp32["value"]
    studies = world == 1 and args.workload == "mesh512_all" and not args.no_studies
    if studies or (args.serve_requests > 0 and world == 1):
        plan.close()
        del delta, host, bufs
        torch.cuda.empty_cache()
    if studies:
        for key, fn in (("precision_study", precision_study), ("mesh1024", mesh1024_study)):
            line[key] = guarded_leg(key, lambda fn=fn: fn(args, dev))
            torch.cuda.empty_cache()
    if args.serve_requests > 0 and world == 1:
        sweep = [float(v) for v in args.serve_sweep.split(",") if v.strip()]
        line["serving"] = guarded_leg("serving", lambda: run_serving(args, dev, sweep=sweep))
        if "error" not in line["serving"]:
            line["serving"]["p99_bound_ms"] = SERVE_P99_BOUND_MS
            line["serving"]["p99_within_bound"] = bool(
                line["serving"].get("p99_ms", 1e30) <= SERVE_P99_BOUND_MS)
        if not args.no_fp32:
            torch.cuda.empty_cache()
            line["serving_fp32"] = guarded_leg(
                "serving_fp32", lambda: run_serving(args, dev, precision="fp32"))
    if rank == 0:
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


SERVE_SIZES = [64, 128, 256, 512]
SERVE_WEIGHTS = [0.4, 0.3, 0.2, 0.1]
SERVE_RATE = 40.0          # req/s of the stated operating point (cfg4 mix)
SERVE_P99_BOUND_MS = 400.0  # stated p99 bound at that rate (bf16x3)


def run_serving(args, dev, precision="bf16x3", sweep=()):
    """Continuous-batching leg: seeded Poisson stream of mixed bispectrum requests.

    Mix (the serving configuration): N in {64, 128, 256, 512} with weights
    {.4, .3, .2, .1}, 30% cross <AAB>, bin set uniform over {all triangles dk=2kf
    to kNyq/2, equilateral, squeezed with k1 in [kf, 3kf] (index 0)}, L = 100 Mpc/h,
    lognormal meshes (a seeded pool per N), ``--serve-requests`` requests at
    ``--serve-rate`` req/s.  ``--serve-small`` drops N = 512 (weights renormalised).
    Before the stream, ``Scheduler.prepare`` admits the groups and captures every
    (instance, bin set) graph and computes every grid information, so nothing of
    that sits on the dispatch path; latency = arrival to result on the host.
    ``sweep``: further offered rates, ``--serve-sweep-requests`` requests each, for
    the p99-vs-rate curve.
    """
    import numpy as np
    import torch

    from bskit_gb300 import serving, synthetic
    sizes = SERVE_SIZES[:3] if args.serve_small else SERVE_SIZES
    w = np.array(SERVE_WEIGHTS[:len(sizes)])
    w = w / w.sum()
    box = 100.0
    kf = 2 * np.pi / box
    pool = {}
    for n in sizes:
        k = {64: 8, 128: 8, 256: 4, 512: 2}[n]
        pool[n] = [synthetic.lognormal_mesh_torch(n, box, seed=1000 * n + i, device=dev)
                   .cpu().pin_memory() for i in range(k)]
    torch.cuda.synchronize()
    sets = ["all", "equilateral", "squeezed"]

    def spec_of(n, kind):
        return dict(kmin=kf, kmax=n / 4 * kf, dk=2 * kf, triangle_type=kind,
                    squeezed_bin_index=0)

    def stream(rng, n_req, rate):
        gaps = rng.exponential(1.0 / rate, size=n_req)
        reqs = []
        for i, t in enumerate(np.cumsum(gaps)):
            n = int(rng.choice(sizes, p=w))
            kind = sets[int(rng.integers(3))]
            cross = rng.random() < 0.3
            p = pool[n]
            second = p[(i + 1) % len(p)] if cross else None
            reqs.append(serving.Request(i, p[i % len(p)], box, spec_of(n, kind), second=second,
                                        arrival=t, precision=precision))
        return reqs

    server = serving.make_server(max_batch=4, device=dev)
    try:
        return _serve_legs(args, server, serving, pool, sizes, w, box, sets, spec_of, stream,
                           precision, sweep)
    finally:
        server.close()


def _serve_legs(args, server, serving, pool, sizes, w, box, sets, spec_of, stream, precision,
                sweep):
    import numpy as np
    warm = [serving.Request(-1, pool[n][0], box, spec_of(n, kind),
                            second=pool[n][1] if cross else None, precision=precision)
            for n in sizes for kind in sets for cross in (False, True)]
    t0 = time.perf_counter()
    for n in sorted(sizes, reverse=True):  # ahead of the stream, largest grid first
        # every group the scheduler may admit for N <= 256 (small), one for 512^3 (~30 GB)
        server.prepare([r for r in warm if r.nmesh == n], groups=1 if n >= 512 else None)
    server.run(warm, realtime=False)
    prep_s = time.perf_counter() - t0

    def serve(reqs):
        server.done = []
        cap0 = server.backend.captures_at_dispatch
        by0 = dict(server.backend.captures_at_dispatch_by_n)
        log0 = len(server.log)
        server.run(reqs, realtime=True)
        st = serving.latency_stats(reqs)
        st["graph_captures_at_dispatch"] = server.backend.captures_at_dispatch - cap0
        st["graph_captures_at_dispatch_by_n"] = {
            str(n): c - by0.get(n, 0) for n, c in server.backend.captures_at_dispatch_by_n.items()
            if c - by0.get(n, 0)}
        ev = {}
        for e in server.log[log0:]:
            if e[0] in ("admit", "evict"):
                k = "%ss_by_n" % e[0]
                ev.setdefault(k, {})
                ev[k][str(e[1][0])] = ev[k].get(str(e[1][0]), 0) + 1
        st.update(ev)
        return st

    rng = np.random.default_rng(2024)
    stats = serve(stream(rng, args.serve_requests, args.serve_rate))
    stats.update({"rate_rps": args.serve_rate,
                  "mix": "N %s, weights %s, 30%% cross, all/equilateral/squeezed"
                         % (sizes, [round(float(x), 3) for x in w]),
                  "prepare_s": prep_s, "precision": precision, "max_batch": 4,
                  "batching": "per shell set (N, box, shell list), bin sets mixed",
                  "resident_groups": len(server.groups),
                  "prepared_groups_by_n": {str(n): sum(1 for g in server.groups
                                                       if g.shell_key[0] == n
                                                       and getattr(g, "pinned", False))
                                           for n in sizes}})
    if sweep:
        curve = []
        for rate in sweep:
            st = serve(stream(np.random.default_rng(int(rate)), args.serve_sweep_requests, rate))
            curve.append({"rate_rps": rate, "p50_ms": st.get("p50_ms"), "p99_ms": st.get("p99_ms"),
                          "throughput_rps": st.get("throughput_rps")})
            if st.get("throughput_rps", 0.0) < 0.8 * rate:
                break  # saturated: served well below the offered rate
        ok = [c["rate_rps"] for c in curve if c["p99_ms"] is not None
              and c["p99_ms"] <= SERVE_P99_BOUND_MS and c["throughput_rps"] >= 0.9 * c["rate_rps"]]
        stats["sweep"] = {"requests_per_rate": args.serve_sweep_requests, "curve": curve,
                          "knee_rps": max(ok) if ok else None,
                          "knee": "highest offered rate served at >= 90%% of the rate with "
                                  "p99 <= %.0f ms" % SERVE_P99_BOUND_MS}
    return stats


def precision_study(args, dev):
    """512^3 cross bispectrum <d1 d1 d2>, d1 lognormal (L = 1000 Mpc/h, seed 1), d2 =
    1.5 d1 + white noise of variance 0.1 var(d1) (seed 2); bins of width 2 k_f from k_f
    to k_Nyq/2: equilateral, isosceles m = 2 (tolerance 0.1) and squeezed with k1 in
    [k_f, 3 k_f] (squeezed_bin_index 0).  Each precision is compared bin by bin with the
    FP64 SIMT contraction of the same FP32 shell fields; returns the record."""
    import numpy as np
    import torch

    from bskit_gb300 import bins, synthetic
    from bskit_gb300.engine import Plan

    n, box = 512, 1000.0
    kf = 2 * math.pi / box
    kw = dict(kmin=kf, kmax=128 * kf, dk=2 * kf)
    edges = bins.generate_bin_edge_list(**kw)
    sets = {
        "equilateral": bins.generate_equilateral_triangle_bin_list(return_indices=True, **kw),
        "isosceles_m2": bins.generate_isosceles_triangle_bin_list(isos_mult=2, isos_tol=0.1,
                                                                  return_indices=True, **kw),
        "squeezed_k1_kf_3kf": bins.generate_squeezed_triangle_bin_list(
            squeezed_bin_index=0, return_indices=True, **kw),
    }
    d1 = synthetic.lognormal_mesh_torch(n, box, seed=1, device=dev).contiguous()
    d2 = synthetic.noisy_copy_torch(d1, seed=2).contiguous()
    plan = Plan(n, box, edges, device=dev)
    plan.paint(0, d1)
    plan.paint(1, d2)
    ng = plan.ngrid
    scale = box ** 6 / float(ng) ** 3
    a1 = torch.stack([plan.field(0, s_).abs().reshape(-1) for s_ in range(len(edges))])
    a2 = torch.stack([plan.field(1, s_).abs().reshape(-1) for s_ in range(len(edges))])
    out, per_bin = {}, {}
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    for name, tri in sets.items():
        ts = plan.triangles(tri)
        b64 = plan.measure_b(ts, slots=(0, 0, 1), precision="fp64")
        babs = plan.contract(ts, a1, a1, a2, precision="fp64") * scale
        live = (babs > 0) & (b64 != 0)
        res = {"bins": int(len(tri)), "live_bins": int(live.sum())}
        pb = {"B_fp64": b64.cpu().tolist(), "abs_sum": babs.cpu().tolist()}
        for prec in ("fp32", "bf16", "bf16x3"):
            plan.measure_b(ts, slots=(0, 0, 1), precision=prec)  # warm
            ev[0].record()
            b = plan.measure_b(ts, slots=(0, 0, 1), precision=prec)
            ev[1].record()
            torch.cuda.synchronize()
            err = (b - b64).abs()[live]
            rel = err / b64[live].abs()
            nrm = err / babs[live]
            well = b64[live].abs() >= 0.1 * babs[live]
            res[prec] = {"contraction_ms": ev[0].elapsed_time(ev[1]),
                         "max_rel": float(rel.max()), "median_rel": float(rel.median()),
                         "n_bins_rel_gt_1e-5": int((rel > 1e-5).sum()),
                         "p99_rel": float(rel.quantile(0.99)),
                         "max_rel_well_conditioned": float(rel[well].max()) if bool(well.any())
                         else None,
                         "well_conditioned_bins": int(well.sum()),
                         "max_normalised": float(nrm.max())}
            pb[prec] = b.cpu().tolist()
        plan.sync_check()
        ts.close()
        out[name] = res
        per_bin[name] = pb
    if args.precision_out:
        with open(args.precision_out, "w") as f:
            json.dump({"triangles": {k: np.asarray(v).tolist() for k, v in sets.items()},
                       "per_bin": per_bin}, f)
    rec = {
        "metric": "precision study: per-bin error vs the FP64 contraction of the same fields",
        "config": {"workload": "512^3 cross bispectrum <d1 d1 d2>, L=1000 Mpc/h, d2 = 1.5 d1 + "
                               "noise (0.1 var d1), 63 shells dk=2kf to kNyq/2",
                   "contraction_grid": ng, "slots": "(0, 0, 1)"},
        "reference": "FP64 SIMT contraction of the same FP32 shell fields",
        "normalised": "|B - B64| / (L^6/Ng^3 sum |I_i I_j I_l|)",
        "well_conditioned": "|B64| >= 0.1 * L^6/Ng^3 sum |I_i I_j I_l|",
        "sets": out}
    plan.close()
    del d1, d2, a1, a2
    torch.cuda.empty_cache()
    return rec


def run_precision_study(args):
    import torch
    torch.cuda.set_device(0)
    print(json.dumps(precision_study(args, torch.device("cuda", 0))))


def cpu_sampled(delta_host, edges, tri, steps=None):
    """The reference algorithm on the host cores over its stratified sample: one sampled shell
    per step until every sampled shell was transformed (or ``steps`` steps)."""
    from oracle.cpu_baseline import ReferenceCPU
    ref = ReferenceCPU(delta_host, BOX, edges, tri)
    try:
        t0 = time.perf_counter()
        est = None
        for _ in range(steps or len(ref.shells)):
            est = ref.step()
        return {"value": 1.0 / est, "unit": "bispectra/s", "cores": ref.P, "kind": "port",
                "sample": ref.describe(), "sample_seconds": time.perf_counter() - t0,
                "bins_timed": ref.n_tri, "seconds_per_bispectrum_extrapolated": est}
    finally:
        ref.close()


def cpu_full_256(value_256=None):
    """The reference algorithm in full (every shell, every bin, not extrapolated) on the 256^3
    all-triangle workload (L = 500, 31 shells, 3321 bins, lognormal seed 1), beside the
    sampled estimate of the same workload: the check of the sampled extrapolation."""
    from bskit_gb300 import synthetic
    from oracle.cpu_baseline import ReferenceCPU
    edges, tri = workload_bins("mesh256_all")
    d = synthetic.lognormal_mesh(256, 500.0, seed=1)
    full = ReferenceCPU(d, 500.0, edges, tri, full=True)
    try:
        secs, _ = full.full_run()
        P = full.P
    finally:
        full.close()
    samp = ReferenceCPU(d, 500.0, edges, tri, sample_shells=12)
    try:
        est = None
        for _ in range(len(samp.shells)):
            est = samp.step()
    finally:
        samp.close()
    rec = {"workload": WORKLOADS["mesh256_all"][4], "cores": P, "measured_s": secs,
           "bispectra_per_s": 1.0 / secs, "sampled_estimate_s": est,
           "sampled_over_measured": est / secs,
           "note": "full run: every shell c2r and all 3321 triangle sums, not extrapolated"}
    if value_256:
        rec["gpu_bispectra_per_s"] = value_256
    return rec


def mesh1024_study(args, dev, steps=5):
    """1024^3 all-triangle auto bispectrum (L = 2000 Mpc/h, 38 shells of width 4 k_f to
    0.3 k_Nyq, 5833 bins), bf16x3, normalised by the grid information: resident (reduced
    480^3 grid, every shell field in HBM) and streamed in chunks of 16 shells (a plan budget
    with room for 16-shell buffers only).  Bispectra/s of each, the grid-information time,
    and the largest difference between the two results over the largest |B|."""
    import torch

    from bskit_gb300 import synthetic
    from bskit_gb300.engine import Plan
    edges, tri = workload_bins("mesh1024_all")
    n, box = 1024, 2000.0
    delta = synthetic.lognormal_mesh_torch(n, box, seed=1, device=dev).contiguous()
    stream = torch.cuda.current_stream()

    def run(plan, ts, ntri):
        def step():
            plan.paint(0, delta)
            return plan.normalize(plan.measure_b(ts, precision="bf16x3"), ntri)
        step()
        plan.sync_check()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            b = step()
        e1.record(stream)
        torch.cuda.synchronize()
        plan.sync_check()
        ms = e0.elapsed_time(e1) / steps
        return {"ms_per_step": ms, "bispectra_per_s": 1e3 / ms}, b

    plan = Plan(n, box, edges, device=dev)
    ts = plan.triangles(tri)
    t0 = time.perf_counter()
    ntri, _ = plan.gridinfo(ts)
    plan.sync_check()
    gi_s = time.perf_counter() - t0
    resident, b_res = run(plan, ts, ntri)
    resident["footprint_gb"] = plan.footprint() / 1e9
    ng = plan.ngrid
    plan.close()
    torch.cuda.empty_cache()
    probe = Plan(n, box, edges, device=dev)
    probe.paint(0, delta)
    fp0 = probe.footprint()
    probe.close()
    K = ng ** 3
    # room for 16-shell streaming buffers (16 bytes per point and shell: three FP32 chunks and
    # the bf16 split of one), not for the 40 resident shells and their split (20 x 16 K)
    budget = fp0 + 18 * 16 * K
    sp = Plan(n, box, edges, mem_budget=budget, device=dev)
    ts2 = sp.triangles(tri)
    streamed, b_str = run(sp, ts2, ntri)
    streamed["chunk_shells"] = sp.stream_chunk()
    streamed["budget_gb"] = budget / 1e9
    sp.close()
    ok = ntri > 0
    diff = float(((b_str - b_res).abs()[ok]).max() / b_res[ok].abs().max())
    del delta
    torch.cuda.empty_cache()
    return {"workload": WORKLOADS["mesh1024_all"][4], "contraction_grid": ng,
            "precision": "bf16x3", "gridinfo_s": gi_s, "resident": resident,
            "streamed": streamed, "max_abs_diff_over_max_abs_B": diff, "steps": steps}


def run_reference(args):
    world, rank, local = dist_env()
    if rank != 0:
        return
    import numpy as np

    from bskit_gb300 import synthetic
    from oracle.cpu_baseline import ReferenceCPU

    edges, tri = workload_bins(args.workload)
    delta = synthetic.lognormal_mesh(NMESH, BOX, seed=1)
    ref = ReferenceCPU(delta, BOX, edges, tri)
    try:
        for _ in range(args.warmup):
            ref.step()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            est = ref.step()  # cumulative: every bin and shell timed so far
        wall = time.perf_counter() - t0
        value = 1.0 / est
        line = {
            "impl": "reference", "metric": METRIC, "value": value, "unit": "bispectra/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": est * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic lognormal mesh (seeded)",
            "config": {"workload": WORKLOAD, "nmesh": NMESH, "n_shells": len(edges),
                       "n_bins": int(len(tri)), "parallelism": "%d host processes" % ref.P},
            "cpu_baseline": {"value": value, "unit": "bispectra/s", "cores": ref.P,
                             "kind": "port", "sample": ref.describe()},
            "e2e": {"value": value, "unit": "bispectra/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "sample_wall_s": wall,
            "bins_timed": ref.n_tri,
        }
    finally:
        ref.close()
    if args.workload == "mesh512_all":
        line["full_256"] = cpu_full_256()
    print(json.dumps(line))


def main():
    args = parse()
    select_workload(args.workload)
    if args.impl == "reference":
        run_reference(args)
    elif args.precision_study:
        run_precision_study(args)
    elif args.serve_only:
        import torch
        torch.cuda.set_device(0)
        sweep = [float(r) for r in args.serve_sweep.split(",") if r] if args.serve_sweep else []
        stats = run_serving(args, torch.device("cuda", 0), sweep=sweep)
        print(json.dumps({"metric": "serve p50/p99 latency", "unit": "ms", "serving": stats}))
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
