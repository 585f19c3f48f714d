#!/usr/bin/env python3
"""GWN queries/s on one GB300: the chosen (mixed-precision) form against the plain FP64 kernel.

Workload (the single-large-open-mesh configuration): an icosphere at subdivision level 6 with the triangles of a
30 degree spherical cap removed (76,496 triangles, a 212-segment boundary loop), seeded Gaussian vertex noise
sigma = 1e-3, and a 256^3 grid of float64 queries over the bounding box scaled by 1.2; x0 a seeded unit vector.
One step = the full GWN (LBVH integer term + fractional term) of every query, eval_gwnr_mesh_batch.  The LBVH is
built once before timing, as the reference's intersector is constructed once.

--impl ours (default) prints one JSON line with:
  value       chosen form, queries/s, inputs resident in device memory (403 MB of queries > L2)
  e2e         the same call with pinned host buffers, H2D of the queries and D2H of the result in each step
  plain       the exact FP64 form (reference arithmetic) on the same inputs
  accuracy    max / p99 |chosen - plain| over all queries; both against the CPU oracle on a seeded sample
  roofline    the fractional kernel (the dominant one) against the FP32 FMA rate measured on this GPU
  cpu_baseline  the CPU oracle (a restatement of the reference, all host threads) on a bounded sample
--impl reference prints the reference arm: the CPU oracle with all host threads, one bounded sample per step.
Under torchrun (N > 1) every rank evaluates its own copy of the workload (weak scaling, no collective on the
data path); timing is the max over ranks.
"""

from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "GWN queries/s on 1 GB300: chosen vs plain form at max err<=1e-7 vs FP64 oracle"
WORKLOAD = ("icosphere L6 minus a 30 deg cap (76,496 tris, 212 boundary segments), noise 1e-3, "
            "256^3 float64 query grid over bbox x1.2, full GWN")
FLOPS_PER_PAIR = 53  # algorithmic FP operations per (query, segment) pair, excluding 2 sqrt + 1 atan2


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--grid", type=int, default=256)
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="CPU baseline sample budget")
    ap.add_argument("--plain-steps", type=int, default=2)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--config", choices=["mesh", "cube", "batch", "robust", "param"], default="mesh",
                    help="mesh: the headline single-mesh workload (default); the others are the secondary "
                         "workloads, each printing its own JSON line (see run_secondary)")
    ap.add_argument("--scale", type=float, default=1.0,
                    help="secondary workloads: fraction of the full query count (batch: of the grid side)")
    ap.add_argument("--plain-scale", type=float, default=0.04,
                    help="param workload: the seeded sample of the queries (fraction) on which the plain FP64 "
                         "integrator and the ablations are timed (default 0.04: the plain form on all 1e6 queries "
                         "takes about 100 s per step)")
    ap.add_argument("--labels", type=float, default=1e7,
                    help="param workload: plain-integrator depth labels the proposal network is trained on")
    ap.add_argument("--train-steps", type=int, default=32000, help="param workload: training steps (batch 8192)")
    ap.add_argument("--patches", type=int, default=256, help="param workload: bicubic patches (4 curves each)")
    ap.add_argument("--integer-cells", type=int, choices=[0, 1], default=1,
                    help="mesh workload: 1 looks the integer term's candidates up in the cell grid (default), 0 walks "
                         "the hierarchy (k_traverse); counts are the same")
    ap.add_argument("--batch-config", default=None,
                    help="batch workload: fixed launch configuration 'block,k,seg_tile,stack' instead of tuning")
    ap.add_argument("--full-integer-check", type=int, choices=[0, 1], default=1,
                    help="mesh workload: 1 (default) compares the integer term of every query with the scan of every "
                         "triangle (NaiveIntersector's rule, no hierarchy) and counts the ties; untimed")
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def reduce_max(x: float, device) -> float:
    """The maximum of ``x`` over all ranks (the identity without a process group)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def p99(t) -> float:
    """The 99th percentile of all values of a tensor or array (the ceil(0.99 n)-th smallest)."""
    import torch
    t = (t if isinstance(t, torch.Tensor) else torch.from_numpy(np.asarray(t))).flatten().double()
    if t.numel() == 0:
        return 0.0
    return float(torch.kthvalue(t, max(1, int(np.ceil(0.99 * t.numel())))).values.item())


def workload(grid):
    from antipodal_gb300 import synth
    return synth.open_icosphere(seed=0, level=6, cap_deg=30.0, sigma=1e-3, grid=grid)


# ---- clocks ---------------------------------------------------------------------------------------------------
class Clocks:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.path = tempfile.mktemp(suffix=".csv")
        self.proc = None

    def start(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait(timeout=5)
        self.f.close()
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower().startswith("active")})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ---- CPU side -------------------------------------------------------------------------------------------------
def cpu_rate(oracle, q, x0, verts, idx, bnd, seconds, rng):
    """Times the oracle's full GWN (fractional + naive integer term) with all host threads on a seeded sample
    sized to about ``seconds`` of work.  Returns (queries/s, sample size, threads)."""
    threads = os.cpu_count() or 1
    pilot = q[rng.choice(len(q), size=min(len(q), 4 * threads), replace=False)]
    t0 = time.perf_counter()
    oracle.full_naive(pilot, x0, verts, idx, bnd, threads=threads)
    dt = max(time.perf_counter() - t0, 1e-6)
    m = int(min(len(q), max(len(pilot), len(pilot) * seconds / dt)))
    sample = q[rng.choice(len(q), size=m, replace=False)]
    t0 = time.perf_counter()
    oracle.full_naive(sample, x0, verts, idx, bnd, threads=threads)
    dt = time.perf_counter() - t0
    return m / dt, m, threads


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    from oracle.oracle import Oracle, LIB, build
    if not os.path.exists(LIB):
        build()
    oracle = Oracle()
    verts, idx, bnd, q, x0 = workload(args.grid)
    rng = np.random.default_rng(1)
    threads = os.cpu_count() or 1
    per_step = max(1.0, 60.0 / max(1, args.steps + args.warmup))
    rate, m, _ = cpu_rate(oracle, q, x0, verts, idx, bnd, per_step, rng)
    times = []
    for s in range(args.warmup + args.steps):
        sample = q[rng.choice(len(q), size=m, replace=False)]
        t0 = time.perf_counter()
        oracle.full_naive(sample, x0, verts, idx, bnd, threads=threads)
        if s >= args.warmup:
            times.append(time.perf_counter() - t0)
    value = m * len(times) / sum(times)
    sample_desc = (f"{m} seeded random queries of the {len(q)}-query grid per step; fractional term + "
                   f"NaiveIntersector-rule integer term (Embree is not available)")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "queries/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "queries_per_step": m, "threads": threads},
            "cpu_baseline": {"value": value, "unit": "queries/s", "cores": threads, "kind": "port",
                             "sample": sample_desc},
            "e2e": {"value": value, "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ---- GPU side -------------------------------------------------------------------------------------------------
def read_traffic(name="frac_mixed_icosphere.md"):
    """DRAM bytes per full launch of a kernel from its committed ncu summary, if present."""
    p = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith("traffic_bytes_per_full_launch:"):
            try:
                return float(line.split(":", 1)[1].strip().split()[0])
            except ValueError:
                return None
    return None


# Algorithmic bytes of the cell-grid integer term: per query its coordinates (24 B) and count (4 B) and its cell's
# two CSR offsets (8 B); per cell-list entry the leaf index (4 B) and the leaf's float corners (48 B); per exact test
# the triangle's nine doubles (72 B).
INT_BYTES_PER_QUERY, INT_BYTES_PER_ENTRY, INT_BYTES_PER_EXACT = 36, 52, 72
HBM_FALLBACK_GBS = 6800.0


def hbm_peak():
    """(GB/s, source) from MEASURED_PEAKS.json, else the machine's fallback figure."""
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        return float(json.load(open(p))["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return HBM_FALLBACK_GBS, "fallback"


def run_ours(args):
    import torch
    import antipodal_gb300 as ag

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream(dev)

    verts, idx, bnd, q, x0 = workload(args.grid)
    Q, S, F = len(q), len(bnd), len(idx) // 3

    disp = ag.CudaDispatcher(device=local, stream=stream, precision="mixed")
    disp.set_option(ag._lib.OPT_INTEGER_CELLS, args.integer_cells)
    t0 = time.perf_counter()
    isect = ag.CudaIntersector(disp, verts, idx)
    disp.synchronize()
    bvh_ms = 1e3 * (time.perf_counter() - t0)
    info = isect.info()

    q_dev = torch.from_numpy(q).to(dev)
    b_dev = torch.from_numpy(bnd).to(dev)
    out_plain = torch.empty(Q, dtype=torch.float64, device=dev)
    out = torch.empty(Q, dtype=torch.float64, device=dev)

    def barrier():
        torch.cuda.synchronize(dev)
        if ws > 1:
            torch.distributed.barrier()

    def timed(n_steps, fn):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        barrier()
        e0.record(stream)
        for _ in range(n_steps):
            fn()
        e1.record(stream)
        barrier()
        return reduce_max(e0.elapsed_time(e1), dev)

    # plain FP64 form (reference arithmetic)
    disp.set_precision("exact")
    ag.eval_gwnr_mesh_batch(disp, isect, q_dev, out_plain, x0, b_dev)
    plain_ms = timed(args.plain_steps, lambda: ag.eval_gwnr_mesh_batch(disp, isect, q_dev, out_plain, x0, b_dev))
    plain_step = plain_ms / args.plain_steps

    # chosen form
    disp.set_precision("mixed")
    for _ in range(args.warmup):
        ag.eval_gwnr_mesh_batch(disp, isect, q_dev, out, x0, b_dev)
    disp.synchronize()
    disp.set_option(ag._lib.OPT_TIMING, 1)
    disp.stats(reset=True)
    clocks = Clocks(local)
    clocks.start()
    ms = timed(args.steps, lambda: ag.eval_gwnr_mesh_batch(disp, isect, q_dev, out, x0, b_dev))
    clk = clocks.stop()
    st = disp.stats(reset=True)
    disp.set_option(ag._lib.OPT_TIMING, 0)
    disp.synchronize()
    step_ms = ms / args.steps
    value = ws * Q / (step_ms * 1e-3)
    launches = int(sum(st["launches"].values()))
    # The steps above run the two kernels in chunks on two streams, overlapped.  For the rooflines each kernel is
    # timed alone over the whole query set (one launch per call, CUDA events around each launch on its stream).
    out_alone = torch.empty(Q, dtype=torch.float64, device=dev)
    cnt_alone = torch.empty(Q, dtype=torch.int32, device=dev)
    disp.set_option(ag._lib.OPT_TIMING, 1)
    disp.stats(reset=True)
    for _ in range(args.steps):
        ag.eval_gwnr_mesh_batch_fractional(disp, q_dev, out_alone, x0, b_dev)
    for _ in range(args.steps):
        ag.eval_gwnr_mesh_batch_integer(disp, isect, q_dev, cnt_alone, x0)
    sk = disp.stats(reset=True)
    disp.set_option(ag._lib.OPT_TIMING, 0)
    disp.synchronize()
    del out_alone, cnt_alone
    frac_ms = sk["kernel_ms"]["fractional"] / max(1, sk["launches"]["fractional"])
    n_int = max(1, sk["launches"]["integer"])
    int_ms = sk["kernel_ms"]["integer"] / n_int
    ic = sk["integer"]
    int_bytes = (ic["queries"] * INT_BYTES_PER_QUERY + ic["cell_entries"] * INT_BYTES_PER_ENTRY +
                 ic["exact_tests"] * INT_BYTES_PER_EXACT) / n_int
    hbm, hbm_src = hbm_peak()
    int_gbs = int_bytes / (int_ms * 1e-3) / 1e9

    # the integer term of every query against the every-triangle scan, which also reports ties (hits exactly on an
    # edge or vertex, where NaiveIntersector counts a crossing once per triangle); untimed
    full_check = None
    if args.full_integer_check:
        cnt_cells = torch.empty(Q, dtype=torch.int32, device=dev)
        cnt_scan = torch.empty(Q, dtype=torch.int32, device=dev)
        ties = torch.empty(Q, dtype=torch.int32, device=dev)
        ag.eval_gwnr_mesh_batch_integer(disp, isect, q_dev, cnt_cells, x0)
        v_dev, i_dev = torch.from_numpy(verts).to(dev), torch.from_numpy(idx).to(dev)
        t0 = time.perf_counter()
        ag.eval_gwnr_mesh_batch_integer_bruteforce(disp, v_dev, i_dev, q_dev, cnt_scan, x0, out_ties=ties)
        disp.synchronize()
        full_check = {"integer_mismatches_full": int((cnt_cells != cnt_scan).sum().item()),
                      "queries_checked": Q, "ties_counted": int((ties > 0).sum().item()),
                      "tie_hits": int(ties.sum().item()), "scan_seconds": time.perf_counter() - t0}
        del cnt_cells, cnt_scan, ties

    # accuracy: chosen vs plain over every query
    diff = (out - out_plain).abs()
    max_err = float(diff.max().item())
    p99_err = p99(diff)
    n_over = int((diff > 1e-7).sum().item())

    # end to end from pinned host buffers (H2D of the queries and D2H of the result inside every step)
    q_pin = torch.from_numpy(q).pin_memory()
    o_pin = torch.empty(Q, dtype=torch.float64).pin_memory()
    qn, on = q_pin.numpy(), o_pin.numpy()
    for _ in range(max(1, args.warmup)):
        ag.eval_gwnr_mesh_batch(disp, isect, qn, on, x0, bnd)
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ag.eval_gwnr_mesh_batch(disp, isect, qn, on, x0, bnd)
    barrier()
    e2e_s = reduce_max(time.perf_counter() - t0, dev)
    e2e_value = ws * Q * args.steps / e2e_s
    e2e_match = bool(np.array_equal(on, out.cpu().numpy()))

    # roofline of the fractional kernel against the measured FP32 FMA rate
    peak = disp.probe_fp32_peak()
    achieved = Q * S * FLOPS_PER_PAIR / (frac_ms * 1e-3) / 1e12
    traffic = read_traffic()

    line = None
    if rank == 0:
        # seeded sample against the CPU oracle: plain and chosen, integer counts
        from oracle.oracle import Oracle, LIB, build
        if not os.path.exists(LIB):
            build()
        oracle = Oracle()
        rng = np.random.default_rng(7)
        pick = rng.choice(Q, size=3000, replace=False)
        ref = oracle.full_naive(q[pick], x0, verts, idx, bnd)
        plain_s = out_plain.cpu().numpy()[pick]
        chosen_s = out.cpu().numpy()[pick]
        counts = np.empty(len(pick), np.int32)
        ag.eval_gwnr_mesh_batch_integer(disp, isect, q[pick], counts, x0)
        ref_counts = oracle.int_naive(q[pick], x0, verts, idx)
        accuracy = {
            "max_abs_err_chosen_vs_plain_fp64": max_err, "p99_abs_err_chosen_vs_plain_fp64": p99_err,
            "queries_over_1e-7": n_over,
            "sample_max_abs_err_plain_vs_cpu_oracle": float(np.max(np.abs(plain_s - ref))),
            "sample_max_abs_err_chosen_vs_cpu_oracle": float(np.max(np.abs(chosen_s - ref))),
            "sample_integer_mismatches_vs_cpu_oracle": int(np.sum(counts != ref_counts)),
            "sample_size": len(pick),
            "fp64_pair_fraction": st["fp64_pairs"] / max(1, st["pairs"]),
        }
        if full_check is not None:
            accuracy.update(full_check)
        cpu = None
        if ws == 1 and not args.no_cpu:
            rate, m, threads = cpu_rate(oracle, q, x0, verts, idx, bnd, args.cpu_seconds, np.random.default_rng(3))
            cpu = {"value": rate, "unit": "queries/s", "cores": threads, "kind": "port",
                   "sample": f"{m} seeded random queries of the grid, full GWN (fractional + naive integer term)"}
        line = {
            "metric": METRIC, "value": value, "unit": "queries/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "queries": Q, "triangles": F, "segments": S,
                       "bvh_depth": info["depth"], "bvh_build_ms": bvh_ms,
                       "l2": "inputs larger than L2 (403 MB of queries per step)",
                       "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU"},
            "plain": {"value": ws * Q / (plain_step * 1e-3), "unit": "queries/s", "ms_per_step": plain_step,
                      "form": "exact FP64, reference arithmetic"},
            "chosen_over_plain": plain_step / step_ms,
            "accuracy": accuracy,
            "kernels_ms_alone": {"fractional": frac_ms, "integer": int_ms,
                                 "note": "each kernel timed alone over all queries; the timed steps run both in 4 "
                                         "chunks on two streams, overlapped"},
            "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "note": f"fractional mixed kernel, {FLOPS_PER_PAIR} algorithmic flop per (query, segment) "
                                 "pair; peak = FP32 FMA rate measured on this GPU in this run",
                         "integer": {"bound": "hbm", "achieved": int_gbs, "peak": hbm, "unit": "GB/s",
                                     "frac": int_gbs / hbm, "traffic": read_traffic("cells_icosphere.md"),
                                     "bytes_per_launch": int_bytes, "ms_per_launch": int_ms,
                                     "per_query": {"cell_entries": ic["cell_entries"] / max(1, ic["queries"]),
                                                   "leaves": ic["leaves"] / max(1, ic["queries"]),
                                                   "exact_tests": ic["exact_tests"] / max(1, ic["queries"])},
                                     "note": f"cell-grid integer kernel; algorithmic bytes = {INT_BYTES_PER_QUERY} B "
                                             f"per query + {INT_BYTES_PER_ENTRY} B per cell-list entry + "
                                             f"{INT_BYTES_PER_EXACT} B per exact test, from the kernel's own counters; "
                                             f"peak = HBM copy bandwidth ({hbm_src})"}},
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": "queries/s", "h2d_bytes_per_step": int(q.nbytes),
                    "d2h_bytes_per_step": int(Q * 8), "matches_device_result": e2e_match},
            "gpu_launches": launches,
            "clocks": clk,
        }
        print(json.dumps(line), flush=True)
    isect.close()
    disp.close()
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


# ---- secondary workloads ----------------------------------------------------------------------------------------
# Each prints one JSON line: the same metric (queries/s) on another configuration, the chosen form against the
# plain one where the configuration has both, accuracy against the CPU oracle on a seeded sample, and the CPU
# oracle's rate on a bounded sample.  Run with --config {cube, batch, robust, param}; single GPU only.

def _timer(stream):
    import torch

    def timed(n, fn):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(n):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / n
    return timed


def _oracle():
    from oracle.oracle import Oracle, LIB, build
    if not os.path.exists(LIB):
        build()
    return Oracle()


def _cpu_sample_rate(fn, n_total, seconds, unit_per_item=1.0):
    """Times fn(m) (m items, all host threads inside fn) on a sample sized to about ``seconds``."""
    m = 16
    t0 = time.perf_counter()
    fn(m)
    dt = max(time.perf_counter() - t0, 1e-6)
    m = int(min(n_total, max(m, m * seconds / dt)))
    t0 = time.perf_counter()
    fn(m)
    dt = time.perf_counter() - t0
    return m * unit_per_item / dt, m


def run_cube(args, ag, torch, stream, disp, timed):
    """Rotated open unit cube (10 triangles, 4 boundary segments), 1e5 float64 queries; full GWN."""
    from antipodal_gb300 import synth
    verts, idx, bnd, q, x0 = synth.rotated_open_cube(seed=0, n_queries=int(100_000 * args.scale))
    Q = len(q)
    isect = ag.CudaIntersector(disp, verts, idx)
    qd, bd = torch.from_numpy(q).cuda(), torch.from_numpy(bnd).cuda()
    plain, out = torch.empty(Q, dtype=torch.float64, device="cuda"), torch.empty(Q, dtype=torch.float64, device="cuda")
    disp.set_precision("exact")
    for _ in range(args.warmup):
        ag.eval_gwnr_mesh_batch(disp, isect, qd, plain, x0, bd)
    ms_plain = timed(args.steps, lambda: ag.eval_gwnr_mesh_batch(disp, isect, qd, plain, x0, bd))
    disp.set_precision("mixed")
    for _ in range(args.warmup):
        ag.eval_gwnr_mesh_batch(disp, isect, qd, out, x0, bd)
    ms = timed(args.steps, lambda: ag.eval_gwnr_mesh_batch(disp, isect, qd, out, x0, bd))
    o = _oracle()
    ref = o.full_naive(q, x0, verts, idx, bnd)
    rate, m = _cpu_sample_rate(lambda m: o.full_naive(q[:m], x0, verts, idx, bnd), Q, args.cpu_seconds)
    isect.close()
    return {"metric": METRIC, "value": Q / (ms * 1e-3), "unit": "queries/s", "ms_per_step": ms,
            "config": {"workload": "rotated open unit cube, 10 triangles, 4 boundary segments, "
                                   f"{Q} uniform float64 queries in [-1.5,1.5]^3, full GWN", "queries": Q},
            "plain": {"value": Q / (ms_plain * 1e-3), "ms_per_step": ms_plain},
            "chosen_over_plain": ms_plain / ms,
            "accuracy": {"max_abs_err_plain_vs_cpu_oracle": float(np.abs(plain.cpu().numpy() - ref).max()),
                         "p99_abs_err_plain_vs_cpu_oracle": p99(np.abs(plain.cpu().numpy() - ref)),
                         "max_abs_err_chosen_vs_cpu_oracle": float(np.abs(out.cpu().numpy() - ref).max()),
                         "p99_abs_err_chosen_vs_cpu_oracle": p99(np.abs(out.cpu().numpy() - ref)),
                         "queries_over_1e-7": int(np.sum(np.abs(out.cpu().numpy() - ref) > 1e-7)),
                         "queries": Q},
            "cpu_baseline": {"value": rate, "unit": "queries/s", "cores": os.cpu_count(), "kind": "port",
                             "sample": f"first {m} queries, full GWN"}}


def batch_workload(scale, seed=2024, n_meshes=64):
    """64 noisy icospheres / tori (1e3..2e5 triangles, log-uniform; 1..20 holes), one float32 grid each with side
    log-uniform in [64, 192] (times ``scale``)."""
    import math
    from antipodal_gb300 import synth
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n_meshes):
        ntri = int(math.exp(rng.uniform(math.log(1e3), math.log(2e5))))
        kind = "icosphere" if rng.random() < 0.5 else "torus"
        v, i = synth.noisy_mesh(kind, ntri, int(rng.integers(1, 21)), rng)
        b = synth.boundary_segments(v, i)
        side = max(4, int(round(math.exp(rng.uniform(math.log(64), math.log(192))) * scale)))
        q = synth.grid_queries(v.min(0), v.max(0), side).astype(np.float32)
        out.append((v.astype(np.float32), i, b.astype(np.float32), q))
    return out


def run_batch(args, ag, torch, stream, disp, timed):
    """64 uneven robust meshes (int64_grid, float32), one persistent launch replayed from a CUDA graph.
    Chosen: the batch with FP32 pairs under the error bound; plain: one exact (FP64) evaluation call per mesh."""
    wl = batch_workload(args.scale)
    meshes = [ag.CudaRobustMeshGwn(disp, v, i, b, precision="int64_grid") for v, i, b, _ in wl]
    pos = [torch.from_numpy(q).cuda() for *_, q in wl]
    outs = [torch.empty(len(q), dtype=torch.float32, device="cuda") for *_, q in wl]
    ref_outs = [torch.empty_like(o) for o in outs]
    batch = ag.CudaRobustBatch(disp, meshes, pos, outs)
    disp.set_robust_precision("mixed")
    t0 = time.perf_counter()
    if args.batch_config:
        batch.set_config(*[int(x) for x in args.batch_config.split(",")])
        tuned = batch.info()
    else:
        tuned = batch.tune(repeats=2)
    tune_s = time.perf_counter() - t0
    Q = tuned["queries"]
    for _ in range(args.warmup):
        batch.run(graph=True)
    ms = timed(args.steps, lambda: batch.run(graph=True))

    # plain: the reference's FP64 fractional term, one call per mesh; and the same FP64 form batched
    disp.set_robust_precision("exact")

    def per_mesh():
        for r, p, o in zip(meshes, pos, ref_outs):
            r.evaluate(p, o)
    per_mesh()
    ms_loop = timed(max(1, args.plain_steps), per_mesh)
    batch.run(graph=True)
    ms_exact_batch = timed(max(1, args.plain_steps), lambda: batch.run(graph=True))
    exact_batch_same = all(torch.equal(a, b) for a, b in zip(outs, ref_outs))
    disp.set_robust_precision("mixed")
    disp.set_option(ag._lib.OPT_TIMING, 1)
    disp.stats(reset=True)
    batch.run(graph=True)
    st = disp.stats(reset=True)
    disp.set_option(ag._lib.OPT_TIMING, 0)
    torch.cuda.synchronize()
    fp64_frac = st["fp64_pairs"] / max(1, st["pairs"])
    diff = torch.cat([(a.double() - b.double()).abs() for a, b in zip(outs, ref_outs)])
    max_diff = float(diff.max().item())
    n_same = int((diff == 0).sum().item())
    # the fractional term in double precision (RobustMeshGwn<double, int64_grid>) on the first meshes: mixed vs FP64
    frac_err, frac_diffs = 0.0, []
    for v, i, b, q in wl[:6]:
        r64 = ag.CudaRobustMeshGwn(disp, v.astype(np.float64), i, b.astype(np.float64), precision="int64_grid")
        q64 = q.astype(np.float64)
        fr = {}
        for mode in ("exact", "mixed"):
            disp.set_robust_precision(mode)
            o_, c_, f_ = np.empty(len(q64)), np.empty(len(q64), np.int32), np.empty(len(q64))
            r64.evaluate(q64, o_, c_, f_)
            fr[mode] = f_
        frac_err = max(frac_err, float(np.abs(fr["exact"] - fr["mixed"]).max()))
        frac_diffs.append(np.abs(fr["exact"] - fr["mixed"]))
        r64.close()
    disp.set_robust_precision("exact")
    # the CPU oracle (the reference's RobustMeshGwn rule) on a few queries of the first meshes, against plain
    o = _oracle()
    worst, n_diff = 0.0, 0
    for (v, i, b, q), out in zip(wl[:8], ref_outs[:8]):
        pick = np.random.default_rng(5).choice(len(q), size=min(len(q), 200), replace=False)
        gw, _, _ = o.robust_eval("int64_grid", v, i, b, q[pick])
        got = out.cpu().numpy()[pick]
        worst = max(worst, float(np.abs(got.astype(np.float64) - gw.astype(np.float64)).max()))
        n_diff += int(np.sum(got != gw))
    v0, i0, b0, q0 = wl[0]
    rate, m = _cpu_sample_rate(lambda m: o.robust_eval("int64_grid", v0, i0, b0, q0[:m]), len(q0), args.cpu_seconds)
    for x in meshes:
        x.close()
    batch.close()
    return {"metric": METRIC, "value": Q / (ms * 1e-3), "unit": "queries/s", "ms_per_step": ms,
            "config": {"workload": "64 noisy icospheres/tori (1e3..2e5 triangles, 1..20 holes), one float32 grid "
                                   f"each (side log-uniform 64..192 x {args.scale}), RobustMeshGwn<float, "
                                   "int64_grid>, one persistent launch, CUDA graph", "queries": Q,
                       "pair_units": tuned["pairs"], "items": tuned["items"], "tuned": tuned["config"],
                       "tune_seconds": tune_s},
            "plain": {"value": Q / (ms_loop * 1e-3), "ms_per_step": ms_loop,
                      "form": "exact FP64 fractional term, one agwn_robust_eval call per mesh"},
            "exact_batched": {"value": Q / (ms_exact_batch * 1e-3), "ms_per_step": ms_exact_batch,
                              "bit_identical_to_per_mesh": bool(exact_batch_same)},
            "chosen_over_plain": ms_loop / ms,
            "fp64_pair_fraction": fp64_frac,
            "accuracy": {"max_abs_diff_chosen_vs_plain": max_diff, "p99_abs_diff_chosen_vs_plain": p99(diff),
                         "values_over_1e-7": int((diff > 1e-7).sum().item()),
                         "max_abs_err_fractional_term_f64_first6_meshes": frac_err,
                         "p99_abs_err_fractional_term_f64_first6_meshes": p99(np.concatenate(frac_diffs)),
                         "fractional_terms_over_1e-7_first6_meshes": int(sum((d > 1e-7).sum() for d in frac_diffs)),
                         "identical_values": n_same, "values": int(diff.numel()),
                         "sample_plain_max_abs_err_vs_cpu_oracle": worst, "sample_plain_values_not_identical": n_diff,
                         "sample_size": 8 * 200},
            "cpu_baseline": {"value": rate, "unit": "queries/s", "cores": os.cpu_count(), "kind": "port",
                             "sample": f"first {m} queries of mesh 0 ({len(b0)} segments), RobustMeshGwn rule"}}


def run_robust(args, ag, torch, stream, disp, timed):
    """Two interpenetrating perturbed tori (1M triangles, 20 holes), 1e7 float64 queries, half within
    1e-9..1e-3 of the surface; RobustMeshGwn<double, int128_grid> and <double, exact_float> in FP64, and the chosen
    form: exact_float with the fractional term in mixed precision (counts exact; FP32 pairs with a first-order bound,
    the others through the evaluator's own FP64 rule)."""
    from antipodal_gb300 import synth
    v, i, b, q = synth.two_tori(seed=0, n_queries=int(10_000_000 * args.scale))
    Q = len(q)
    qd = torch.from_numpy(q).cuda()
    res = {}
    o = _oracle()
    pick = np.random.default_rng(9).choice(Q, size=400, replace=False)
    exact = {}
    for pol in ("int128_grid", "exact_float"):
        t0 = time.perf_counter()
        r = ag.CudaRobustMeshGwn(disp, v, i, b, precision=pol)
        disp.synchronize()
        build_ms = 1e3 * (time.perf_counter() - t0)
        out = torch.empty(Q, dtype=torch.float64, device="cuda")
        cnt = torch.empty(Q, dtype=torch.int32, device="cuda")
        r.evaluate(qd, out, cnt)
        ms = timed(args.steps, lambda: r.evaluate(qd, out, cnt))
        gw, rc, _ = o.robust_eval(pol, v, i, b, q[pick])
        res[pol] = {"value": Q / (ms * 1e-3), "ms_per_step": ms, "build_ms": build_ms,
                    "sample_count_mismatches_vs_cpu_oracle": int(np.sum(cnt.cpu().numpy()[pick] != rc)),
                    "sample_max_abs_err_vs_cpu_oracle": float(np.abs(out.cpu().numpy()[pick] - gw).max())}
        if pol == "exact_float":
            exact = {"out": out, "cnt": cnt, "r": r, "gw": gw, "rc": rc}
        else:
            r.close()
    # chosen: exact_float, fractional term in mixed precision
    r = exact["r"]
    out = torch.empty(Q, dtype=torch.float64, device="cuda")
    cnt = torch.empty(Q, dtype=torch.int32, device="cuda")
    disp.set_robust_precision("mixed")
    try:
        r.evaluate(qd, out, cnt)
        ms = timed(args.steps, lambda: r.evaluate(qd, out, cnt))
        # the timed calls run counts and fractional term in chunks on two streams, overlapped; with the fractional
        # term as an output of its own the call runs each kernel once over all queries: their times alone
        fr_alone = torch.empty(Q, dtype=torch.float64, device="cuda")
        out_alone = torch.empty(Q, dtype=torch.float64, device="cuda")
        cnt_alone = torch.empty(Q, dtype=torch.int32, device="cuda")
        disp.set_option(ag._lib.OPT_TIMING, 1)
        disp.stats(reset=True)
        r.evaluate(qd, out_alone, cnt_alone, fr_alone)
        st = disp.stats(reset=True)
        disp.set_option(ag._lib.OPT_TIMING, 0)
        same_as_alone = bool(torch.equal(out_alone, out))
        del fr_alone, out_alone, cnt_alone
    finally:
        disp.set_robust_precision("exact")
    d = (out - exact["out"]).abs()
    chosen = {"value": Q / (ms * 1e-3), "ms_per_step": ms,
              "form": "exact_float counts + mixed fractional term (FP32 pairs, FP64 by the evaluator's rule)",
              "max_abs_err_vs_exact_float_fp64": float(d.max().item()),
              "p99_abs_err_vs_exact_float_fp64": p99(d),
              "queries_over_1e-7": int((d > 1e-7).sum().item()),
              "counts_identical_to_exact": bool(torch.equal(cnt, exact["cnt"])),
              "sample_max_abs_err_vs_cpu_oracle": float(np.abs(out.cpu().numpy()[pick] - exact["gw"]).max()),
              "fp64_pair_fraction": st["fp64_pairs"] / max(1, st["pairs"]),
              "kernels_ms_alone": {"counts (robust predicates)": st["kernel_ms"]["robust"],
                                   "fractional (mixed)": st["kernel_ms"]["fractional"],
                                   "other": st["kernel_ms"]["other"],
                                   "note": "each kernel once over all queries; the timed steps run both in 8 chunks "
                                           "on two streams, overlapped"},
              "chunked_equals_alone": same_as_alone}
    r.close()
    rate, m = _cpu_sample_rate(lambda m: o.robust_eval("exact_float", v, i, b, q[:m]), Q, args.cpu_seconds)
    return {"metric": METRIC, "value": chosen["value"], "unit": "queries/s", "ms_per_step": ms,
            "config": {"workload": f"two perturbed tori, {len(i) // 3} triangles, {len(b)} boundary segments, "
                                   f"{Q} float64 queries (half uniform, half 1e-9..1e-3 off the surface)",
                       "queries": Q},
            "chosen": chosen, "plain": {"form": "exact_float, FP64 fractional term", **res["exact_float"]},
            "chosen_over_plain": chosen["value"] / res["exact_float"]["value"],
            "policies": res,
            "cpu_baseline": {"value": rate, "unit": "queries/s", "cores": os.cpu_count(), "kind": "port",
                             "sample": f"first {m} queries, exact_float"}}


def run_param(args, ag, torch, stream, disp, timed):
    """256 bicubic patches (1,024 boundary cubics), 1e6 float64 queries (30% within 1e-3 of a curve), GK15 at
    tol 1e-10: the chosen form (learned start depths from a network trained here on 1e7 labels of the plain
    integrator, double-float panels) on every query, against the plain adaptive FP64 integrator timed on a seeded
    sample of the same queries (``--plain-scale``; the full plain form takes about 100 s per step) and reported both
    as measured and extrapolated per query."""
    from antipodal_gb300 import synth
    n_q = max(64, int(1_000_000 * args.scale))
    curves, q, x0, patches = synth.bezier_patches(seed=0, n_patches=args.patches, n_queries=n_q, return_patches=True)
    cfg = ag.IntegrateConfig(0, 10, 1e-10)
    Q, Cn = len(q), len(curves)
    # the network: trained on labels of the plain integrator (the shallowest accepted depth per pair) on other
    # seeded queries and patches, args.labels of them
    # alpha 0.9: the labels are each pair's shallowest accepted depth, a lower bound on the cheapest start depth (most
    # of a pair's tree lies deeper), so starting near the upper end of the predicted distribution evaluates the fewest
    # panels; every evaluated panel is still verified by the plain test
    net = ag.LearnedGK15Proposal(disp, seed=3, n_classes=11, alpha=0.9)
    n_train_q = max(16, int(round(args.labels / (256 * 4))))
    tc, tq, tx = synth.bezier_patches(seed=101, n_patches=256, n_queries=n_train_q)
    t0 = time.perf_counter()
    tqd, tcd = torch.from_numpy(tq).cuda(), torch.from_numpy(tc).cuda()
    lab = net.labels(tqd, tx, tcd, cfg)
    feat = net.features(tqd, tx, tcd, cfg.tol)
    hist = net.train(feat, lab, steps=args.train_steps, batch=8192, lr=2e-3, seed=1)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    n_labels = int(lab.numel())
    del tqd, tcd, lab, feat
    qd, cd = torch.from_numpy(q).cuda(), torch.from_numpy(curves).cuda()
    # chosen: learned start depths + double-float panels, every query
    disp.set_param_precision("mixed")
    out = torch.empty(Q, dtype=torch.float64, device="cuda")
    nodes_c = torch.empty(Q, dtype=torch.int32, device="cuda")
    ag.eval_gwnr_parametric_batch_fractional(disp, qd, out, x0, cd, cfg, integrator=net, nodes_per_query=nodes_c)
    ms = timed(args.steps, lambda: ag.eval_gwnr_parametric_batch_fractional(disp, qd, out, x0, cd, cfg,
                                                                            integrator=net))
    # the integer term over the patches themselves (the Bezier-patch intersector): the full parametric GWN is the
    # chosen fractional term plus these counts
    isect = ag.CudaBezierPatchIntersector(disp, patches)
    cnt = torch.empty(Q, dtype=torch.int32, device="cuda")
    ag.eval_gwnr_parametric_batch_integer(disp, isect, qd, cnt, x0)
    ms_int = timed(args.steps, lambda: ag.eval_gwnr_parametric_batch_integer(disp, isect, qd, cnt, x0))
    n_cross = int(cnt.abs().sum().item())
    # its work counters (one more, untimed launch) and its FP32 rate: 864 flop per cell blossomed (3 coordinates x
    # 8 restricted cubics x 12 lerps of 3 flop) and 72 per boundary-cubic piece (2 x 12 lerps)
    disp.set_option(ag._lib.OPT_TIMING, 1)
    disp.stats(reset=True)
    deg = torch.empty(Q, dtype=torch.int32, device="cuda")
    ag.eval_gwnr_parametric_batch_integer(disp, isect, qd, cnt, x0, out_degenerate=deg)
    pst = disp.stats(reset=True)["patches"]
    disp.set_option(ag._lib.OPT_TIMING, 0)
    n_degenerate = int((deg > 0).sum().item())
    int_flop = 864.0 * pst["cells"] + 72.0 * pst["pieces"]
    fp32_peak = disp.probe_fp32_peak()
    isect.close()
    # the sample: the first Qs queries (the generator shuffles them, so they are a seeded random sample)
    Qs = max(32, min(Q, int(round(args.plain_scale * Q))))
    qs = qd[:Qs].contiguous()
    out_df = torch.empty(Qs, dtype=torch.float64, device="cuda")
    ag.eval_gwnr_parametric_batch_fractional(disp, qs, out_df, x0, cd, cfg)
    ms_df = timed(args.steps, lambda: ag.eval_gwnr_parametric_batch_fractional(disp, qs, out_df, x0, cd, cfg))
    disp.set_param_precision("exact")
    plain = torch.empty(Qs, dtype=torch.float64, device="cuda")
    nodes_p = torch.empty(Qs, dtype=torch.int32, device="cuda")
    ag.eval_gwnr_parametric_batch_fractional(disp, qs, plain, x0, cd, cfg, nodes_per_query=nodes_p)
    ms_plain = timed(args.steps, lambda: ag.eval_gwnr_parametric_batch_fractional(disp, qs, plain, x0, cd, cfg))
    # learned start depths with the plain FP64 arithmetic (the ablation of the network alone)
    out_l = torch.empty(Qs, dtype=torch.float64, device="cuda")
    nodes_l = torch.empty_like(nodes_p)
    ag.eval_gwnr_parametric_batch_fractional(disp, qs, out_l, x0, cd, cfg, integrator=net, nodes_per_query=nodes_l)
    ms_learned = timed(args.steps, lambda: ag.eval_gwnr_parametric_batch_fractional(disp, qs, out_l, x0, cd, cfg,
                                                                                    integrator=net))
    d = (out[:Qs] - plain).abs()
    err, err_p99, n_over = float(d.max().item()), p99(d), int((d > 1e-7).sum().item())
    err_learned = float((out_l - plain).abs().max().item())
    err_df = float((out_df - plain).abs().max().item())
    panels_p, panels_l = int(nodes_p.sum().item()), int(nodes_l.sum().item())
    fp64 = disp.probe_fp64_peak()
    achieved = panels_p * 15 * 150 / (ms_plain * 1e-3) / 1e12
    o = _oracle()
    pick = np.random.default_rng(4).choice(Qs, size=32, replace=False)
    ref = o.param_frac_bezier3(q[pick], x0, curves, 0, 10, 1e-10)
    rate, m = _cpu_sample_rate(lambda m: o.param_frac_bezier3(q[:m], x0, curves, 0, 10, 1e-10), Q, args.cpu_seconds)
    net.close()
    plain_rate = Qs / (ms_plain * 1e-3)
    return {"metric": METRIC, "value": Q / (ms * 1e-3), "unit": "queries/s", "ms_per_step": ms,
            "config": {"workload": f"{args.patches} bicubic Bezier patches ({Cn} boundary cubics), {Q} float64 queries "
                                   "(30% within 1e-3 of a curve), adaptive GK15 tol 1e-10, max depth 10",
                       "queries": Q, "pairs": Q * Cn, "sample_queries": Qs},
            "chosen": {"form": "learned start depths + double-float panels", "queries": Q,
                       "panels_per_pair": int(nodes_c.sum().item()) / (Q * Cn)},
            "integer_term": {"form": "Bezier-patch intersector (winding numbers of cell boundaries), 256 patches",
                             "ms_per_step": ms_int, "value": Q / (ms_int * 1e-3), "unit": "queries/s",
                             "abs_counts_per_query": n_cross / Q,
                             "full_gwn_ms_per_step": ms + ms_int,
                             "per_query": {"pairs_past_box": pst["pairs"] / Q, "cells": pst["cells"] / Q,
                                           "pieces": pst["pieces"] / Q},
                             "fp64_jobs_per_pair": pst["fp64_pairs"] / max(1, pst["pairs"]),
                             "degenerate_queries": n_degenerate,
                             "roofline": {"bound": "fp32", "achieved": int_flop / (ms_int * 1e-3) / 1e12,
                                          "peak": fp32_peak, "unit": "TFLOP/s",
                                          "frac": int_flop / (ms_int * 1e-3) / 1e12 / fp32_peak,
                                          "note": "algorithmic flop of the blossoms from the kernel's own counters; "
                                                  "peak = FP32 FMA rate measured on this GPU in this run"}},
            "plain": {"value": plain_rate, "ms_per_step_sample": ms_plain,
                      "ms_per_step_extrapolated_full": ms_plain * Q / Qs,
                      "panels_per_pair": panels_p / (Qs * Cn),
                      "note": f"timed on the seeded {Qs}-query sample; queries/s is per query, so it extrapolates "
                              "linearly to the full set"},
            "learned_fp64": {"value": Qs / (ms_learned * 1e-3), "ms_per_step_sample": ms_learned,
                             "panels_per_pair": panels_l / (Qs * Cn), "train_seconds": train_s,
                             "train_steps": args.train_steps,
                             "train_loss_first_last": [float(hist[:20].mean()), float(hist[-100:].mean())],
                             "labels": n_labels, "max_abs_err_vs_plain": err_learned},
            "double_float_only": {"value": Qs / (ms_df * 1e-3), "ms_per_step_sample": ms_df,
                                  "max_abs_err_vs_plain": err_df},
            "chosen_over_plain": (Q / (ms * 1e-3)) / plain_rate,
            "accuracy": {"max_abs_err_chosen_vs_plain": err, "p99_abs_err_chosen_vs_plain": err_p99,
                         "queries_over_1e-7": n_over, "queries_compared": Qs,
                         "sample_plain_bit_identical_to_cpu_oracle": bool(np.array_equal(plain.cpu().numpy()[pick], ref))},
            "roofline": {"bound": "fp64", "achieved": achieved, "peak": fp64, "unit": "TFLOP/s",
                         "frac": achieved / fp64,
                         "note": "plain integrator, 15 integrand evaluations x 150 algorithmic FP64 flop per panel; "
                                 "peak = FP64 FMA rate measured on this GPU in this run"},
            "cpu_baseline": {"value": rate, "unit": "queries/s", "cores": os.cpu_count(), "kind": "port",
                             "sample": f"first {m} queries x {Cn} curves"}}


def run_secondary(args):
    import torch
    import antipodal_gb300 as ag
    torch.cuda.set_device(0)
    stream = torch.cuda.current_stream()
    disp = ag.CudaDispatcher(device=0, stream=stream)
    timed = _timer(stream)
    fn = {"cube": run_cube, "batch": run_batch, "robust": run_robust, "param": run_param}[args.config]
    clocks = Clocks(0)
    clocks.start()
    line = fn(args, ag, torch, stream, disp, timed)
    line["clocks"] = clocks.stop()
    line.update({"n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
                 "scaling": "weak", "vs_baseline": None, "data": "synthetic", "config_name": args.config})
    print(json.dumps(line), flush=True)
    disp.close()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.config != "mesh":
        return run_secondary(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
