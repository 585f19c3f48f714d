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
def read_traffic():
    """DRAM bytes per launch of the mixed fractional kernel from the committed ncu summary, if present."""
    p = os.path.join(ROOT, "profiles", "frac_mixed_icosphere.md")
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith("traffic_bytes_per_full_launch:"):
            try:
                return float(line.split(":", 1)[1].strip().split()[0])
            except ValueError:
                return None
    return None


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
    frac_ms = st["kernel_ms"]["fractional"] / max(1, st["launches"]["fractional"])
    int_ms = st["kernel_ms"]["integer"] / max(1, st["launches"]["integer"])

    # accuracy: chosen vs plain over every query
    diff = (out - out_plain).abs()
    max_err = float(diff.max().item())
    p99_err = float(torch.quantile(diff[torch.randperm(Q, device=dev)[:1_000_000]].float(), 0.99).item())
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
            "kernels_ms_per_step": {"fractional": frac_ms, "integer": int_ms},
            "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "note": f"fractional mixed kernel, {FLOPS_PER_PAIR} algorithmic flop per (query, segment) "
                                 "pair; peak = FP32 FMA rate measured on this GPU in this run"},
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


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
