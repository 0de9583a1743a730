"""IVF-PQ query throughput on one GB300 (and N replicas under torchrun).

Workload: 1,000,000 x 128 SIFT-like float32 rows (integer-valued, 1,024-
centre Gaussian mixture, std 20, clipped to [0, 255]), IVF nlist 4096, PQ
M = 16 x 8 bit, 10,000 queries, k = 10. Index trained on the GPU (plain exact
k-means) from a 131,072-row sample, 10 iterations each for the coarse and
the PQ codebooks, then all rows added. A step is one search of the whole
10,000-query batch.

`value` times steps with the queries and results resident in HBM (CUDA
events on the launching stream, L2 flushed with a 256 MiB write before each
step, outside the timed interval); `e2e` times the public host-buffer C-ABI
call (mv_ivfpq_search) including the host->device copy of the queries from
pinned memory and the device->host copy of distances and ids.

`--impl reference` times the oracle (the C++ restatement of the reference's
CPU path) on the host cores over a bounded query sample of the same
workload, with an index it builds itself on the CPU.
"""

from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NB = 1_000_000
D = 128
N_CENTERS = 1024
NQ = 10_000
NLIST = 4096
M = 16
K = 10
TRAIN_N = 131_072
NITER = 10
METRIC = "IVF-PQ QPS at recall@10>=0.95 (1Mx128), BF16+rerank vs plain FP32, same GB300"


def _env_int(name, default):
    try:
        return int(os.environ.get(name, default))
    except ValueError:
        return default


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
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
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for name, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(name)
        return {
            "sm_mhz": float(np.median(sm)) if sm else None,
            "sm_max_mhz": float(max(smax)) if smax else None,
            "reasons": sorted(reasons),
            "samples": len(sm),
        }


def build_workload():
    from mojovec_gb300 import synth

    base, queries = synth.sift_like(NB, d=D, n_centers=N_CENTERS, nq=NQ)
    return base, queries


def probed_code_bytes(index, queries, nprobe):
    """Algorithmic ADC bytes of one step: sum over queries of the code bytes
    of the probed lists (sum |L_p| * M). Probes are recomputed on the host
    from the exported centroids (FP32, same selection rule)."""
    cent, _ = index.codebooks()
    off, _, _ = index.lists()
    sizes = np.diff(off)
    total = 0
    for q0 in range(0, queries.shape[0], 2048):
        q = queries[q0:q0 + 2048]
        d2 = (q * q).sum(1, keepdims=True) - 2.0 * q @ cent.T + (cent * cent).sum(1)[None, :]
        part = np.argpartition(d2, nprobe - 1, axis=1)[:, :nprobe]
        total += int(sizes[part].sum())
    return total * M


def recall_at(gt, labels, k=10):
    hits = 0
    for g, l in zip(gt[:, :k], labels[:, :k]):
        hits += len(set(g.tolist()) & set(l.tolist()))
    return hits / (gt.shape[0] * k)


def cpu_baseline(index, queries, nprobe, threads, sample):
    """The oracle searching the same index (codebooks and lists loaded from
    the GPU index) on a bounded sample of queries."""
    from oracle import oracle as orc

    cent, pq = index.codebooks()
    off, ids, codes = index.lists()
    ref = orc.IVFPQ(D, NLIST, M)
    ref.set_codebooks(cent, pq)
    ref.set_lists(off, ids, codes)
    q = queries[:sample]
    ref.search(q[:32], K, nprobe, nthreads=threads, lut_threads=threads)  # warm
    t0 = time.perf_counter()
    _, lab = ref.search(q, K, nprobe, nthreads=threads, lut_threads=threads)
    dt = time.perf_counter() - t0
    return sample / dt, lab


def run_gpu(args, rank, world):
    import torch

    import mojovec_gb300 as mv

    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    ctx = mv.Context(dev)
    t_setup = time.perf_counter()
    base, queries = build_workload()
    index = mv.IndexIVFPQ(D, NLIST, M, mv.METRIC_L2, ctx=ctx)
    index.train(base[:TRAIN_N], niter_coarse=NITER, niter_pq=NITER)
    index.add(base)
    nprobe = args.nprobe
    index.nprobe = nprobe

    # Ground truth: exact FP32 Flat search. Every SIFT-like component is an
    # integer in [0, 255], so every FP32 product and partial sum of a squared
    # distance is an integer below 2^24 and the FP32 distances equal FP64.
    flat = mv.IndexFlat(D, mv.METRIC_L2, ctx=ctx)
    flat.add(base)
    _, gt = flat.search(queries, K)
    del flat
    setup_s = time.perf_counter() - t_setup

    form = mv.FORM_FAST if args.form == "fast" else mv.FORM_PLAIN
    sopts = dict(form=form, nprobe=nprobe, rerank=args.rerank)
    d_q = torch.from_numpy(queries).cuda()
    d_dist = torch.empty((NQ, K), dtype=torch.float32, device="cuda")
    d_lab = torch.empty((NQ, K), dtype=torch.int64, device="cuda")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()

    def step():
        index.search_device(d_q.data_ptr(), NQ, K, d_dist.data_ptr(), d_lab.data_ptr(),
                            stream=stream.cuda_stream, **sopts)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    labels = d_lab.cpu().numpy()
    rec = recall_at(gt, labels, K)

    # ---- timed region (device-resident) ----
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(dev)
    clocks.start()
    ctx.profile(True)
    launches0 = ctx.kernel_launches()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(args.steps)]
    for a, b in evs:
        flush.fill_(1.0)
        a.record(stream)
        step()
        b.record(stream)
    torch.cuda.synchronize()
    launches = ctx.kernel_launches() - launches0
    stage = ctx.stage_times()
    ctx.profile(False)
    clk = clocks.stop()
    step_ms = [a.elapsed_time(b) for a, b in evs]
    total_ms = float(sum(step_ms))
    if world > 1:
        t = torch.tensor([total_ms], dtype=torch.float64, device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    value = world * NQ * args.steps / (total_ms / 1e3)

    # ---- e2e through the host-buffer C ABI, pinned queries ----
    pinned = torch.empty((NQ, D), dtype=torch.float32).pin_memory()
    pinned.copy_(torch.from_numpy(queries))
    hq = pinned.numpy()
    index.search(hq, K, **sopts)
    if world > 1:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        _, elab = index.search(hq, K, **sopts)
    e2e_s = time.perf_counter() - t0
    if world > 1:
        t = torch.tensor([e2e_s], dtype=torch.float64, device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e_qps = world * NQ * args.steps / e2e_s
    assert np.array_equal(elab, labels), "host-buffer and device-buffer searches disagree"

    # ---- roofline of the dominant kernel ----
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    scan_ms, scan_n = stage.get("scan", (0.0, 0))
    code_bytes = probed_code_bytes(index, queries, nprobe)
    per_launch_ms = scan_ms / max(scan_n, 1)
    achieved = code_bytes / (per_launch_ms / 1e3) / 1e9 if per_launch_ms > 0 else 0.0

    out = {
        "metric": METRIC,
        "value": round(value, 1),
        "unit": "queries/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(total_ms / args.steps, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32" if form == mv.FORM_PLAIN else "bf16+f32",
        "data": "synthetic SIFT-like (seeded Gaussian mixture, integer-valued), not SIFT1M",
        "config": {
            "workload": "ivfpq_1Mx128_nlist4096_M16_nq10000_k10",
            "form": args.form,
            "nprobe": nprobe,
            "rerank": args.rerank,
            "nb": NB, "d": D, "nlist": NLIST, "M": M, "nq": NQ, "k": K,
            "train_rows": TRAIN_N, "train_niter": NITER,
            "recall_at_10": round(rec, 4),
            "l2_policy": "flush: 256 MiB device write before every timed step (outside the events)",
            "parallelism": f"replicas x{world}",
            "setup_s": round(setup_s, 1),
        },
        "e2e": {
            "value": round(e2e_qps, 1),
            "unit": "queries/s",
            "h2d_bytes_per_step": NQ * D * 4,
            "d2h_bytes_per_step": NQ * K * (4 + 8),
        },
        "gpu_launches": int(launches),
        "roofline": {
            "bound": "hbm",
            "kernel": "k_ivfpq_scan_plain" if form == mv.FORM_PLAIN else "ivfpq fast ADC scan",
            "achieved": round(achieved, 1),
            "peak": hbm_peak,
            "peak_source": peak_src,
            "unit": "GB/s",
            "frac": round(achieved / hbm_peak, 4),
            "traffic": None,
            "algorithmic_bytes_per_launch": code_bytes,
            "launch_ms": round(per_launch_ms, 4),
        },
        "stages_ms_per_step": {k: round(v[0] / args.steps, 4) for k, v in stage.items()},
        "clocks": clk,
    }
    if rank == 0 and not args.no_cpu:
        sample = args.cpu_sample
        threads = os.cpu_count() or 1
        qps, clab = cpu_baseline(index, queries, nprobe, threads, sample)
        plain_match = None
        if form == mv.FORM_PLAIN:
            plain_match = bool(np.array_equal(clab, labels[:sample]))
        out["cpu_baseline"] = {
            "value": round(qps, 1),
            "unit": "queries/s",
            "cores": threads,
            "kind": "port",
            "sample": f"{sample} of the {NQ} queries, same index (codebooks + lists loaded "
                      f"from the GPU index), nprobe {nprobe}, coarse and LUT+ADC query-parallel "
                      f"on {threads} threads",
            "ids_equal_to_gpu": plain_match,
        }
    return out


def run_reference(args):
    """The oracle (C++ restatement of the reference CPU path) builds the same
    index on the host and answers a bounded query sample."""
    from oracle import oracle as orc

    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    base, queries = build_workload()
    ref = orc.IVFPQ(D, NLIST, M)
    ref.train(base[:TRAIN_N], niter_coarse=NITER, niter_pq=NITER, nthreads=threads)
    ref.add(base, nthreads=threads)
    setup_s = time.perf_counter() - t0
    sample = args.cpu_sample
    q = queries[:sample]
    for _ in range(max(args.warmup, 0)):
        ref.search(q[:32], K, args.nprobe, nthreads=threads, lut_threads=threads)
    times = []
    for _ in range(args.steps):
        t = time.perf_counter()
        ref.search(q, K, args.nprobe, nthreads=threads, lut_threads=threads)
        times.append(time.perf_counter() - t)
    total = sum(times)
    qps = sample * args.steps / total
    return {
        "metric": METRIC,
        "impl": "reference",
        "value": round(qps, 1),
        "unit": "queries/s",
        "n_gpus": 0,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(1e3 * total / args.steps, 3),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic SIFT-like (seeded Gaussian mixture, integer-valued), not SIFT1M",
        "config": {
            "workload": "ivfpq_1Mx128_nlist4096_M16_nq10000_k10",
            "form": "reference CPU path (oracle port)",
            "nprobe": args.nprobe,
            "nb": NB, "d": D, "nlist": NLIST, "M": M, "nq": NQ, "k": K,
            "train_rows": TRAIN_N, "train_niter": NITER,
            "setup_s": round(setup_s, 1),
        },
        "cpu_baseline": {
            "value": round(qps, 1),
            "unit": "queries/s",
            "cores": threads,
            "kind": "port",
            "sample": f"{sample} queries per step of the {NQ}; index trained and filled by the "
                      f"oracle on the CPU; coarse and LUT+ADC query-parallel on {threads} threads",
        },
        "e2e": {"value": round(qps, 1), "unit": "queries/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--form", default="plain", choices=["plain", "fast"])
    ap.add_argument("--nprobe", type=int, default=64)
    ap.add_argument("--rerank", type=int, default=0)
    ap.add_argument("--cpu-sample", type=int, default=500)
    ap.add_argument("--no-cpu", action="store_true")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    world = _env_int("WORLD_SIZE", 1)
    rank = _env_int("RANK", 0)

    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(run_reference(args)), flush=True)
        return

    if world > 1:
        import torch

        torch.distributed.init_process_group("nccl")
    out = run_gpu(args, rank, world)
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        import torch

        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
