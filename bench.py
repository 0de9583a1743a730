"""IVF-PQ query throughput on one GB300 (and N replicas under torchrun).

Workload: 1,000,000 x 128 SIFT-like float32 rows (integer-valued, 1,024-
centre Gaussian mixture, std 20, clipped to [0, 255]), IVF nlist 4096, PQ
M = 16 x 8 bit, 10,000 queries, k = 10. Index trained on the GPU (plain exact
k-means) from a 131,072-row sample, 10 iterations each for the coarse and
the PQ codebooks, then all rows added. A step is one search of the whole
10,000-query batch.

The headline form is the fast form (BF16 tensor-core coarse GEMM with an
exact FP32 recheck, per-query LUT, exact FP32 rerank of a shortlist) at the
operating point that reaches recall@10 >= 0.95; the plain FP32 form (the
reference's own algorithm, bit-exact) is timed in the same run at the same
nprobe and reported beside it.

`value` times steps with the queries and results resident in HBM (CUDA
events on the launching stream, L2 flushed with a 256 MiB write before each
step, outside the timed interval); `e2e` times the public host-buffer C-ABI
call (mv_ivfpq_search) including the host->device copy of the queries from
pinned memory and the device->host copy of distances and ids into
caller-provided pinned result arrays.

`--impl reference` times the oracle (the C++ restatement of the reference's
CPU path) on the host cores over a bounded query sample of the same
workload, with an index it builds itself on the CPU.

`--workload flat` measures the flat scan instead (1,000,000 x 128 of the
same rows, 10,000 queries, k = 10 or 100, L2 or IP): the fast form (BF16
tcgen05 GEMM with a per-row heap epilogue, exact FP32 rerank of a k * 4
shortlist) against the plain FP32 form, with the GEMM's tensor roofline.
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

D = 128
N_CENTERS = 1024
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
    """Samples nvidia-smi clocks and throttle reasons during the timed region.

    start() returns once nvidia-smi is producing samples, so sampling is
    live when the region begins; stop() waits for one more sample, so a
    region shorter than the sampling period still has the sample taken as it
    ends. The record covers the samples from start() to that one."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    PERIOD_MS = 50

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.lines = []
        self.first = 0

    def _wait_lines(self, count, timeout_s):
        t0 = time.perf_counter()
        while len(self.lines) < count and time.perf_counter() - t0 < timeout_s:
            time.sleep(0.005)

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", str(self.PERIOD_MS)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
            self._wait_lines(1, 5.0)
            self.first = len(self.lines)  # samples from here on
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self._wait_lines(len(self.lines) + 1, 1.0)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines[self.first:]:
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


NB = 1_000_000
NQ = 10_000


def build_workload(nb=None, nq=None, d=D):
    from mojovec_gb300 import synth

    base, queries = synth.sift_like(nb or NB, d=d, n_centers=N_CENTERS, nq=nq or NQ)
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


def distance_error_vs_fp64(base, queries, dist, labels, metric="l2", sample=256):
    """Relative error of each returned distance against the FP64 distance of
    the same (query, row) pair, over the first `sample` queries (computed on
    the host, outside every timed region). metric "l2": squared L2; "ip":
    the inner product (the index returns it un-negated). Labels are row
    numbers of `base`; -1 slots are skipped. For PQ forms without a rerank
    the returned value is the ADC approximation, so its error is the
    quantization error, not arithmetic error."""
    n = min(sample, len(queries))
    lab = np.asarray(labels[:n])
    ok = lab >= 0
    if not ok.any():
        return {"max_rel": None, "mean_rel": None, "results": 0, "queries": n}
    qi = np.nonzero(ok)[0]
    rows = base[lab[ok]].astype(np.float64)
    qs = queries[:n][qi].astype(np.float64)
    if metric == "l2":
        ref = ((qs - rows) ** 2).sum(1)
    else:
        ref = (qs * rows).sum(1)
    got = np.asarray(dist[:n], np.float64)[ok]
    rel = np.abs(got - ref) / np.maximum(np.abs(ref), 1e-30)
    return {"max_rel": float(f"{rel.max():.3e}"), "mean_rel": float(f"{rel.mean():.3e}"),
            "results": int(ok.sum()), "queries": n,
            "definition": "|returned - FP64(query, returned row)| / |FP64|, per result"}


def smem_roofline(lookups, launch_ms, peaks, clk, sms=152):
    """The ADC scan's shared-memory bound: one table lookup per code byte,
    at most 32 lookups (one conflict-free wavefront) per SM per clock."""
    mhz = (clk or {}).get("sm_mhz") or peaks.get("sm_max_mhz", 2070.0)
    peak = 32.0 * sms * float(mhz) * 1e6
    achieved = lookups / (launch_ms / 1e3) if launch_ms > 0 else 0.0
    return {"achieved": round(achieved / 1e9, 1), "peak": round(peak / 1e9, 1),
            "unit": "G lookups/s", "frac": round(achieved / peak, 4),
            "peak_basis": f"32 lookups per SM per clock x {sms} SMs x {float(mhz):.0f} MHz "
                          "(median SM clock of the timed region)"}


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


def _timed_steps(torch, step, steps, stream, flush):
    """Times `steps` calls with CUDA events on the launching stream; L2 is
    flushed (256 MiB write) before each step, outside the events."""
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(steps)]
    for a, b in evs:
        flush.fill_(1.0)
        a.record(stream)
        step()
        b.record(stream)
    torch.cuda.synchronize()
    return float(sum(a.elapsed_time(b) for a, b in evs))


def _pinned_results(torch, nq, k):
    """Caller-provided result arrays in pinned host memory, allocated once
    (the search writes distances and labels into them every call, as the
    reference's search writes into the caller's spans)."""
    d = torch.empty((nq, k), dtype=torch.float32).pin_memory()
    lab = torch.empty((nq, k), dtype=torch.int64).pin_memory()
    return (d, lab), {"distances": d.numpy(), "labels": lab.numpy()}


def _max_over_ranks(torch, world, v, device="cuda"):
    """The slowest rank's time: all ranks' work counts as done only when the
    last rank finishes."""
    if world == 1:
        return v
    t = torch.tensor([v], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def aggregate_qps(world, nq, steps, max_ms):
    """Whole-job throughput: every rank answered nq queries per step."""
    return world * nq * steps / (max_ms / 1e3)


def run_gpu(args, rank, world):
    import torch

    import mojovec_gb300 as mv

    nb, nq = args.nb, args.nq
    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    ctx = mv.Context(dev)
    t_setup = time.perf_counter()
    base, queries = build_workload(nb, nq)
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

    fast = dict(form=mv.FORM_FAST, nprobe=nprobe, rerank=args.rerank, lut=args.lut)
    plain = dict(form=mv.FORM_PLAIN, nprobe=nprobe)
    batched = args.form == "batched"
    headline = plain if args.form == "plain" else fast
    plan, tuned = None, None
    if batched:
        # The batched form: one plan (device buffers, persistent scan, tuned
        # launch shapes) replayed as a CUDA graph, every query at this nprobe / k.
        plan = mv.IVFPQBatchPlan(index, nq, nprobe, K, rerank=args.rerank, lut=args.lut)
        npv = np.full(nq, nprobe, np.int32)
        kv = np.full(nq, K, np.int32)
        plan.set_queries(queries, npv, kv)
        tuned = plan.tune(nq)
    d_q = torch.from_numpy(queries).cuda()
    d_dist = torch.empty((nq, K), dtype=torch.float32, device="cuda")
    d_lab = torch.empty((nq, K), dtype=torch.int64, device="cuda")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()

    def make_step(opts, graph=True):
        if batched and opts is headline:
            def step():
                plan.run(nq, use_graph=graph, stream=stream.cuda_stream)
            return step

        def step():
            index.search_device(d_q.data_ptr(), nq, K, d_dist.data_ptr(), d_lab.data_ptr(),
                                stream=stream.cuda_stream, **opts)
        return step

    results = {}
    for name, opts in (("plain", plain), ("headline", headline)):
        step = make_step(opts)
        for _ in range(args.warmup):
            step()
        torch.cuda.synchronize()
        if batched and name == "headline":
            dists, labels = plan.results(nq)
        else:
            dists, labels = d_dist.cpu().numpy(), d_lab.cpu().numpy()
        results[name] = {"recall": recall_at(gt, labels, K), "labels": labels,
                         "derr": distance_error_vs_fp64(base, queries, dists, labels)}
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        if name == "headline":
            clocks = ClockSampler(dev)
            clocks.start()
            launches0 = ctx.kernel_launches()
        torch.cuda.nvtx.range_push(f"timed_{name}")
        ms = _timed_steps(torch, step, args.steps, stream, flush)
        torch.cuda.nvtx.range_pop()
        if name == "headline":
            launches = ctx.kernel_launches() - launches0
            clk = clocks.stop()
            # Per-stage times (CUDA events around each stage) from a separate,
            # untimed pass of the same steps: the events are not part of the job.
            # (graph replays run no host code: the batched form's stages are
            # timed on direct runs of the same plan)
            ctx.profile(True)
            _timed_steps(torch, make_step(opts, graph=False), args.steps, stream, flush)
            stage = ctx.stage_times()
            ctx.profile(False)
        results[name]["ms"] = _max_over_ranks(torch, world, ms)
    total_ms = results["headline"]["ms"]
    value = aggregate_qps(world, nq, args.steps, total_ms)
    plain_qps = aggregate_qps(world, nq, args.steps, results["plain"]["ms"])
    labels = results["headline"]["labels"]

    # ---- e2e through the host-buffer C ABI, queries in pinned memory ----
    pinned = torch.empty((nq, D), dtype=torch.float32).pin_memory()
    pinned.copy_(torch.from_numpy(queries))
    hq = pinned.numpy()
    keep, outs = _pinned_results(torch, nq, K)
    if batched:
        # the plan's public calls: host queries in, graph replay, results out
        def e2e_step():
            plan.set_queries(hq, npv, kv)
            plan.run(nq, use_graph=True)
            return plan.results(nq, **outs)
    else:
        def e2e_step():
            return index.search(hq, K, **headline, **outs)
    e2e_step()
    if world > 1:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        _, elab = e2e_step()
    e2e_s = _max_over_ranks(torch, world, time.perf_counter() - t0)
    e2e_qps = world * nq * args.steps / e2e_s
    assert np.array_equal(elab, labels), "host-buffer and device-buffer searches disagree"

    # ---- roofline of the dominant kernel (the ADC scan) ----
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    # the dominant kernel's own time: the two-kernel scan's table + ADC kernel
    # has its own stage events ("adc", inside "scan"); other scans are one kernel
    scan_ms, scan_n = stage.get("adc", stage.get("scan", (0.0, 0)))
    code_bytes = probed_code_bytes(index, queries, nprobe)
    per_launch_ms = scan_ms / max(scan_n, 1)
    achieved = code_bytes / (per_launch_ms / 1e3) / 1e9 if per_launch_ms > 0 else 0.0
    fast_form = args.form in ("fast", "batched")
    workload = f"ivfpq_{nb}x128_nlist4096_M16_nq{nq}_k10"
    # the fast scan's ADC kernel: by default (and lut 7) the two-kernel scan's
    # k_ivfpq_rows (its per-query select runs after it in the scan stage)
    scan_kernel = ({6: "k_ivfpq_scan_rt", None: "k_ivfpq_rows", 0: "k_ivfpq_rows", 7: "k_ivfpq_rows"}
                   .get(args.lut, "k_ivfpq_scan_fast")) if fast_form else "k_ivfpq_scan_plain"
    traffic = None  # DRAM bytes per launch from the committed ncu capture of this config
    try:
        t = json.load(open(os.path.join(ROOT, "profiles", "dram_traffic.json"))).get(
            scan_kernel, {})
        if fast_form and t.get("workload") == workload and t.get("nprobe") == nprobe:
            traffic = int(t["dram_bytes_per_launch"])
    except (OSError, ValueError, KeyError):
        pass

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
        "dtype": "bf16+f32" if fast_form else "f32",
        "data": "synthetic SIFT-like (seeded Gaussian mixture, integer-valued), not SIFT1M",
        "config": {
            "workload": workload,
            "form": ("fast: two-pass BF16 tcgen05 coarse GEMM + FP32 recheck, per-query table from the "
                     "FP16 codebook (codes read from L2) writing per-candidate distance rows, warp-per-query "
                     "streaming select, certified rerank from an 8-bit row copy (the full FP32 rerank's "
                     "results)"
                     + ("; batched: one plan (persistent scan, tuned launch shapes) replayed as a "
                        "CUDA graph" if batched else ""))
                    if fast_form else "plain FP32 (reference algorithm, bit-exact)",
            **({"batch_tuned": tuned} if batched else {}),
            "nprobe": nprobe,
            "rerank": args.rerank if fast_form else 0,
            "nb": nb, "d": D, "nlist": NLIST, "M": M, "nq": nq, "k": K,
            "train_rows": TRAIN_N, "train_niter": NITER,
            "recall_at_10": round(results["headline"]["recall"], 4),
            "plain_fp32_qps_same_nprobe": round(plain_qps, 1),
            "plain_fp32_recall_at_10": round(results["plain"]["recall"], 4),
            "speedup_vs_plain_fp32": round(value / plain_qps, 2),
            "l2_policy": "flush: 256 MiB device write before every timed step (outside the events)",
            "parallelism": f"replicas x{world}",
            "setup_s": round(setup_s, 1),
        },
        "e2e": {
            "value": round(e2e_qps, 1),
            "unit": "queries/s",
            "h2d_bytes_per_step": nq * D * 4 + (nq * 12 if batched else 0),  # + nprobe, k, order
            "d2h_bytes_per_step": nq * K * (4 + 8),
        },
        "gpu_launches": int(launches),
        "roofline": {
            "bound": "hbm",
            "kernel": scan_kernel,
            "achieved": round(achieved, 1),
            "peak": hbm_peak,
            "peak_source": peak_src,
            "unit": "GB/s",
            "frac": round(achieved / hbm_peak, 4),
            "traffic": traffic,
            "algorithmic_bytes_per_launch": code_bytes,
            "note": "codes (16 MB) are L2-resident at this size: DRAM traffic (codes, and the "
                    "distance rows of the two-kernel scan) is far below the algorithmic bytes; the "
                    "ADC kernel is bound by its LSU data pipe (bank-conflicted table lookups), see "
                    "smem_lookups for the shared-memory table's own bound; launch_ms is the "
                    "kernel alone (stage events around it) when the two-kernel scan runs",
            "launch_ms": round(per_launch_ms, 4),
            "smem_lookups": smem_roofline(code_bytes, per_launch_ms, peaks, clk),
        },
        "stages_ms_per_step": {k: round(v[0] / args.steps, 4) for k, v in stage.items()},
        "clocks": clk,
        "distance_error_vs_fp64": results["headline"]["derr"],
    }
    out["config"]["plain_fp32_distance_error_vs_fp64"] = results["plain"]["derr"]
    if rank == 0 and not args.no_cpu:
        sample = min(args.cpu_sample, nq)
        threads = os.cpu_count() or 1
        qps, clab = cpu_baseline(index, queries, nprobe, threads, sample)
        out["cpu_baseline"] = {
            "value": round(qps, 1),
            "unit": "queries/s",
            "cores": threads,
            "kind": "port",
            "sample": f"{sample} of the {nq} queries, same index (codebooks + lists loaded "
                      f"from the GPU index), nprobe {nprobe}, reference algorithm (plain form), "
                      f"coarse and LUT+ADC query-parallel on {threads} threads",
            "ids_equal_to_gpu_plain": bool(np.array_equal(clab, results["plain"]["labels"][:sample])),
        }
    return out


FLAT_METRIC = ("Flat QPS (1Mx128 SIFT-like, 10k queries), exact FP32 results: certified BF16 tcgen05 "
               "shortlist vs the FP32 SIMT scan")
SQ8_METRIC = ("SQ8 QPS (1Mx128 SIFT-like, 10k queries, FP32 rerank of k*2), exact results: tensor-core "
              "shortlist vs the integer scan (identical results)")


def run_flat(args, rank, world):
    """Flat or SQ8 scan. Flat: plain FP32 (the reference's IndexFlat
    arithmetic) against the fast form (BF16 shortlist + exact FP32 rerank).
    SQ8: the integer (dp4a) scan against the tensor-core scan over the same
    codes, both with the exact FP32 rerank of k * rerank_factor; the two
    must return identical results. Recall is against the exact FP32 flat
    search, which equals FP64 on these integer-valued rows."""
    import torch

    import mojovec_gb300 as mv

    nb, nq, k, dim = args.nb, args.nq, args.k, args.dim
    sq8 = args.workload == "sq8"
    metric = mv.METRIC_L2 if args.metric == "l2" else mv.METRIC_IP
    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    ctx = mv.Context(dev)
    t_setup = time.perf_counter()
    base, queries = build_workload(nb, nq, dim)
    exact = mv.IndexFlat(dim, metric, ctx=ctx)
    exact.add(base)
    if sq8:
        flat = mv.IndexFlatSQ8(dim, metric, ctx=ctx)
        flat.add(base)
        _, gt_exact = exact.search(queries, k)
        del exact
        factor = args.rerank_factor
        fast = dict(form=mv.FORM_FAST, rerank_factor=factor)
        plain = dict(form=mv.FORM_PLAIN, rerank_factor=factor)
        scan = dict(form=mv.FORM_PLAIN, rerank_factor=factor, plain_scan=True)
        rerank = k * factor
    else:
        flat = exact
        rerank = args.rerank
        fast = dict(form=mv.FORM_FAST, rerank=rerank)
        plain = dict(form=mv.FORM_PLAIN)
        scan = dict(form=mv.FORM_PLAIN, plain_scan=True)
        fp8 = dict(form=mv.FORM_FAST, rerank=rerank, e4m3=True)
    setup_s = time.perf_counter() - t_setup
    d_q = torch.from_numpy(queries).cuda()
    d_dist = torch.empty((nq, k), dtype=torch.float32, device="cuda")
    d_lab = torch.empty((nq, k), dtype=torch.int64, device="cuda")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()

    def make_step(opts):
        def step():
            flat.search_device(d_q.data_ptr(), nq, k, d_dist.data_ptr(), d_lab.data_ptr(),
                               stream=stream.cuda_stream, **opts)
        return step

    # The headline is the plain form (exact results, tensor-core shortlist);
    # the SIMT / integer scan alone and the fast form are timed beside it.
    results = {}
    scan_steps = max(1, min(args.steps, 3))  # the scans alone are 7-30x slower
    cert0 = ctx.certify_stats()
    forms = [("scan", scan, scan_steps), ("plain", plain, args.steps), ("fast", fast, args.steps)]
    if not sq8:
        forms.append(("fp8", fp8, args.steps))
    for name, opts, steps in forms:
        step = make_step(opts)
        for _ in range(args.warmup if name != "scan" else 1):
            step()
        torch.cuda.synchronize()
        results[name] = {"labels": d_lab.cpu().numpy(), "dist": d_dist.cpu().numpy()}
        results[name]["derr"] = distance_error_vs_fp64(base, queries, results[name]["dist"],
                                                       results[name]["labels"], args.metric)
        if world > 1:
            torch.distributed.barrier()
        if name == "plain":
            clocks = ClockSampler(dev)
            clocks.start()
            launches0 = ctx.kernel_launches()
        torch.cuda.nvtx.range_push(f"timed_{args.workload}_{name}")
        ms = _timed_steps(torch, step, steps, stream, flush)
        torch.cuda.nvtx.range_pop()
        if name == "plain":
            launches = ctx.kernel_launches() - launches0
            clk = clocks.stop()
            # Per-stage times from a separate, untimed pass of the same steps.
            ctx.profile(True)
            _timed_steps(torch, step, steps, stream, flush)
            stage = ctx.stage_times()
            ctx.profile(False)
        results[name]["ms"] = _max_over_ranks(torch, world, ms) / steps
    cert1 = ctx.certify_stats()
    gt = results["scan"]["labels"]
    identical = bool(np.array_equal(results["plain"]["labels"], gt) and
                     np.array_equal(results["plain"]["dist"], results["scan"]["dist"]))
    rec = recall_at(gt, results["fast"]["labels"], k)
    if sq8:
        rec_exact = recall_at(gt_exact, results["plain"]["labels"], k)
    value = world * nq / (results["plain"]["ms"] / 1e3)
    scan_qps = world * nq / (results["scan"]["ms"] / 1e3)
    fast_qps = world * nq / (results["fast"]["ms"] / 1e3)

    pinned = torch.empty((nq, dim), dtype=torch.float32).pin_memory()
    pinned.copy_(torch.from_numpy(queries))
    hq = pinned.numpy()
    keep, outs = _pinned_results(torch, nq, k)
    flat.search(hq, k, **plain, **outs)
    if world > 1:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        _, elab = flat.search(hq, k, **plain, **outs)
    e2e_s = _max_over_ranks(torch, world, time.perf_counter() - t0)
    e2e_qps = world * nq * args.steps / e2e_s
    assert np.array_equal(elab, results["plain"]["labels"]), "host and device searches disagree"

    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    tc_peak = float(peaks.get("bf16_tflops", 1900.0))
    gemm_ms, gemm_n = stage.get("flat", (0.0, 0))
    per_launch_ms = gemm_ms / max(gemm_n, 1)
    flops = 2.0 * nq * nb * dim
    achieved = flops / (per_launch_ms / 1e3) / 1e12 if per_launch_ms > 0 else 0.0
    out = {
        "metric": SQ8_METRIC if sq8 else FLAT_METRIC,
        "value": round(value, 1),
        "unit": "queries/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(results["plain"]["ms"], 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "bf16+f32",
        "data": "synthetic SIFT-like (seeded Gaussian mixture, integer-valued), not SIFT1M",
        "config": {
            "workload": f"{'sq8' if sq8 else 'flat'}_{nb}x{dim}_{args.metric}_nq{nq}_k{k}",
            "form": ("plain: SQ8 codes as BF16 on tcgen05 (exact integer dots) + per-row heap, "
                     f"reference formula and tie check, exact FP32 rerank of {rerank}") if sq8 else
                    ("plain: BF16 tcgen05 GEMM + per-row heap shortlist, reference FP32 distances "
                     "of the shortlist, BF16 error-bound certificate, exact scan for open queries"),
            ("identical_to_integer_scan" if sq8 else "identical_to_fp32_scan"): identical,
            **({"recall_at_k_vs_exact_fp32": round(rec_exact, 5)} if sq8 else
               {"queries_recomputed_by_scan": int(cert1["flat_fallback"] - cert0["flat_fallback"])}),
            ("integer_scan_qps" if sq8 else "fp32_scan_qps"): round(scan_qps, 1),
            "speedup_vs_scan": round(value / scan_qps, 2),
            "fast_form_qps": round(fast_qps, 1),
            "fast_form_recall_at_k": round(rec, 5),
            "fast_form": (f"SQ8 fast form (same shortlist path, rerank of {rerank})" if sq8 else
                          f"BF16 shortlist + FP32 rerank of {rerank}"),
            **({} if sq8 else {
                "fp8_form_qps": round(world * nq / (results["fp8"]["ms"] / 1e3), 1),
                "fp8_form_recall_at_k": round(recall_at(gt, results["fp8"]["labels"], k), 5),
                "fp8_form": f"E4M3 (per-row scales) tcgen05 shortlist + FP32 rerank of {rerank}"}),
            "l2_policy": f"inputs larger than L2 ({nb * dim * 2 / 1e6:.0f} MB BF16 rows) and a "
                         "256 MiB flush per step",
            "parallelism": f"replicas x{world}",
            "setup_s": round(setup_s, 1),
        },
        "e2e": {"value": round(e2e_qps, 1), "unit": "queries/s",
                "h2d_bytes_per_step": nq * dim * 4, "d2h_bytes_per_step": nq * k * 12},
        "gpu_launches": int(launches),
        "roofline": {
            "bound": "tensor",
            "kernel": "k_umma_topk (includes the query BF16 conversion)",
            "achieved": round(achieved, 1),
            "peak": tc_peak,
            "peak_source": "measured" if "bf16_tflops" in peaks else "fallback",
            "unit": "TFLOP/s",
            "frac": round(achieved / tc_peak, 4),
            "traffic": None,
            "algorithmic_flops_per_launch": flops,
            "launch_ms": round(per_launch_ms, 4),
        },
        "stages_ms_per_step": {kk: round(v[0] / args.steps, 4) for kk, v in stage.items()},
        "clocks": clk,
        "distance_error_vs_fp64": results["plain"]["derr"],
    }
    out["config"]["fast_form_distance_error_vs_fp64"] = results["fast"]["derr"]
    if not sq8:
        out["config"]["fp8_form_distance_error_vs_fp64"] = results["fp8"]["derr"]
    if rank == 0 and not args.no_cpu and sq8:
        from oracle import oracle as orc

        sample = min(args.cpu_sample // 100, nq)
        threads = os.cpu_count() or 1
        ref = orc.SQ8(dim, metric)
        ref.add(base)
        ref.search(queries[:2], k, nthreads=threads)
        t0 = time.perf_counter()
        _, clab = ref.search(queries[:sample], k, nthreads=threads)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {
            "value": round(sample / dt, 1), "unit": "queries/s", "cores": threads, "kind": "port",
            "sample": f"{sample} of the {nq} queries over all {nb} codes, reference IndexFlatSQ8 "
                      f"integer scan (no rerank), query-parallel on {threads} threads",
        }
    elif rank == 0 and not args.no_cpu:
        from oracle import oracle as orc

        sample = min(args.cpu_sample // 100, nq)
        threads = os.cpu_count() or 1
        orc.flat_search(base, queries[:4], k, metric=metric, nthreads=threads)
        t0 = time.perf_counter()
        _, clab = orc.flat_search(base, queries[:sample], k, metric=metric, nthreads=threads)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {
            "value": round(sample / dt, 1), "unit": "queries/s", "cores": threads, "kind": "port",
            "sample": f"{sample} of the {nq} queries over all {nb} rows, reference IndexFlat "
                      f"arithmetic, query-parallel on {threads} threads",
            "ids_equal_to_gpu_plain": bool(np.array_equal(clab, gt[:sample])),
        }
    return out


def run_reference(args):
    """The oracle (C++ restatement of the reference CPU path) builds the same
    index on the host and answers a bounded query sample."""
    from oracle import oracle as orc

    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    base, queries = build_workload(args.nb, args.nq)
    ref = orc.IVFPQ(D, NLIST, M)
    ref.train(base[:TRAIN_N], niter_coarse=NITER, niter_pq=NITER, nthreads=threads)
    ref.add(base, nthreads=threads)
    setup_s = time.perf_counter() - t0
    sample = min(args.cpu_sample, args.nq)
    q = queries[:sample]
    for _ in range(max(args.warmup, 0)):
        ref.search(q[:32], K, args.nprobe, nthreads=threads, lut_threads=threads)
    times = []
    for _ in range(args.steps):
        t = time.perf_counter()
        rd, rl = ref.search(q, K, args.nprobe, nthreads=threads, lut_threads=threads)
        times.append(time.perf_counter() - t)
    total = sum(times)
    qps = sample * args.steps / total
    derr = distance_error_vs_fp64(base, q, rd, rl) if args.steps else None
    return {
        "distance_error_vs_fp64": derr,
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
            "workload": f"ivfpq_{args.nb}x128_nlist4096_M16_nq{args.nq}_k10",
            "form": "reference CPU path (oracle port)",
            "nprobe": args.nprobe,
            "nb": args.nb, "d": D, "nlist": NLIST, "M": M, "nq": args.nq, "k": K,
            "train_rows": TRAIN_N, "train_niter": NITER,
            "setup_s": round(setup_s, 1),
        },
        "cpu_baseline": {
            "value": round(qps, 1),
            "unit": "queries/s",
            "cores": threads,
            "kind": "port",
            "sample": f"{sample} queries per step of the {args.nq}; index trained and filled by the "
                      f"oracle on the CPU; coarse and LUT+ADC query-parallel on {threads} threads",
        },
        "e2e": {"value": round(qps, 1), "unit": "queries/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }


KM_METRIC = "k-means training throughput (1M x 96 cosine mixture, k 16384, 25 iterations)"
BATCH_METRIC = ("Batched uneven IVF-PQ QPS (10M x 96 cosine, nlist 16384, M 24, 20k queries, "
                "nprobe U{8..256}, k U{1,10,100}), tuned persistent scan under a CUDA graph")


def run_batch(args, rank, world):
    """Batched uneven IVF-PQ: per-query nprobe drawn from {8, ..., 256} and k
    from {1, 10, 100} (seeded), one plan replayed as a CUDA graph after the
    tuner picked its launch shapes. Inputs (queries, per-query parameters)
    are resident in the plan's device buffers when `value` is timed; `e2e`
    is the host-buffer call mv_ivfpq_search_batch (copies included). The
    untuned, graph-free run of the same plan is timed beside it."""
    import torch

    import mojovec_gb300 as mv
    from mojovec_gb300 import synth

    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    ctx = mv.Context(dev)
    nb, nq, d = args.batch_nb, args.batch_nq, 96
    t0 = time.perf_counter()
    base, queries = synth.cos_mixture(nb, d=d, n_centers=4096, std=0.05, nq=nq)
    gen_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    ix = mv.IndexIVFPQ(d, 16384, 24, mv.METRIC_IP, ctx=ctx)
    ix.train(base[: min(nb, 1_000_000)], niter_coarse=25, niter_pq=15, form=mv.FORM_FAST)
    for r0 in range(0, nb, 2_000_000):
        ix.add(base[r0:r0 + 2_000_000])
    build_s = time.perf_counter() - t0
    rng = np.random.default_rng(np.random.SeedSequence(20261203).spawn(8)[5])
    nprobe = rng.integers(8, 257, size=nq).astype(np.int32)
    k = rng.choice(np.array([1, 10, 100], np.int32), size=nq)
    rerank = 200
    plan = mv.IVFPQBatchPlan(ix, nq, 256, 100, rerank=rerank, lut=args.lut)
    plan.set_queries(queries, nprobe, k)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()

    def timed(step, steps):
        return _timed_steps(torch, step, steps, stream, flush) / steps

    # untuned, one CTA per query... the plan's defaults, no graph
    plan.run(nq, use_graph=False, stream=stream.cuda_stream)
    untuned_ms = timed(lambda: plan.run(nq, use_graph=False, stream=stream.cuda_stream), 3)
    cfg = plan.tune(nq)
    plan.run(nq, use_graph=True, stream=stream.cuda_stream)
    for _ in range(args.warmup):
        plan.run(nq, use_graph=True, stream=stream.cuda_stream)
    clocks = ClockSampler(dev)
    clocks.start()
    l0 = ctx.kernel_launches()
    torch.cuda.nvtx.range_push("timed_batch")
    ms = timed(lambda: plan.run(nq, use_graph=True, stream=stream.cuda_stream), args.steps)
    torch.cuda.nvtx.range_pop()
    launches = ctx.kernel_launches() - l0
    clk = clocks.stop()
    dist, lab = plan.results(nq)
    # e2e: host-buffer batch call
    t0 = time.perf_counter()
    e2e_steps = max(2, min(args.steps, 5))
    for _ in range(e2e_steps):
        ix.search_batch(queries, nprobe, k, rerank=rerank, lut=args.lut)
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    # recall@10 on a sample of the k >= 10 queries against the fast flat
    # search with a deep exact rerank (BF16 shortlist of 400, FP32 distances)
    sel = np.where(k >= 10)[0][:500]
    flat = mv.IndexFlat(d, mv.METRIC_IP, ctx=ctx)
    flat.add(base)
    _, gt = flat.search(queries[sel], 10, form=mv.FORM_FAST, rerank=400)
    rec = recall_at(gt, lab[sel, :10], 10)
    sizes = np.diff(ix.lists()[0])
    adc_bytes = float(nprobe.sum()) * float(sizes.mean()) * 24  # mean-list approximation
    hbm_peak = (float(json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))).get("hbm_gbs", 6800.0))
                if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")) else 6800.0)
    achieved = adc_bytes / (ms / 1e3) / 1e9
    out = {
        "metric": BATCH_METRIC,
        "value": round(nq / (ms / 1e3), 1),
        "unit": "queries/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "bf16+f32",
        "data": "synthetic unit-normalised Gaussian mixture (seeded), not a public dataset",
        "config": {
            "workload": f"ivfpq_batch_{nb}x96_nlist16384_M24_nq{nq}",
            "form": f"fast: BF16 coarse GEMM + FP32 recheck, persistent LUT/ADC scan, "
                    f"exact FP32 rerank of {rerank}; one CUDA graph per batch",
            "tuned": cfg,
            "untuned_no_graph_ms": round(untuned_ms, 4),
            "speedup_tuned_graph_vs_untuned": round(untuned_ms / ms, 3),
            "mean_nprobe": float(nprobe.mean()),
            "recall_at_10_sample": round(rec, 4),
            "recall_reference": "fast flat search (BF16 shortlist 400 + exact FP32 rerank), "
                                "500 queries with k >= 10",
            "adc_bytes_per_step_approx": adc_bytes,
            "data_gen_s": round(gen_s, 1), "index_build_s": round(build_s, 1),
            "l2_policy": "codes (240 MB) larger than L2, plus a 256 MiB flush per step",
        },
        "e2e": {"value": round(nq / e2e_s, 1), "unit": "queries/s",
                "h2d_bytes_per_step": nq * d * 4 + nq * 8,
                "d2h_bytes_per_step": nq * 100 * 12},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "kernel": "whole batch (ADC bytes, mean-list approximation)",
                     "achieved": round(achieved, 1), "peak": hbm_peak,
                     "frac": round(achieved / hbm_peak, 4), "unit": "GB/s", "traffic": None},
        "clocks": clk,
        "distance_error_vs_fp64": distance_error_vs_fp64(base, queries, dist, lab, "ip"),
    }
    if not args.no_cpu:
        # The oracle (plain IVF-PQ restatement) over the same lists, on a
        # bounded sample of the batch, each query with its own nprobe, k 100.
        from oracle import oracle as orc

        threads = os.cpu_count() or 1
        cent, pq = ix.codebooks()
        off, ids, codes = ix.lists()
        ref = orc.IVFPQ(d, 16384, 24, orc.METRIC_IP)
        ref.set_codebooks(cent, pq)
        ref.set_lists(off, ids, codes)
        smp = np.random.default_rng(7).choice(nq, 200, replace=False)
        t0 = time.perf_counter()
        for npv in np.unique(nprobe[smp]):
            grp = smp[nprobe[smp] == npv]
            ref.search(queries[grp], 100, int(npv), nthreads=threads, lut_threads=threads)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {
            "value": round(len(smp) / dt, 1), "unit": "queries/s", "cores": threads,
            "kind": "port",
            "sample": f"200 of the {nq} queries with their own nprobe and k 100, plain IVF-PQ "
                      f"restatement over the GPU index's lists, query-parallel on {threads} threads",
        }
    return out


def run_kmeans(args, rank, world):
    """k-means training as the IVF coarse quantizer of the batched workload:
    1,000,000 x 96 rows of a 4,096-component unit-normalised mixture (per-dim
    std 0.05, rows L2-normalised), 16,384 centroids, 25 iterations. Both
    forms run through the public C ABI (mv_kmeans_train_ex); the device time
    of the training is taken from the context's stage events (inputs already
    copied), e2e includes the host->device copy of the rows and the copy back
    of centroids and assignments. The objective (sum of squared distances of
    the final centroids) of the fast form is compared with the plain,
    reference-exact form's."""
    import torch

    import mojovec_gb300 as mv
    from mojovec_gb300 import synth

    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    ctx = mv.Context(dev)
    n, d, k, niter = args.km_n, 96, args.km_k, args.km_iter
    x, _ = synth.cos_mixture(n, d=d, n_centers=4096, std=0.05)
    out = {}
    for name, form in (("plain", mv.FORM_PLAIN), ("fast", mv.FORM_FAST)):
        km = mv.KMeans(d, k, niter=niter, ctx=ctx, form=form)
        if name == "fast":  # warm-up of the fast path (kernels, smem limits)
            mv.KMeans(d, k, niter=1, ctx=ctx, form=form).train(x[:200000])
        clocks = ClockSampler(dev)
        clocks.start()
        ctx.profile(True)
        l0 = ctx.kernel_launches()
        t0 = time.perf_counter()
        torch.cuda.nvtx.range_push(f"timed_kmeans_{name}")
        km.train(x)
        torch.cuda.nvtx.range_pop()
        e2e_s = time.perf_counter() - t0
        st = ctx.stage_times()
        ctx.profile(False)
        out[name] = {"km": km, "dev_ms": st.get("coarse", (0.0, 0))[0], "e2e_s": e2e_s,
                     "launches": ctx.kernel_launches() - l0, "clocks": clocks.stop()}
    f, p = out["fast"], out["plain"]
    rel = abs(f["km"].objective[-1] - p["km"].objective[-1]) / p["km"].objective[-1]
    # The fast form's final objective against the same sum recomputed in FP64
    # on the host from its centroids and assignments.
    obj64 = 0.0
    for r0 in range(0, n, 1 << 17):
        xa = x[r0:r0 + (1 << 17)].astype(np.float64)
        ca = f["km"].centroids[f["km"].assignments[r0:r0 + (1 << 17)]].astype(np.float64)
        obj64 += float(((xa - ca) ** 2).sum())
    obj_rel = abs(f["km"].objective[-1] - obj64) / obj64
    value = niter / (f["dev_ms"] / 1e3)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    tc_peak = float(peaks.get("bf16_tflops", 1900.0))
    flops = 2.0 * n * k * d * (niter + 1)  # assignment GEMMs (niter steps + final objective)
    achieved = flops / (f["dev_ms"] / 1e3) / 1e12
    return {
        "metric": KM_METRIC,
        "value": round(value, 3),
        "unit": "iterations/s",
        "n_gpus": 1, "steps": niter, "warmup": 1,
        "ms_per_step": round(f["dev_ms"] / niter, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "bf16+f32+f64",
        "data": "synthetic unit-normalised Gaussian mixture (seeded), not a public dataset",
        "config": {
            "workload": f"kmeans_{n}x{d}_k{k}_iter{niter}",
            "form": "fast: tcgen05 BF16 candidates (4 per row) + FP32 recheck, FP64 ordered sums",
            "objective_fast": f["km"].objective[-1],
            "objective_plain": p["km"].objective[-1],
            "objective_rel_diff": rel,
            "plain_iterations_per_s": round(niter / (p["dev_ms"] / 1e3), 3),
            "speedup_vs_plain": round(p["dev_ms"] / f["dev_ms"], 2),
        },
        "e2e": {"value": round(niter / f["e2e_s"], 3), "unit": "iterations/s",
                "h2d_bytes_per_step": n * d * 4 // niter, "d2h_bytes_per_step": (k * d * 4 + n * 8) // niter},
        "gpu_launches": int(f["launches"]),
        "roofline": {"bound": "tensor", "kernel": "whole training (assignment GEMMs counted)",
                     "achieved": round(achieved, 1), "peak": tc_peak, "unit": "TFLOP/s",
                     "frac": round(achieved / tc_peak, 4), "traffic": None},
        "clocks": f["clocks"],
        "distance_error_vs_fp64": {"max_rel": float(f"{obj_rel:.3e}"), "mean_rel": None,
                                   "definition": "final objective (sum of squared distances to "
                                                 "the assigned centroids) against its FP64 "
                                                 "recomputation from the same centroids and "
                                                 "assignments"},
    }


SERVE_METRIC = ("Serving: sustained QPS and p50/p99 latency, 3 resident collections "
                "(IVF-PQ 1Mx128, SQ8 2Mx768 cosine, Flat 500kx256 IP), Poisson arrivals")


def run_serve(args, rank, world):
    """Serving loop over three resident collections: (a) IVF-PQ 1M x 128 L2
    (nlist 4096, M 16), (b) SQ8 2M x 768 cosine (rows L2-normalised, 2,048-
    component mixture), (c) Flat 500k x 256 IP (unnormalised SIFT-like).
    Requests arrive as a Poisson process at each offered rate, each a batch
    of 1-1024 queries (log-uniform) to a random collection with k in
    {10, 100}, all seeded. The plain form and the precision+batched form are
    served in turn through mv_server_* (continuous batching, 4 lanes, HBM
    budget); latency is submit-to-completion per request."""
    import threading

    import torch

    import mojovec_gb300 as mv
    from mojovec_gb300 import synth

    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    ctx = mv.Context(dev)
    s = args.serve_scale
    t0 = time.perf_counter()
    a_base, a_q = synth.sift_like(int(1_000_000 * s), d=128, n_centers=1024, nq=4096)
    b_base, b_q = synth.cos_mixture(int(2_000_000 * s), d=768, n_centers=2048, std=0.05, nq=4096,
                                    seed=synth.BASE_SEED + 7)
    c_base, c_q = synth.sift_like(int(500_000 * s), d=256, n_centers=1024, nq=4096,
                                  seed=synth.BASE_SEED + 9)
    ivf = mv.IndexIVFPQ(128, 4096, 16, mv.METRIC_L2, ctx=ctx)
    ivf.train(a_base[:131072], niter_coarse=10, niter_pq=10, form=mv.FORM_FAST)
    ivf.add(a_base)
    sq8 = mv.IndexFlatSQ8(768, mv.METRIC_IP, ctx=ctx)
    sq8.add(b_base)
    flat = mv.IndexFlat(256, mv.METRIC_IP, ctx=ctx)
    flat.add(c_base)
    setup_s = time.perf_counter() - t0
    colls = [("ivfpq_1Mx128_l2", ivf, a_q), ("sq8_2Mx768_cos", sq8, b_q),
             ("flat_500kx256_ip", flat, c_q)]
    forms = {
        "plain": [dict(form=mv.FORM_PLAIN, nprobe=8), dict(form=mv.FORM_PLAIN, rerank_factor=2),
                  dict(form=mv.FORM_PLAIN)],
        "fast": [dict(form=mv.FORM_FAST, nprobe=8, rerank=224),
                 dict(form=mv.FORM_FAST, rerank_factor=2), dict(form=mv.FORM_FAST, rerank=40)],
    }
    rng = np.random.default_rng(np.random.SeedSequence(20261203).spawn(8)[6])
    nreq = args.serve_requests
    sizes = np.exp(rng.uniform(0, np.log(1024), size=nreq)).astype(np.int64).clip(1, 1024)
    which = rng.integers(0, 3, size=nreq)
    ks = rng.choice([10, 100], size=nreq)
    offsets = [int(rng.integers(0, 4096 - 1024)) for _ in range(nreq)]
    gaps = rng.exponential(1.0, size=nreq)

    def recall_of(form_name):
        out, err = {}, {}
        for ci, (name, idx, q) in enumerate(colls):
            qq = q[:200]
            opts = dict(forms[form_name][ci])
            if isinstance(idx, mv.IndexFlatSQ8):
                d_, l_ = idx.search(qq, 10, **opts)
                gt_idx = mv.IndexFlat(idx.d, mv.METRIC_IP, ctx=ctx)
                gt_idx.add(b_base)
            elif isinstance(idx, mv.IndexIVFPQ):
                d_, l_ = idx.search(qq, 10, **opts)
                gt_idx = mv.IndexFlat(128, mv.METRIC_L2, ctx=ctx)
                gt_idx.add(a_base)
            else:
                d_, l_ = idx.search(qq, 10, **opts)
                gt_idx = flat
            _, gt = gt_idx.search(qq, 10)
            out[name] = round(recall_at(gt, l_, 10), 4)
            rows = a_base if ci == 0 else (b_base if ci == 1 else c_base)
            err[name] = distance_error_vs_fp64(rows, qq, d_, l_, "l2" if ci == 0 else "ip")
            del gt_idx
        return out, err

    results = {}
    clocks = ClockSampler(dev)
    for form_name in ("plain", "fast"):
        srv = mv.Server(ctx=ctx, hbm_budget=args.serve_budget_gb << 30, lanes=4,
                        max_batch_queries=4096)
        ids = [srv.add(idx, **forms[form_name][ci]) for ci, (_, idx, _) in enumerate(colls)]
        # warm-up: one request per collection and k
        for ci, (_, idx, q) in enumerate(colls):
            for k in (10, 100):
                srv.wait(srv.submit(ids[ci], q[:64], k))
        per_rate = []
        if form_name == "fast":
            clocks.start()
        for rate in args.serve_rates:
            times = np.cumsum(gaps / rate)
            lat = [None] * nreq
            rids = [None] * nreq
            done_q = [0]

            def waiter():
                for i in range(nreq):
                    while rids[i] is None:
                        time.sleep(0.0002)
                    _, _, lat[i] = srv.wait(rids[i])

            th = threading.Thread(target=waiter)
            th.start()
            t_start = time.perf_counter()
            for i in range(nreq):
                dt = t_start + times[i] - time.perf_counter()
                if dt > 0:
                    time.sleep(dt)
                _, _, q = colls[which[i]]
                rids[i] = srv.submit(ids[which[i]], q[offsets[i]:offsets[i] + sizes[i]], int(ks[i]))
            th.join()
            wall = time.perf_counter() - t_start
            lat_ms = np.array(lat) * 1e3
            per_rate.append({
                "offered_requests_per_s": rate,
                "offered_queries_per_s": round(float(rate * sizes.mean()), 1),
                "sustained_queries_per_s": round(float(sizes.sum() / wall), 1),
                "p50_ms": round(float(np.percentile(lat_ms, 50)), 3),
                "p99_ms": round(float(np.percentile(lat_ms, 99)), 3),
            })
        if form_name == "fast":
            clk = clocks.stop()
        st = srv.stats()
        srv.close()
        rec, derr = recall_of(form_name)
        results[form_name] = {"rates": per_rate, "recall_at_10": rec,
                              "distance_error_vs_fp64": derr,
                              "batches": st["batches"], "batched_queries": st["batched_queries"],
                              "peak_inflight_gb": round(st["peak_inflight_bytes"] / 2**30, 2)}
    top = results["fast"]["rates"][-1]
    return {
        "metric": SERVE_METRIC,
        "value": top["sustained_queries_per_s"],
        "unit": "queries/s",
        "n_gpus": 1, "steps": nreq, "warmup": 6, "ms_per_step": None,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "bf16+f32 (fast) / f32 + int8 (plain)",
        "data": "synthetic seeded mixtures (SIFT-like and unit-normalised), not public datasets",
        "config": {
            "workload": f"serve_ivfpq1M_sq8_2Mx768_flat500kx256_req{nreq}_scale{s}",
            "arrivals": "Poisson; batch size log-uniform on [1, 1024]; collection uniform; k in {10, 100}",
            "server": f"4 lanes, HBM budget {args.serve_budget_gb} GB, batches up to 4096 queries",
            "forms": {"plain": "IVF-PQ plain nprobe 8; SQ8 integer keys from the tensor cores "
                               "(exact for s8 codes at d <= 1040) + FP32 rerank of 2k; Flat exact "
                               "FP32 (certified tensor-core shortlist)",
                      "fast": "IVF-PQ fast nprobe 8 rerank 224; SQ8 as plain; Flat BF16 + FP32 "
                              "rerank of max(k, 40)"},
            "results": results,
            "setup_s": round(setup_s, 1),
        },
        "e2e": {"value": top["sustained_queries_per_s"], "unit": "queries/s",
                "h2d_bytes_per_step": None, "d2h_bytes_per_step": None},
        "distance_error_vs_fp64": {
            "max_rel": max(v["max_rel"] for v in results["fast"]["distance_error_vs_fp64"].values()),
            "mean_rel": None,
            "definition": "largest over the collections, fast form; per collection and form in "
                          "config.results"},
        "gpu_launches": None,
        "clocks": clk,
    }


CURVE_METRIC = "IVF-PQ QPS-recall curve (1M x 128 SIFT-like, nlist 4096, M 16/32, 10k queries, k 10)"


def run_curve(args, rank, world):
    """QPS against recall@10 for nprobe 8..128 and M 16 / 32: the plain form
    and fast variants (BF16 or FP32 coarse, FP32 or FP16 tables, with and
    without the exact rerank of 40). Device-resident queries, CUDA events,
    L2 flushed per step; recall against the exact FP32 flat search (equal to
    FP64 on these integer-valued rows)."""
    import torch

    import mojovec_gb300 as mv

    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    ctx = mv.Context(dev)
    base, queries = build_workload(args.nb, args.nq)
    nq = queries.shape[0]
    flat = mv.IndexFlat(D, mv.METRIC_L2, ctx=ctx)
    flat.add(base)
    _, gt = flat.search(queries, K)
    del flat
    d_q = torch.from_numpy(queries).cuda()
    d_dist = torch.empty((nq, K), dtype=torch.float32, device="cuda")
    d_lab = torch.empty((nq, K), dtype=torch.int64, device="cuda")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    variants = {
        "plain": dict(form=mv.FORM_PLAIN),
        "fast_bf16coarse_fp32lut_rerank40": dict(form=mv.FORM_FAST, rerank=40),
        "fast_fp32coarse_fp32lut_rerank40": dict(form=mv.FORM_FAST, rerank=40, coarse_fp32=True),
        "fast_bf16coarse_fp16lut_rerank40": dict(form=mv.FORM_FAST, rerank=40, lut_fp16=True),
        "fast_bf16coarse_fp32lut_norerank": dict(form=mv.FORM_FAST),
    }
    curve = []
    for m in (16, 32):
        index = mv.IndexIVFPQ(D, NLIST, m, mv.METRIC_L2, ctx=ctx)
        index.train(base[:TRAIN_N], niter_coarse=NITER, niter_pq=NITER)
        index.add(base)
        for nprobe in (8, 16, 32, 64, 128):
            for name, opts in variants.items():
                def step():
                    index.search_device(d_q.data_ptr(), nq, K, d_dist.data_ptr(), d_lab.data_ptr(),
                                        stream=stream.cuda_stream, nprobe=nprobe, **opts)
                step()
                torch.cuda.synchronize()
                lab = d_lab.cpu().numpy()
                rec = recall_at(gt, lab, K)
                derr = distance_error_vs_fp64(base, queries, d_dist.cpu().numpy(), lab)
                steps = 3 if name == "plain" else 5
                ms = _timed_steps(torch, step, steps, stream, flush) / steps
                curve.append({"M": m, "nprobe": nprobe, "variant": name,
                              "qps": round(nq / (ms / 1e3), 1), "recall_at_10": round(rec, 4),
                              "dist_err_max_rel": derr["max_rel"],
                              "dist_err_mean_rel": derr["mean_rel"]})
        del index
    head = [c for c in curve if c["M"] == 16 and c["nprobe"] == 16 and
            c["variant"] == "fast_bf16coarse_fp32lut_rerank40"][0]
    return {
        "metric": CURVE_METRIC, "value": head["qps"], "unit": "queries/s", "n_gpus": 1,
        "steps": 5, "warmup": 1, "ms_per_step": round(nq / head["qps"] * 1e3, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "bf16+f32",
        "data": "synthetic SIFT-like (seeded Gaussian mixture, integer-valued), not SIFT1M",
        "config": {"workload": f"ivfpq_curve_{args.nb}x128_nlist4096_nq{nq}_k10",
                   "value_is": "M 16, nprobe 16, BF16 coarse, FP32 tables, rerank 40",
                   "curve": curve},
        "distance_error_vs_fp64": {"max_rel": head["dist_err_max_rel"],
                                   "mean_rel": head["dist_err_mean_rel"],
                                   "definition": "per point of the curve in config.curve"},
        "e2e": None, "gpu_launches": None,
    }


IVFFLAT_METRIC = ("IVF-Flat QPS (1Mx128 SIFT-like, nlist 4096, nprobe 8, 10k queries, k 10): exact "
                  "per-list FP32 scan; plain bit-exact (certified tensor-core coarse step)")
IVFFLAT_TRAIN, IVFFLAT_NITER = 65536, 8
RERANK_METRIC = ("Shortlist rerank QPS (1Mx128 SIFT-like FP32 rows, 10k queries, 2k = 20 candidates "
                 "each, k 10), exact FP32 l2_distance_simd[64] semantics")


def _build_ivfflat(mv, base, ctx=None):
    ix = mv.IndexIVFFlat(D, NLIST, mv.METRIC_L2, **({"ctx": ctx} if ctx else {}))
    ix.train(base[:IVFFLAT_TRAIN], niter=IVFFLAT_NITER)
    ix.add(base)
    return ix


def run_ivfflat(args, rank, world):
    """IVF-Flat search (index/index_ivf_flat.mojo:149-243): the plain form
    (bit-exact, certified coarse step) is the line's value, the fast form
    (BF16 two-pass coarse step) is timed beside it."""
    import torch

    import mojovec_gb300 as mv

    nb, nq, k, nprobe = args.nb, args.nq, K, args.nprobe
    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    ctx = mv.Context(dev)
    t0 = time.perf_counter()
    base, queries = build_workload(nb, nq)
    ix = _build_ivfflat(mv, base, ctx)
    flat = mv.IndexFlat(D, mv.METRIC_L2, ctx=ctx)
    flat.add(base)
    _, gt = flat.search(queries, k)
    del flat
    setup_s = time.perf_counter() - t0
    d_q = torch.from_numpy(queries).cuda()
    d_dist = torch.empty((nq, k), dtype=torch.float32, device="cuda")
    d_lab = torch.empty((nq, k), dtype=torch.int64, device="cuda")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    res = {}
    for name, form in (("fast", mv.FORM_FAST), ("plain", mv.FORM_PLAIN)):
        def step(form=form):
            ix.search_device(d_q.data_ptr(), nq, k, d_dist.data_ptr(), d_lab.data_ptr(),
                             stream=stream.cuda_stream, nprobe=nprobe, form=form)
        for _ in range(args.warmup):
            step()
        torch.cuda.synchronize()
        lab = d_lab.cpu().numpy()
        derr = distance_error_vs_fp64(base, queries, d_dist.cpu().numpy(), lab)
        if name == "plain":
            clocks = ClockSampler(dev)
            clocks.start()
            launches0 = ctx.kernel_launches()
        torch.cuda.nvtx.range_push(f"timed_ivfflat_{name}")
        ms = _timed_steps(torch, step, args.steps, stream, flush) / args.steps
        torch.cuda.nvtx.range_pop()
        if name == "plain":
            launches = ctx.kernel_launches() - launches0
            clk = clocks.stop()
            ctx.profile(True)
            _timed_steps(torch, step, args.steps, stream, flush)
            stage = ctx.stage_times()
            ctx.profile(False)
        res[name] = {"ms": _max_over_ranks(torch, world, ms), "labels": lab, "derr": derr}
    value = world * nq / (res["plain"]["ms"] / 1e3)
    pinned = torch.empty((nq, D), dtype=torch.float32).pin_memory()
    pinned.copy_(torch.from_numpy(queries))
    hq = pinned.numpy()
    keep, outs = _pinned_results(torch, nq, k)
    ix.search(hq, k, nprobe=nprobe, **outs)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        _, elab = ix.search(hq, k, nprobe=nprobe, **outs)
    e2e_qps = world * nq * args.steps / _max_over_ranks(torch, world, time.perf_counter() - t0)
    assert np.array_equal(elab, res["plain"]["labels"]), "host and device searches disagree"
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    scan_ms, scan_n = stage.get("scan", (0.0, 0))
    per_launch = scan_ms / max(scan_n, 1)
    mean_list = nb / NLIST
    alg_bytes = nq * nprobe * mean_list * D * 4
    achieved = alg_bytes / (per_launch / 1e3) / 1e9 if per_launch > 0 else 0.0
    out = {
        "metric": IVFFLAT_METRIC, "value": round(value, 1), "unit": "queries/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(res["plain"]["ms"], 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic SIFT-like (seeded Gaussian mixture, integer-valued), not SIFT1M",
        "config": {
            "workload": f"ivfflat_{nb}x128_nlist{NLIST}_nprobe{nprobe}_nq{nq}_k{k}",
            "train_rows": IVFFLAT_TRAIN, "train_niter": IVFFLAT_NITER,
            "recall_at_10_vs_exact": round(recall_at(gt, res["plain"]["labels"], k), 4),
            "fast_form_qps": round(world * nq / (res["fast"]["ms"] / 1e3), 1),
            "fast_form_recall_at_10": round(recall_at(gt, res["fast"]["labels"], k), 4),
            "fast_form": "BF16 two-pass tcgen05 coarse + FP32 recheck, same exact list scan",
            "l2_policy": "rows (512 MB) larger than L2, plus a 256 MiB flush per step",
            "parallelism": f"replicas x{world}", "setup_s": round(setup_s, 1),
        },
        "e2e": {"value": round(e2e_qps, 1), "unit": "queries/s",
                "h2d_bytes_per_step": nq * D * 4, "d2h_bytes_per_step": nq * k * 12},
        "gpu_launches": int(launches),
        "roofline": {
            "bound": "hbm", "kernel": "k_lm_scan (exact FP32 list-major scan) + count/place/merge",
            "achieved": round(achieved, 1), "peak": hbm,
            "peak_source": "measured" if "hbm_gbs" in peaks else "fallback", "unit": "GB/s",
            "frac": round(achieved / hbm, 4), "traffic": None,
            "algorithmic_bytes_per_launch": int(alg_bytes),
            "note": ("row bytes of the probed lists per query, mean-list approximation (nb / nlist "
                     "rows each); the list-major scan reads each list once per 4 of its queries, "
                     "so DRAM traffic is below these algorithmic bytes"),
            "launch_ms": round(per_launch, 4),
        },
        "stages_ms_per_step": {kk: round(v[0] / args.steps, 4) for kk, v in stage.items()},
        "clocks": clk,
        "distance_error_vs_fp64": res["plain"]["derr"],
    }
    out["config"]["fast_form_distance_error_vs_fp64"] = res["fast"]["derr"]
    if rank == 0 and not args.no_cpu:
        from oracle import oracle as orc

        threads = os.cpu_count() or 1
        ref = orc.IVFFlat(D, NLIST, 0)
        ref.train(base[:IVFFLAT_TRAIN], niter=IVFFLAT_NITER, nthreads=threads)
        ref.add(base, nthreads=threads)
        sample = min(args.cpu_sample // 2, nq)
        ref.search(queries[:4], k, nprobe, nthreads=threads)
        t0 = time.perf_counter()
        _, clab = ref.search(queries[:sample], k, nprobe, nthreads=threads)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {
            "value": round(sample / dt, 1), "unit": "queries/s", "cores": threads, "kind": "port",
            "sample": f"{sample} of the {nq} queries; index trained and filled by the oracle on "
                      f"the CPU; query-parallel on {threads} threads",
            "ids_equal_to_gpu_plain": bool(np.array_equal(clab, res["plain"]["labels"][:sample])),
        }
    return out


def _rerank_workload(mv, nb, nq, k, ctx=None):
    base, queries = build_workload(nb, nq)
    flat = mv.IndexFlat(D, mv.METRIC_L2, **({"ctx": ctx} if ctx else {}))
    flat.add(base)
    rng = np.random.default_rng(np.random.SeedSequence(20261203).spawn(8)[5])
    # the shortlist: the 2k nearest rows in a random order (as a graph walk
    # would hand them over)
    _, cand = flat.search(queries, 2 * k)
    cand = np.take_along_axis(cand, rng.permuted(np.tile(np.arange(2 * k), (nq, 1)), axis=1), 1)
    return base, queries, flat, np.ascontiguousarray(cand, np.int64)


def run_rerank(args, rank, world):
    """The exact rerank service for a shortlist (index/index_hnsw.mojo:433-497)."""
    import torch

    import mojovec_gb300 as mv

    nq, k = args.nq, K
    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    ctx = mv.Context(dev)
    base, queries, flat, cand = _rerank_workload(mv, args.nb, nq, k, ctx)
    ncand = cand.shape[1]
    d_q = torch.from_numpy(queries).cuda()
    d_c = torch.from_numpy(cand).cuda()
    d_dist = torch.empty((nq, k), dtype=torch.float32, device="cuda")
    d_lab = torch.empty((nq, k), dtype=torch.int64, device="cuda")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()

    def step():
        flat.rerank_device(d_q.data_ptr(), nq, d_c.data_ptr(), ncand, k, d_dist.data_ptr(),
                           d_lab.data_ptr(), stream=stream.cuda_stream)
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    lab = d_lab.cpu().numpy()
    clocks = ClockSampler(dev)
    clocks.start()
    l0 = ctx.kernel_launches()
    torch.cuda.nvtx.range_push("timed_rerank")
    ms = _timed_steps(torch, step, args.steps, stream, flush) / args.steps
    torch.cuda.nvtx.range_pop()
    launches = ctx.kernel_launches() - l0
    clk = clocks.stop()
    ms = _max_over_ranks(torch, world, ms)
    hd, hl = flat.rerank(queries, cand, k)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        hd, hl = flat.rerank(queries, cand, k)
    e2e_qps = world * nq * args.steps / _max_over_ranks(torch, world, time.perf_counter() - t0)
    assert np.array_equal(hl, lab), "host and device reranks disagree"
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    alg = nq * ncand * D * 4
    achieved = alg / (ms / 1e3) / 1e9
    out = {
        "metric": RERANK_METRIC, "value": round(world * nq / (ms / 1e3), 1), "unit": "queries/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic SIFT-like rows; shortlists are each query's 20 nearest rows, shuffled",
        "config": {"workload": f"rerank_{args.nb}x128_nq{nq}_ncand{ncand}_k{k}",
                   "parallelism": f"replicas x{world}",
                   "l2_policy": "rows (512 MB) larger than L2, plus a 256 MiB flush per step"},
        "e2e": {"value": round(e2e_qps, 1), "unit": "queries/s",
                "h2d_bytes_per_step": nq * D * 4 + nq * ncand * 8, "d2h_bytes_per_step": nq * k * 12},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "kernel": "k_rerank_simd64 (whole step)",
                     "achieved": round(achieved, 1), "peak": hbm,
                     "peak_source": "measured" if "hbm_gbs" in peaks else "fallback",
                     "unit": "GB/s", "frac": round(achieved / hbm, 4), "traffic": None,
                     "algorithmic_bytes_per_launch": int(alg),
                     "note": "candidate rows gathered (nq x 2k x d x 4 bytes); latency-bound at this size"},
        "clocks": clk,
        "distance_error_vs_fp64": distance_error_vs_fp64(base, queries, hd, hl),
    }
    if rank == 0 and not args.no_cpu:
        from oracle import oracle as orc

        threads = os.cpu_count() or 1
        sample = min(nq, 2000)
        orc.rerank(base, queries[:4], cand[:4], k, nthreads=threads)
        t0 = time.perf_counter()
        _, clab = orc.rerank(base, queries[:sample], cand[:sample], k, nthreads=threads)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {
            "value": round(sample / dt, 1), "unit": "queries/s", "cores": threads, "kind": "port",
            "sample": f"{sample} of the {nq} queries, query-parallel on {threads} threads",
            "ids_equal_to_gpu": bool(np.array_equal(clab, lab[:sample])),
        }
    return out


def run_reference_ivfflat(args):
    """The oracle's IVF-Flat (same training recipe) on a bounded query sample."""
    from oracle import oracle as orc

    threads = os.cpu_count() or 1
    base, queries = build_workload(args.nb, args.nq)
    ref = orc.IVFFlat(D, NLIST, 0)
    ref.train(base[:IVFFLAT_TRAIN], niter=IVFFLAT_NITER, nthreads=threads)
    ref.add(base, nthreads=threads)
    sample = min(max(args.cpu_sample // 2, 1), args.nq)
    for _ in range(args.warmup):
        ref.search(queries[:4], K, args.nprobe, nthreads=threads)
    t = time.perf_counter()
    for _ in range(args.steps):
        rd, rl = ref.search(queries[:sample], K, args.nprobe, nthreads=threads)
    total = time.perf_counter() - t
    qps = sample * args.steps / total
    return _reference_line(args, IVFFLAT_METRIC, qps, total, threads,
                           f"ivfflat_{args.nb}x128_nlist{NLIST}_nprobe{args.nprobe}_nq{args.nq}_k{K}",
                           f"{sample} queries per step, query-parallel on {threads} threads",
                           distance_error_vs_fp64(base, queries[:sample], rd, rl))


def run_reference_rerank(args):
    """The oracle's rerank (l2_distance_simd[64] semantics) on a bounded sample."""
    import mojovec_gb300  # noqa: F401  (synthetic data generator only)
    from oracle import oracle as orc

    threads = os.cpu_count() or 1
    base, queries = build_workload(args.nb, args.nq)
    rng = np.random.default_rng(np.random.SeedSequence(20261203).spawn(8)[5])
    sample = min(args.nq, 2000)
    q = queries[:sample]
    # shortlists: the 20 nearest rows by the oracle's exact search, shuffled
    _, cand = orc.flat_search(base, q, 2 * K, nthreads=threads)
    cand = np.ascontiguousarray(np.take_along_axis(
        cand, rng.permuted(np.tile(np.arange(2 * K), (sample, 1)), axis=1), 1), np.int64)
    for _ in range(args.warmup):
        orc.rerank(base, q[:4], cand[:4], K, nthreads=threads)
    t = time.perf_counter()
    for _ in range(args.steps):
        rd, rl = orc.rerank(base, q, cand, K, nthreads=threads)
    total = time.perf_counter() - t
    qps = sample * args.steps / total
    return _reference_line(args, RERANK_METRIC, qps, total, threads,
                           f"rerank_{args.nb}x128_nq{args.nq}_ncand{2 * K}_k{K}",
                           f"{sample} queries per step, query-parallel on {threads} threads",
                           distance_error_vs_fp64(base, q, rd, rl))


def _reference_line(args, metric, qps, total, threads, workload, sample, derr=None):
    return {
        "distance_error_vs_fp64": derr,
        "metric": metric, "impl": "reference", "value": round(qps, 1), "unit": "queries/s",
        "n_gpus": 0, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1e3 * total / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic SIFT-like (seeded Gaussian mixture, integer-valued), not SIFT1M",
        "config": {"workload": workload, "form": "reference CPU path (oracle port)"},
        "cpu_baseline": {"value": round(qps, 1), "unit": "queries/s", "cores": threads,
                         "kind": "port", "sample": sample},
        "e2e": {"value": round(qps, 1), "unit": "queries/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }


def run_reference_flat(args):
    """The oracle's IndexFlat search over all rows for a bounded query sample."""
    from oracle import oracle as orc

    threads = os.cpu_count() or 1
    base, queries = build_workload(args.nb, args.nq, args.dim)
    metric = 0 if args.metric == "l2" else 1
    sample = min(max(args.cpu_sample // 100, 1), args.nq)
    q = queries[:sample]
    if args.workload == "sq8":
        ref = orc.SQ8(args.dim, metric)
        ref.add(base)
        run = lambda qq: ref.search(qq, args.k, nthreads=threads)  # noqa: E731
    else:
        run = lambda qq: orc.flat_search(base, qq, args.k, metric=metric, nthreads=threads)  # noqa: E731
    for _ in range(max(args.warmup, 0)):
        run(q[:2])
    t = time.perf_counter()
    for _ in range(args.steps):
        rd, rl = run(q)
    total = time.perf_counter() - t
    qps = sample * args.steps / total
    return {
        "distance_error_vs_fp64": distance_error_vs_fp64(base, q, rd, rl, args.metric),
        "metric": SQ8_METRIC if args.workload == "sq8" else FLAT_METRIC, "impl": "reference",
        "value": round(qps, 1), "unit": "queries/s",
        "n_gpus": 0, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1e3 * total / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic SIFT-like (seeded Gaussian mixture, integer-valued), not SIFT1M",
        "config": {"workload": f"{args.workload}_{args.nb}x{args.dim}_{args.metric}_nq{args.nq}_k{args.k}",
                   "form": "reference CPU path (oracle port)"},
        "cpu_baseline": {"value": round(qps, 1), "unit": "queries/s", "cores": threads,
                         "kind": "port",
                         "sample": f"{sample} queries per step over all {args.nb} rows, "
                                   f"query-parallel on {threads} threads"},
        "e2e": {"value": round(qps, 1), "unit": "queries/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--form", default="fast", choices=["plain", "fast", "batched"])
    ap.add_argument("--nprobe", type=int, default=8)
    ap.add_argument("--lut", type=int, default=None,
                    help="ivfpq workload: fast-form scan variant (default: FP32 tables, two-kernel "
                         "scan where it pays; 2 = single-kernel; 6 = bank-rotated fixed-point tables "
                         "with per-candidate slots; 7 = two-kernel always)")
    ap.add_argument("--rerank", type=int, default=None,
                    help="shortlist depth (IVF-PQ default 256, flat default k * 4)")
    ap.add_argument("--nb", type=int, default=NB, help="base rows (profiling runs use fewer)")
    ap.add_argument("--nq", type=int, default=NQ, help="queries per step")
    ap.add_argument("--cpu-sample", type=int, default=10000)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--workload", default="ivfpq",
                    choices=["ivfpq", "flat", "sq8", "kmeans", "batch", "serve", "curve", "ivfflat",
                             "rerank"])
    ap.add_argument("--batch-nb", type=int, default=10_000_000)
    ap.add_argument("--serve-scale", type=float, default=1.0)
    ap.add_argument("--serve-requests", type=int, default=300)
    ap.add_argument("--serve-rates", type=float, nargs="+", default=[20.0, 80.0, 320.0, 1280.0, 5120.0])
    ap.add_argument("--serve-budget-gb", type=int, default=24)
    ap.add_argument("--batch-nq", type=int, default=20_000)
    ap.add_argument("--km-n", type=int, default=1_000_000)
    ap.add_argument("--km-k", type=int, default=16384)
    ap.add_argument("--km-iter", type=int, default=25)
    ap.add_argument("--rerank-factor", type=int, default=2, help="sq8 workload: shortlist k * factor")
    ap.add_argument("--k", type=int, default=K, help="flat workload: results per query")
    ap.add_argument("--metric", default="l2", choices=["l2", "ip"], help="flat workload metric")
    ap.add_argument("--dim", type=int, default=D, help="flat/sq8 workloads: row length")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.rerank is None:
        args.rerank = 224 if args.workload == "ivfpq" else 4 * args.k
    world = _env_int("WORLD_SIZE", 1)
    rank = _env_int("RANK", 0)

    if args.impl == "reference":
        if rank == 0:
            if args.workload in ("flat", "sq8"):
                ref = run_reference_flat(args)
            elif args.workload == "ivfflat":
                ref = run_reference_ivfflat(args)
            elif args.workload == "rerank":
                ref = run_reference_rerank(args)
            else:
                ref = run_reference(args)
            print(json.dumps(ref), flush=True)
        return

    if world > 1:
        import torch

        torch.distributed.init_process_group("nccl")
    if args.workload == "kmeans":
        out = run_kmeans(args, rank, world)
    elif args.workload == "batch":
        out = run_batch(args, rank, world)
    elif args.workload == "serve":
        out = run_serve(args, rank, world)
    elif args.workload == "curve":
        out = run_curve(args, rank, world)
    elif args.workload in ("flat", "sq8"):
        out = run_flat(args, rank, world)
    elif args.workload == "ivfflat":
        out = run_ivfflat(args, rank, world)
    elif args.workload == "rerank":
        out = run_rerank(args, rank, world)
    else:
        out = run_gpu(args, rank, world)
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        import torch

        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
