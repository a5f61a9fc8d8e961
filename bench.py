#!/usr/bin/env python3
"""Benchmark: bulk stream-mode SDBF digest generation on GB300.

Workload (the configuration the headline "digest input GB/s" is quoted on):
4096 files with sizes log-uniform over 4 KiB..64 MiB (seeded), content a
per-file mixture of 50% uniform-random regions, 25% low-entropy runs and 25%
order-1 Markov text, digested in stream mode (sdhash -b 0).  Synthetic,
seeded (sdhash_gb300/csrc/synth.c); ~26 GiB, larger than L2 by 200x, so no
L2 flush is needed between steps.

One step = digest every file of the rank's shard once.
  value -- device-resident: inputs already in HBM, digests left in HBM
           (sdbfg_digest_batch_device), CUDA events on the launch stream.
  e2e   -- through the public C ABI with HOST buffers (sdbfg_digest_batch):
           host->device copy of the inputs from pinned memory, generation,
           device->host copy of the packed filters and per-file results into
           the caller's host buffers, every step (python_api_value: the same
           batch once through Context.digest_packed, Digest objects built).

--impl reference times the reference's CPU implementation of the path (the
oracle port of sdhash's generation, all host threads) on the same workload.

Multi-GPU (torchrun, --gpus N): files are size-balanced across ranks with no
data-path collective (weak scaling of the total bytes); timings are max over
ranks.
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

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "digest input GB/s"
UNIT = "GB/s"
CONFIG_BASE = {"workload": "bulk stream-mode digest generation", "files": 4096, "sizes": "log-uniform 4 KiB..64 MiB",
               "content": "mixture: 50% random / 25% low-entropy runs / 25% order-1 Markov text",
               "mode": "stream (-b 0)", "l2": "inputs larger than L2 (no flush needed)"}


KERNELS = ("k_stream_ranks", "k_stream_tiles", "k_stream_fails", "k_stream_fix_list", "k_stream_check", "k_stream_fix",
           "k_stream_commit", "k_pack_filters", "k_scan_offsets")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--nfiles", type=int, default=4096)
    ap.add_argument("--seed", type=int, default=2)
    ap.add_argument("--max-bytes", type=int, default=64 << 20, help="largest file")
    ap.add_argument("--cpu-sample-gib", type=float, default=3.0)
    ap.add_argument("--plain-gib", type=float, default=2.0,
                    help="stream: sample timed through the plain per-file GPU path (0: off)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--workload", default="stream", choices=["stream", "allpairs", "image", "serve", "load", "index",
                                                         "index-build"],
                    help="stream: bulk digest generation (headline); allpairs: batched uneven all-pairs compare; "
                         "image: block-mode disk image + query fragments compared against it; serve: continuous-batching "
                         "server under Poisson load; load: bulk SDBF text load into a resident set; index: "
                         "block-mode index search; index-build: sdhash --index for one 640 MiB group")
    ap.add_argument("--image-gib", type=int, default=16, help="image: disk image size (GiB, multiple of 128 MiB)")
    ap.add_argument("--queries", type=int, default=100000, help="image: query fragments")
    ap.add_argument("--ref-filters", type=int, default=244 * 8192, help="serve: block filters in the reference set")
    ap.add_argument("--rate", type=float, default=5000.0, help="serve: offered Poisson load (queries/s)")
    ap.add_argument("--serve-queries", type=int, default=1500, help="serve: queries per load run")
    ap.add_argument("--search-gib", type=float, default=4.0, help="index: input size (GiB, 128 MiB segments)")
    ap.add_argument("--indexes", type=int, default=8, help="index: 64 MiB index filters searched")
    ap.add_argument("--digests", type=int, default=20000, help="allpairs: digests in the set")
    ap.add_argument("--max-filters", type=int, default=2000, help="allpairs: largest digest (filters)")
    ap.add_argument("--plain-pairs", type=int, default=400, help="allpairs: pairs timed one call each")
    ap.add_argument("--cpu-pairs", type=int, default=256, help="allpairs: pairs timed on the host (oracle)")
    ap.add_argument("--quick", action="store_true",
                    help="index-build: skip the comparison runs (sequential commit, shared pool, block group)")
    ap.add_argument("--phases", action="store_true",
                    help="allpairs: one more run with the tensor-core kernel's per-phase cycle counters")
    ap.add_argument("--variant", type=int, default=-1,
                    help="comparison kernel variant (0-4 CUDA cores, 5 tensor cores); -1: autotune")
    return ap.parse_args()


def dist_setup(n):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(world, v: float) -> float:
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def allsum(world, v: float) -> float:
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def make_workload(args, rank, world, pinned: bool):
    """This rank's files, packed 16-byte aligned into one (pinned) host buffer."""
    from sdhash_gb300 import shard, synth
    sizes_all = synth.log_uniform_sizes(args.seed, args.nfiles, 4096, args.max_bytes)
    mine = shard.shard_sizes(sizes_all, world)[rank]
    sizes = sizes_all[mine]
    offs, total = synth.packed_layout(sizes)
    if pinned:
        import torch
        buf = torch.empty(max(16, total), dtype=torch.uint8, pin_memory=True)
        data = buf.numpy()
    else:
        buf = None
        data = np.empty(max(16, total), dtype=np.uint8)
    # generate file by file with the global file index as the stream id, so a
    # file's bytes do not depend on the sharding
    import ctypes as C
    L = synth.lib()
    from concurrent.futures import ThreadPoolExecutor
    with ThreadPoolExecutor(max_workers=min(64, os.cpu_count() or 1)) as ex:
        list(ex.map(lambda k: L.synth_fill_mixture(args.seed, int(mine[k]), data.ctypes.data + int(offs[k]),
                                                   int(sizes[k])), range(len(mine))))
    return buf, data, offs, sizes, sizes_all


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(r[1]) for r in self.rows if num(r[1]) is not None]
        mx = [num(r[2]) for r in self.rows if num(r[2]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def compare_roofline(pairs_per_s: float, variant: int, sm_mhz=None):
    """Roofline of the comparison kernel.  The tensor-core variant counts
    popcount(a & b) of two 2,048-bit filters as an e4m3 dot product of length
    2,048 (4,096 fp8 FLOPs per filter pair) against the fp8 dense rate, taken
    as twice the measured bf16 rate (MEASURED_PEAKS.json has no fp8 figure;
    nominal dense fp8 is 4.5 PFLOP/s).  The CUDA-core variants are integer
    issue bound: 64 AND + 64 POPC + 63 adds per filter pair against 128
    integer lanes per SM per clock."""
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            pk = json.load(f)
        bf16, src = float(pk["bf16_tflops"]), "measured"
    except (OSError, KeyError, ValueError):
        bf16, src = 1900.0, "fallback"
    if variant == 5:
        peak = 2 * bf16
        ach = pairs_per_s * 4096 / 1e12
        return {"bound": "tensor", "kernel": "k_matrix_tc", "achieved": ach, "peak": peak, "unit": "TFLOP/s",
                "frac": ach / peak, "traffic": None,
                "work_per_filter_pair": "4096 fp8 FLOPs (2048-bit AND-popcount as an e4m3 0/1 dot product)",
                "peak_source": f"2 x {src} bf16 burst (MEASURED_PEAKS.json bf16_tflops; fp8 dense = 2 x bf16)",
                "mma_bound_filter_pairs_per_s": peak * 1e12 / 4096}
    mhz = sm_mhz or 2070.0
    peak = 152 * 128 * mhz * 1e6 / 1e12
    ach = pairs_per_s * 191 / 1e12
    return {"bound": "int", "kernel": "k_matrix", "achieved": ach, "peak": peak, "unit": "Tops/s", "frac": ach / peak,
            "traffic": None, "work_per_filter_pair": "191 integer lane ops (64 AND, 64 POPC, 63 adds)",
            "peak_source": f"152 SMs x 128 integer lanes x {mhz:.0f} MHz"}


def profiled_value(kernel: str, key: str):
    """A per-input-byte figure of `kernel` from its committed ncu summary."""
    path = os.path.join(REPO, "profiles", f"{kernel}_ncu.md")
    try:
        for line in open(path):
            if line.startswith(key + ":"):
                return float(line.split(":", 1)[1].strip())
    except OSError:
        pass
    return None


def profiled_traffic(kernel: str):
    """dram bytes per input byte of `kernel` from the committed ncu summary."""
    return profiled_value(kernel, "dram_bytes_per_input_byte")


def sample_files(sizes, gib: float, seed: int):
    """Indices of files drawn at random until they hold `gib` GiB."""
    rng = np.random.default_rng(seed)
    target = int(gib * (1 << 30))
    pick, tot = [], 0
    for i in rng.permutation(len(sizes)):
        if tot >= target:
            break
        pick.append(int(i))
        tot += int(sizes[i])
    return pick, tot


def cpu_baseline(args, data, offs, sizes, nthreads=None, seed=7, keep=False):
    """The oracle port of sdhash's generation (file-parallel on all host
    threads, as sdhash -p N) on a bounded random sample of the workload.
    keep=True also returns the sample's indices and oracle digests (the
    parity check of the GPU output reads them after the timing)."""
    from oracle import Oracle
    O = Oracle()
    pick, tot = sample_files(sizes, args.cpu_sample_gib, seed)
    nt = nthreads or (os.cpu_count() or 1)
    bufs = [data[int(offs[i]):int(offs[i]) + int(sizes[i])] for i in pick]
    t0 = time.perf_counter()
    res = O.digest_many(bufs, 0, nt)
    dt = time.perf_counter() - t0
    assert all(r is not None or int(sizes[i]) < 512 for r, i in zip(res, pick))
    info = {"value": tot / dt / 1e9, "unit": UNIT, "cores": nt, "kind": "port",
            "sample": f"{len(pick)} files, {tot / (1 << 30):.2f} GiB drawn at random from the same workload",
            "seconds": round(dt, 3)}
    if keep:
        return info, pick, res
    del res
    return info


def parity_vs_oracle(pick, oracle_res, sizes, dev_res, out_host):
    """Files of the oracle sample whose GPU digest (filters, bf_count,
    last_count of the timed step's device output) differs from the oracle's."""
    bad, nbytes = [], 0
    for i, od in zip(pick, oracle_res):
        r = dev_res[i]
        nbytes += int(sizes[i])
        if od is None:
            if r.status == 0:
                bad.append(i)
            continue
        got = out_host[r.filter_offset * 256:(r.filter_offset + r.bf_count) * 256].tobytes()
        if r.status != 0 or (r.bf_count, r.last_count) != (od.bf_count, od.last_count) or got != od.filters():
            bad.append(i)
    return bad, nbytes


def parity_host_vs_device(res_dev, out_dev_host, res_host, out_host, n):
    """Files whose host-buffer C-ABI result differs from the device-resident one."""
    bad = []
    for i in range(n):
        a, b = res_dev[i], res_host[i]
        if (a.status, a.bf_count, a.last_count) != (b.status, b.bf_count, b.last_count):
            bad.append(i)
            continue
        if a.status == 0:
            x = out_dev_host[a.filter_offset * 256:(a.filter_offset + a.bf_count) * 256]
            y = out_host[b.filter_offset * 256:(b.filter_offset + b.bf_count) * 256]
            if not np.array_equal(x, y):
                bad.append(i)
    return bad


def plain_per_call(ctx, dev, offs, sizes, gib: float, seed: int = 11):
    """The plain per-file GPU path: one sdbfg_digest_batch_device call per
    file (as the reference's worker threads build one sdbf per file,
    sdhash_threads.cc:152-186), on a random sample of the workload with the
    inputs already in HBM.  Returns the sample's GB/s and description."""
    import torch
    pick, tot = sample_files(sizes, gib, seed)
    cap = max(ctx.capacity([int(sizes[i])], 0) for i in pick)
    out = torch.empty(max(1, cap) * 256, dtype=torch.uint8, device="cuda")
    base = dev.data_ptr()

    def one(i):
        return ctx.digest_device(base + int(offs[i]), [0], [int(sizes[i])], 0, out.data_ptr(), cap)

    for i in pick[:4]:
        one(i)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in pick:
        one(i)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    return {"value": tot / dt / 1e9, "unit": UNIT, "calls": len(pick), "seconds": round(dt, 3),
            "sample": f"{len(pick)} files, {tot / (1 << 30):.2f} GiB drawn at random from the same workload, "
                      "one sdbfg_digest_batch_device call per file (inputs in HBM)"}


def run_reference(args):
    rank, world, local = dist_setup(args.gpus)
    if rank != 0:
        return 0
    _, data, offs, sizes, _ = make_workload(args, 0, 1, pinned=False)
    nt = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_baseline(args, data, offs, sizes, nt, seed=1)
    vals, secs = [], 0.0
    base = None
    for k in range(args.steps):
        cb = cpu_baseline(args, data, offs, sizes, nt, seed=100 + k)
        vals.append(cb["value"])
        secs += cb["seconds"]
        base = cb
    v = float(np.mean(vals))
    base["value"] = v
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * secs / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
            "config": dict(CONFIG_BASE, sample_per_step=base["sample"]), "cpu_baseline": base,
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ----------------------------------------------------------------- allpairs
AP_METRIC = "filter-pair compares/s (batched all-pairs)"
AP_UNIT = "filter pairs/s"


def allpairs_digests(args, ctx):
    """20,000 stream digests with filter counts about round(exp(U(0, ln 2000))).

    Each digest is generated on the GPU from its own mixture content sized
    n x 12 KiB (mixture content yields one stream filter per ~12.3 KiB), so
    filters and element counts come from generation.  Content is produced and
    digested in groups to bound host memory."""
    from sdhash_gb300 import synth
    rng = np.random.default_rng(args.seed + 1000)
    target = np.clip(np.rint(np.exp(rng.uniform(0.0, np.log(args.max_filters), args.digests))), 1,
                     args.max_filters).astype(np.int64)
    sizes = (target * (12 << 10)).astype(np.uint64)
    names = [f"d{i:05d}" for i in range(args.digests)]
    digs = []
    step = 1000
    for g0 in range(0, args.digests, step):
        sz = sizes[g0:g0 + step]
        data, offs, lens = synth.fill_many(args.seed + 1001 + g0, "mixture", sz)
        digs += ctx.digest_packed(data, offs, lens, 0, names=names[g0:g0 + step])
        del data
    counts = np.array([d.bf_count for d in digs], dtype=np.int64)
    return digs, counts, int(sizes.sum())


TC_PHASES = ("compose", "fill", "fetch_wait", "stage_wait", "widen", "issue", "producer_step", "acc_wait", "score",
             "mark", "walk", "fold", "consumer_step", "step_barrier", "tmem_ld")


def tc_phases(ctx, run):
    """SM cycles per tile of each phase of the tensor-core kernel (one CTA's
    clock, summed over CTAs, divided by the tiles counted) for one more run."""
    import torch
    ctx.profile(True)
    run()
    torch.cuda.synchronize()
    tiles = ctx.kernel_time("k_matrix_tc.tiles")[0] or 1.0
    out = {k: round(ctx.kernel_time("k_matrix_tc." + k)[0] / tiles) for k in TC_PHASES}
    out["tiles"] = int(tiles)
    ctx.profile(False)
    return out


def main_allpairs(args):
    import torch
    import sdhash_gb300 as g
    torch.cuda.set_device(0)
    ctx = g.Context(0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    t0 = time.perf_counter()
    digs, counts, content_bytes = allpairs_digests(args, ctx)
    t_build = time.perf_counter() - t0
    n = len(digs)
    npairs = n * (n - 1) // 2
    dev = ctx.upload(digs)
    fpairs = ctx.filter_pairs(dev)
    out = torch.empty(npairs, dtype=torch.int32, device="cuda")
    # autotuner on a sample of the job's units (also the warm-up)
    t0 = time.perf_counter()
    if args.variant < 0:
        variant, unit_work, tuned_rate = ctx.autotune_compare(dev, sample_pairs=1 << 35)
    else:
        ctx.set_compare_tuning(args.variant, 1 << 22, True)
        (variant, unit_work), tuned_rate = ctx.compare_tuning(), None
    t_tune = time.perf_counter() - t0
    for _ in range(args.warmup):  # a capture-and-replay run of the full job
        ctx.compare_all_device(dev, out.data_ptr())
    torch.cuda.synchronize()
    clocks = ClockSampler(0)
    clocks.start()
    l0 = ctx.launch_count
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        ctx.compare_all_device(dev, out.data_ptr())
    e1.record(stream)
    torch.cuda.synchronize()
    clocks.stop()
    launches = ctx.launch_count - l0
    ms = e0.elapsed_time(e1) / args.steps
    value = fpairs / (ms / 1e3)
    scores = out.cpu().numpy()

    # plain per-call GPU path: one sdbf::compare-style call (one launch, one
    # pair, result read back) per pair, on random pairs of the same set
    rng = np.random.default_rng(5)
    pi = rng.integers(0, n, 4 * args.plain_pairs)
    pj = rng.integers(0, n, 4 * args.plain_pairs)
    keep = pi != pj
    pi, pj = np.minimum(pi, pj)[keep][: args.plain_pairs], np.maximum(pi, pj)[keep][: args.plain_pairs]
    ctx.score_pairs(dev, dev, pi[:4], pj[:4])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    plain_scores = [int(ctx.score_pairs(dev, dev, [int(a)], [int(b)])[0]) for a, b in zip(pi, pj)]
    t_plain = time.perf_counter() - t0
    plain_work = int(sum(int(counts[a]) * int(counts[b]) for a, b in zip(pi, pj)))
    idx = pi * (2 * n - pi - 1) // 2 + (pj - pi - 1)
    assert plain_scores == [int(x) for x in scores[idx]], "per-call and batched scores differ"
    plain_rate = plain_work / t_plain

    # CPU reference path (oracle port, all host threads) on random pairs
    from oracle import Oracle
    O = Oracle()
    ci, cj = pi[: args.cpu_pairs], pj[: args.cpu_pairs]
    used = sorted(set(ci.tolist()) | set(cj.tolist()))
    loc = {d: k for k, d in enumerate(used)}
    ods = [O.parse(digs[d].to_string()) for d in used]
    nt = os.cpu_count() or 1
    t0 = time.perf_counter()
    cpu_scores = O.score_pairs(ods, [loc[int(a)] for a in ci], [loc[int(b)] for b in cj], nt)
    t_cpu = time.perf_counter() - t0
    assert [int(x) for x in cpu_scores] == [int(x) for x in scores[idx[: len(ci)]]], "oracle and GPU scores differ"
    cpu_work = int(sum(int(counts[a]) * int(counts[b]) for a, b in zip(ci, cj)))

    e2e, e2e_bad = None, None
    if not args.no_e2e:
        # public host API: upload the set (H2D), all pairs, scores back (D2H)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s2 = ctx.upload(digs)
        host_scores = ctx.compare_all(s2)
        s2.close()
        t_e2e = time.perf_counter() - t0
        assert np.array_equal(host_scores, scores)
        e2e = {"value": fpairs / t_e2e, "unit": AP_UNIT, "h2d_bytes_per_step": int(counts.sum()) * 256,
               "d2h_bytes_per_step": int(npairs) * 4, "ms_per_step": t_e2e * 1e3}
    line = {"metric": AP_METRIC, "value": value, "unit": AP_UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u32 (2048-bit Bloom filters, integer scores)", "data": "synthetic",
            "config": {"workload": "batched uneven all-pairs compare", "digests": n, "pairs": npairs,
                       "filters_per_digest": f"log-uniform 1..{args.max_filters}", "filters": int(counts.sum()),
                       "filter_pairs_per_step": fpairs, "threshold": 1,
                       "filter_source": f"stream digests of {content_bytes / 1e9:.1f} GB mixture content "
                                        "(n x 12 KiB per digest) generated on the GPU",
                       "variant": variant, "unit_work": unit_work, "autotune_s": round(t_tune, 2),
                       "autotune_sample_rate": tuned_rate, "build_s": round(t_build, 1),
                       "l2": "filters 5x larger than L2"},
            "gpu_launches": launches, "clocks": clocks.summary(),
            "roofline": compare_roofline(value, variant, clocks.summary().get("sm_mhz")),
            "plain_per_call": {"value": plain_rate, "unit": AP_UNIT, "pairs": len(pi), "filter_pairs": plain_work,
                               "seconds": round(t_plain, 3),
                               "path": "sdbfg_score_pairs with one pair per call (one launch + sync each)"},
            "batched_over_plain": value / plain_rate,
            "e2e": e2e,
            "cpu_baseline": {"value": cpu_work / t_cpu, "unit": AP_UNIT, "cores": nt, "kind": "port",
                             "sample": f"{len(ci)} random pairs ({cpu_work} filter pairs)",
                             "seconds": round(t_cpu, 3)},
            "scores_ge_1": int((scores >= 1).sum())}
    if args.phases and variant == 5:
        line["tc_phase_cycles_per_tile"] = tc_phases(ctx, lambda: ctx.compare_all_device(dev, out.data_ptr()))
    print(json.dumps(line), flush=True)
    return 0


# -------------------------------------------------------------------- image
IM_METRIC = "query-vs-image filter-pair compares/s"
SEG = 128 << 20  # sdhash -b segments files above 128 MiB into 128 MiB digests


def digests_from_device(g, res, names, lens, dd, out_dev, counts_dev):
    filt = out_dev.cpu().numpy()
    cnt = counts_dev.cpu().numpy() if counts_dev is not None else None
    ds = []
    for i in range(len(names)):
        r = res[i]
        if r.status != 0:
            ds.append(None)
            continue
        o, k = int(r.filter_offset), int(r.bf_count)
        f = filt[o * 256:(o + k) * 256].copy()
        if dd:
            ds.append(g.Digest(names[i], int(lens[i]), k, 0, 192, dd, f, cnt[o:o + k].copy()))
        else:
            ds.append(g.Digest(names[i], int(lens[i]), k, int(r.last_count), 160, 0, f, None))
    return ds


def timed(stream, fn, reps=1):
    import torch
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(reps):
        r = fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return r, e0.elapsed_time(e1) / reps


def main_image(args):
    """Block-mode image digest (-b 16, 128 MiB segments) and query-fragment
    digests (-b 16, 1..64 filters each), then every query against every
    image segment."""
    import torch
    import sdhash_gb300 as g
    from sdhash_gb300 import synth
    torch.cuda.set_device(0)
    ctx = g.Context(0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    dd = 16384
    nseg = args.image_gib * (1 << 30) // SEG
    t0 = time.perf_counter()
    image, ioffs, ilens = synth.fill_many(args.seed + 2000, "mixture", np.full(nseg, SEG, dtype=np.uint64))
    t_synth = time.perf_counter() - t0
    inames = [f"image.{k * SEG // (1 << 20):04d}M" for k in range(nseg)]
    # ---- block-mode image digest, device resident
    dimg = torch.from_numpy(image).cuda()
    cap = ctx.capacity(ilens, dd)
    iout = torch.empty(cap * 256, dtype=torch.uint8, device="cuda")
    icnt = torch.empty(cap, dtype=torch.uint16, device="cuda")
    run = lambda: ctx.digest_device(dimg.data_ptr(), ioffs, ilens, dd, iout.data_ptr(), cap, icnt.data_ptr())
    for _ in range(args.warmup):
        run()
    ires, img_ms = timed(stream, run)
    idigs = digests_from_device(g, ires, inames, ilens, dd, iout, icnt)
    del dimg
    # ---- query fragments: 60% cut from the image, 40% fresh random data
    rng = np.random.default_rng(args.seed + 2001)
    qsz = synth.log_uniform_sizes(args.seed + 2002, args.queries, 4096, 1 << 20)
    cut = rng.random(args.queries) < 0.6
    qoffs, qtot = synth.packed_layout(qsz)
    qdata = np.empty(max(16, qtot), dtype=np.uint8)
    src = rng.integers(0, len(image) - qsz.astype(np.int64))
    fresh = np.nonzero(~cut)[0]
    fr_data, fr_offs, _ = synth.fill_many(args.seed + 2003, "random", qsz[fresh])
    for k, i in enumerate(fresh):
        qdata[int(qoffs[i]):int(qoffs[i]) + int(qsz[i])] = fr_data[int(fr_offs[k]):int(fr_offs[k]) + int(qsz[i])]
    del fr_data
    for i in np.nonzero(cut)[0]:
        qdata[int(qoffs[i]):int(qoffs[i]) + int(qsz[i])] = image[int(src[i]):int(src[i]) + int(qsz[i])]
    qnames = [f"q{i:06d}" for i in range(args.queries)]
    dq = torch.from_numpy(qdata).cuda()
    qcap = ctx.capacity(qsz, dd)
    qout = torch.empty(qcap * 256, dtype=torch.uint8, device="cuda")
    qcnt = torch.empty(qcap, dtype=torch.uint16, device="cuda")
    runq = lambda: ctx.digest_device(dq.data_ptr(), qoffs, qsz, dd, qout.data_ptr(), qcap, qcnt.data_ptr())
    for _ in range(args.warmup):
        runq()
    qres, q_ms = timed(stream, runq)
    qdigs = digests_from_device(g, qres, qnames, qsz, dd, qout, qcnt)
    del dq
    # ---- parity spot checks against the oracle (sampled)
    from oracle import Oracle
    O = Oracle()
    chk = [0, nseg - 1]
    refs = O.digest_many([image[int(ioffs[k]):int(ioffs[k]) + SEG] for k in chk], dd, len(chk),
                         names=[inames[k] for k in chk])
    for k, ref in zip(chk, refs):
        assert ref.to_string() == idigs[k].to_string(), inames[k]
    for i in rng.choice(args.queries, 24, replace=False):
        ref = O.digest(qnames[i], qdata[int(qoffs[i]):int(qoffs[i]) + int(qsz[i])].tobytes(), dd)
        assert ref.to_string() == qdigs[i].to_string(), qnames[i]
    # ---- comparison: every query x every segment
    qset, iset = ctx.upload(qdigs), ctx.upload(idigs)
    fpairs = ctx.filter_pairs(qset, iset)
    scores_dev = torch.empty(args.queries * nseg, dtype=torch.int32, device="cuda")
    t0 = time.perf_counter()
    if args.variant < 0:
        variant, unit_work, tuned = ctx.autotune_compare(qset, iset, sample_pairs=1 << 33)
    else:
        ctx.set_compare_tuning(args.variant, 1 << 22, True)
        variant, unit_work = ctx.compare_tuning()
    t_tune = time.perf_counter() - t0
    runc = lambda: ctx.compare_to_device(qset, iset, scores_dev.data_ptr())
    for _ in range(max(1, args.warmup)):
        runc()
    clocks = ClockSampler(0)
    clocks.start()
    l0 = ctx.launch_count
    _, cmp_ms = timed(stream, runc, args.steps)
    launches = ctx.launch_count - l0
    clocks.stop()
    scores = scores_dev.cpu().numpy().reshape(args.queries, nseg)
    best = scores.argmax(1)
    seg_of = (src // SEG).astype(np.int64)
    seg_end = ((src + qsz.astype(np.int64) - 1) // SEG).astype(np.int64)
    found = cut & ((best == seg_of) | (best == seg_end)) & (scores.max(1) >= 1)
    # e2e: host query buffer -> digests -> compare against the resident image set -> scores on the host
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    q2 = ctx.digest_packed(qdata, qoffs, qsz, dd, names=qnames)
    qs2 = ctx.upload(q2)
    host_scores = ctx.compare_to(qs2, iset)
    t_e2e = time.perf_counter() - t0
    assert np.array_equal(host_scores, scores)
    qs2.close()
    # plain per-call GPU path: one query per call against the resident image set
    pick = rng.choice(args.queries, min(200, args.queries), replace=False)
    ctx.compare_to(ctx.upload([qdigs[pick[0]]]), iset)
    t0 = time.perf_counter()
    for i in pick:
        one = ctx.upload([qdigs[i]])
        r = ctx.compare_to(one, iset)
        one.close()
        assert np.array_equal(r[0], scores[i])
    t_plain = time.perf_counter() - t0
    plain_work = int(sum(qdigs[i].bf_count for i in pick)) * sum(d.bf_count for d in idigs)
    # CPU reference path on a sample (oracle, all host threads)
    segs = list(range(0, nseg, max(1, nseg // 8)))
    cq = pick[:16]
    oq = [O.parse(qdigs[i].to_string()) for i in cq]
    oi = [O.parse(idigs[k].to_string()) for k in segs]
    nt = os.cpu_count() or 1
    t0 = time.perf_counter()
    cpu = O.score_cross_matrix(oq, oi, nt)
    t_cpu = time.perf_counter() - t0
    assert np.array_equal(cpu, scores[np.ix_(cq, segs)])
    cpu_work = int(sum(qdigs[i].bf_count for i in cq)) * sum(idigs[k].bf_count for k in segs)
    value = fpairs / (cmp_ms / 1e3)
    line = {"metric": IM_METRIC, "value": value, "unit": AP_UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": cmp_ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u32 (2048-bit Bloom filters, integer scores)", "data": "synthetic",
            "config": {"workload": "block-mode image vs query fragments", "image_bytes": int(ilens.sum()),
                       "image_segments": nseg, "dd_block_size": dd, "image_filters": sum(d.bf_count for d in idigs),
                       "queries": args.queries, "query_bytes": int(qsz.sum()),
                       "query_filters": sum(d.bf_count for d in qdigs), "query_sizes": "log-uniform 4 KiB..1 MiB",
                       "cut_from_image": int(cut.sum()), "filter_pairs_per_step": fpairs, "threshold": 1,
                       "variant": variant, "unit_work": unit_work, "autotune_s": round(t_tune, 2),
                       "synth_s": round(t_synth, 1)},
            "image_digest": {"value": int(ilens.sum()) / (img_ms / 1e3) / 1e9, "unit": "GB/s", "ms": img_ms,
                             "mode": "block (-b 16), device resident"},
            "query_digest": {"value": int(qsz.sum()) / (q_ms / 1e3) / 1e9, "unit": "GB/s", "ms": q_ms,
                             "mode": "block (-b 16), device resident"},
            "top_match": {"cut_queries_best_segment_found": int(found.sum()), "cut_queries": int(cut.sum()),
                          "queries_with_score_ge_1": int((scores.max(1) >= 1).sum())},
            "gpu_launches": launches, "clocks": clocks.summary(),
            "roofline": compare_roofline(value, variant, clocks.summary().get("sm_mhz")),
            "plain_per_call": {"value": plain_work / t_plain, "unit": AP_UNIT, "queries": len(pick),
                               "seconds": round(t_plain, 3),
                               "path": "one query per call: upload + compare_to + scores back"},
            "batched_over_plain": value / (plain_work / t_plain),
            "e2e": {"value": fpairs / t_e2e, "unit": AP_UNIT, "h2d_bytes_per_step": int(qsz.sum()),
                    "d2h_bytes_per_step": int(args.queries) * nseg * 4, "ms_per_step": t_e2e * 1e3,
                    "path": "host query bytes -> digests -> compare_to -> host scores"},
            "cpu_baseline": {"value": cpu_work / t_cpu, "unit": AP_UNIT, "cores": nt, "kind": "port",
                             "sample": f"{len(cq)} queries x {len(segs)} segments", "seconds": round(t_cpu, 3)}}
    print(json.dumps(line), flush=True)
    return 0


# -------------------------------------------------------------------- serve
SV_METRIC = "served queries/s (p50/p99 latency)"


def serve_reference_set(args, ctx, stream, pool_queries):
    """Reference set: a disk image of `ref_filters` 16 KiB blocks digested in
    block mode (-b 16) in 128 MiB segments, generated and digested a few GiB
    at a time.  Query digests: block mode, round(exp(U(0, ln 4096))) filters
    (n x 16 KiB of content), 60% cut from the image, 40% fresh random data."""
    import torch
    import sdhash_gb300 as g
    from sdhash_gb300 import synth
    dd = 16384
    total = args.ref_filters * dd
    seg_sizes = [SEG] * (total // SEG) + ([total % SEG] if total % SEG else [])
    names = [f"image.{k * SEG // (1 << 20):04d}M" for k in range(len(seg_sizes))]
    rng = np.random.default_rng(args.seed + 3000)
    qn = np.clip(np.rint(np.exp(rng.uniform(0.0, np.log(4096), pool_queries))), 1, 4096).astype(np.int64)
    qsz = (qn * dd).astype(np.uint64)  # one block-mode filter per 16 KiB block
    cut = rng.random(pool_queries) < 0.6
    qbufs = [None] * pool_queries
    digs = []
    per = 16  # segments per group (2 GiB)
    for g0 in range(0, len(seg_sizes), per):
        sz = np.array(seg_sizes[g0:g0 + per], dtype=np.uint64)
        data, offs, lens = synth.fill_many(args.seed + 3100 + g0, "mixture", sz)
        dimg = torch.from_numpy(data).cuda()
        cap = ctx.capacity(lens, dd)
        out = torch.empty(cap * 256, dtype=torch.uint8, device="cuda")
        cnt = torch.empty(cap, dtype=torch.uint16, device="cuda")
        res = ctx.digest_device(dimg.data_ptr(), offs, lens, dd, out.data_ptr(), cap, cnt.data_ptr())
        digs += digests_from_device(g, res, names[g0:g0 + per], lens, dd, out, cnt)
        for i in np.nonzero(cut)[0]:   # queries cut from this part of the image
            if qbufs[i] is None and rng.random() < per / len(seg_sizes) * 1.5 and int(qsz[i]) < len(data):
                o = int(rng.integers(0, len(data) - int(qsz[i])))
                qbufs[i] = data[o:o + int(qsz[i])].copy()
        del dimg, data
    for i in range(pool_queries):
        if qbufs[i] is None:
            qbufs[i] = synth.random_bytes(args.seed + 3002, i, int(qsz[i]))
    qnames = [f"q{i:05d}" for i in range(pool_queries)]
    queries = []
    for k in range(0, pool_queries, 64):
        queries += ctx.digest_buffers([b.tobytes() for b in qbufs[k:k + 64]], qnames[k:k + 64], dd)
    return digs, [q for q in queries if q is not None], cut


def poisson_run(srv, pool, rate, n, seed):
    """Submit n queries (cycling over the pool) at Poisson arrival times from
    a feeder thread; collect every result.  Returns (results, wall seconds)."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, n)
    order = rng.integers(0, len(pool), n)
    got = {}
    done = threading.Event()

    def feed():
        t0 = time.perf_counter()
        at = 0.0
        for k in range(n):
            at += gaps[k]
            while True:
                d = at - (time.perf_counter() - t0)
                if d <= 0:
                    break
                time.sleep(min(d, 0.0005) if d > 0.0002 else 0)
            srv.submit(pool[int(order[k])], k)
        done.set()

    th = threading.Thread(target=feed)
    t0 = time.perf_counter()
    th.start()
    while len(got) < n:
        for r, row in srv.poll(256, timeout_ms=20, scores=False):
            got[int(r.tag)] = (int(r.submit_ns), int(r.start_ns), int(r.done_ns), int(r.batch_queries),
                               int(r.best_score), int(r.matches))
    th.join()
    return got, order, time.perf_counter() - t0


def lat_summary(got):
    lat = np.array([(v[2] - v[0]) / 1e6 for v in got.values()])
    first = min(v[0] for v in got.values())
    last = max(v[2] for v in got.values())
    return {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "mean_ms": float(lat.mean()), "throughput_qps": len(got) / ((last - first) / 1e9),
            "mean_batch": float(np.mean([v[3] for v in got.values()]))}


def main_serve(args):
    import torch
    import sdhash_gb300 as g
    torch.cuda.set_device(0)
    ctx = g.Context(0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    t0 = time.perf_counter()
    refs, pool, cut = serve_reference_set(args, ctx, stream, 600)
    t_build = time.perf_counter() - t0
    tset = ctx.upload(refs)
    nt = len(refs)
    ref_filters = sum(d.bf_count for d in refs)
    qf = np.array([q.bf_count for q in pool])
    # solo scores of every pool query (one batched compare_to): the served rows must equal them
    poolset = ctx.upload(pool)
    if args.variant < 0:
        tuned = ctx.autotune_compare(poolset, tset, sample_pairs=1 << 33)
    else:
        ctx.set_compare_tuning(args.variant, 1 << 22, True)
        tuned = ctx.compare_tuning()
    solo = ctx.compare_to(poolset, tset)
    srv = g.Server(ctx, tset, slots=3, max_batch_queries=64, memory_budget=1 << 30, threshold=1)
    try:
        warm, _, _ = poisson_run(srv, pool, args.rate, 64, seed=1)
        clocks = ClockSampler(0)
        clocks.start()
        got_a, order_a, wall_a = poisson_run(srv, pool, args.rate, args.serve_queries, seed=2)
        clocks.stop()
        sa = lat_summary(got_a)
        rate_b = 0.7 * sa["throughput_qps"]
        got_b, order_b, wall_b = poisson_run(srv, pool, rate_b, max(200, args.serve_queries // 2), seed=3)
        sb = lat_summary(got_b)
        for k, v in list(got_a.items())[:200]:
            q = int(order_a[k])
            assert v[4] == solo[q].max() and v[5] == int((solo[q] >= 1).sum()), "served result differs"
        stats = srv.stats()
    finally:
        srv.close()
    # plain per-call GPU path: one query per call (upload, compare_to, scores back), one at a time;
    # its latency under the same Poisson load follows from the FIFO recurrence on measured service times
    rng = np.random.default_rng(4)
    pick = rng.integers(0, len(pool), 200)
    ctx.compare_to(ctx.upload([pool[0]]), tset)
    svc = []
    for q in pick:
        t1 = time.perf_counter()
        one = ctx.upload([pool[int(q)]])
        row = ctx.compare_to(one, tset)
        one.close()
        svc.append(time.perf_counter() - t1)
        assert np.array_equal(row[0], solo[int(q)])
    svc = np.array(svc)
    plain_qps = len(svc) / svc.sum()
    # plain per-pair path (sdbf::compare: one query digest against one
    # reference digest per call, scores read back each time)
    tcounts = np.array([d.bf_count for d in refs], dtype=np.int64)
    pq = rng.integers(0, len(pool), 400)
    pt = rng.integers(0, nt, 400)
    ctx.score_pairs(poolset, tset, pq[:4], pt[:4])
    t1 = time.perf_counter()
    pair_scores = [int(ctx.score_pairs(poolset, tset, [int(a)], [int(b)])[0]) for a, b in zip(pq, pt)]
    t_pairs = time.perf_counter() - t1
    assert pair_scores == [int(solo[a, b]) for a, b in zip(pq, pt)], "per-pair and served scores differ"
    pair_rate = float(sum(int(qf[a]) * int(tcounts[b]) for a, b in zip(pq, pt))) / t_pairs

    def fifo(rate, seed):
        r = np.random.default_rng(seed)
        arr = np.cumsum(r.exponential(1.0 / rate, len(svc)))
        fin, lat = 0.0, []
        for a, s_ in zip(arr, svc):
            fin = max(fin, a) + s_
            lat.append((fin - a) * 1e3)
        return {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99))}

    # CPU reference path (oracle, all host threads): a few queries against the whole reference set
    from oracle import Oracle
    O = Oracle()
    oref = [O.parse(d.to_string()) for d in refs]
    cq = [int(q) for q in pick[:3]]
    oq = [O.parse(pool[q].to_string()) for q in cq]
    ncpu = os.cpu_count() or 1
    t1 = time.perf_counter()
    cpu = O.score_cross_matrix(oq, oref, ncpu)
    t_cpu = time.perf_counter() - t1
    assert np.array_equal(cpu, solo[cq])
    served_fp = float(qf[order_a].sum()) * ref_filters / (
        (max(v[2] for v in got_a.values()) - min(v[0] for v in got_a.values())) / 1e9)
    line = {"metric": SV_METRIC, "value": sa["throughput_qps"], "unit": "queries/s", "n_gpus": 1,
            "steps": 1, "warmup": 1, "ms_per_step": wall_a * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u32 (2048-bit Bloom filters, integer scores)", "data": "synthetic",
            "config": {"workload": "serving: Poisson query digests vs resident block-mode reference set",
                       "ref_filters": ref_filters, "ref_segments": nt, "ref_bytes": ref_filters * 256,
                       "query_pool": len(pool), "query_filters": f"{int(qf.min())}..{int(qf.max())} "
                       f"(mean {qf.mean():.0f}, median {np.median(qf):.0f})", "offered_rate_qps": args.rate,
                       "queries": args.serve_queries, "slots": 3, "max_batch_queries": 64, "memory_budget": 1 << 30,
                       "threshold": 1, "build_s": round(t_build, 1), "tuning": list(tuned)},
            "latency_at_offered_rate": sa,
            "latency_at_70pct_of_capacity": dict(sb, offered_rate_qps=rate_b),
            "filter_pairs_per_s": served_fp,
            "served_over_plain_per_pair": served_fp / pair_rate,
            "server_stats": stats, "clocks": clocks.summary(), "gpu_launches": int(stats["launches"]),
            "roofline": compare_roofline(served_fp, tuned[0] if tuned else 5, clocks.summary().get("sm_mhz")),
            "plain_per_call": {"value": plain_qps, "unit": "queries/s", "queries": len(svc),
                               "mean_service_ms": float(svc.mean() * 1e3),
                               "latency_at_70pct_of_served_capacity": fifo(rate_b, 5),
                               "path": "one query per call: upload + compare_to + scores back"},
            "served_over_plain": sa["throughput_qps"] / plain_qps,
            "plain_per_pair": {"value": pair_rate, "unit": "filter pairs/s", "pairs": len(pq),
                               "seconds": round(t_pairs, 3),
                               "path": "sdbfg_score_pairs with one (query, reference digest) pair per call"},
            "e2e": {"value": sa["throughput_qps"], "unit": "queries/s",
                    "h2d_bytes_per_step": int(qf[order_a].sum()) * 256,
                    "d2h_bytes_per_step": args.serve_queries * nt * 4,
                    "path": "host query digests submitted -> score rows polled on the host"},
            "cpu_baseline": {"value": len(cq) / t_cpu, "unit": "queries/s", "cores": ncpu, "kind": "port",
                             "sample": f"{len(cq)} pool queries against all {nt} segments",
                             "seconds": round(t_cpu, 3)}}
    print(json.dumps(line), flush=True)
    return 0


IX_METRIC = "index-searched input GB/s (block mode)"


def main_index(args):
    """sdhash --index-search on the GPU (sdbfg_digest_batch_search): an image
    of 128 MiB segments (mixture content) digested in 16 KiB block mode with
    every fourth counted feature of each block looked up in `--indexes`
    64 MiB index filters.  The index filters are seeded random bits at
    12.5 % density, near the ~10 % of a 64 MiB index built from the 640 MB
    group sdhash --index writes (about 17 features per KiB x 5 bits).  value: device time of the two kernels (block digest
    with feature sampling + k_index_query, CUDA events); e2e: the whole call
    from pinned host memory (copies, digests and hit counts back);
    cpu_baseline: the oracle's restatement of the same search on a sample,
    all host threads."""
    import ctypes as C
    import torch
    import sdhash_gb300 as g
    from sdhash_gb300 import DigestResult, lib, synth, _ptr
    torch.cuda.set_device(0)
    ctx = g.Context(0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    dd = 16384
    nseg = max(1, int(args.search_gib * 1024) // 128)
    sizes = np.full(nseg, SEG, dtype=np.uint64)
    offs, total = synth.packed_layout(sizes)
    pinned = torch.empty(max(16, total), dtype=torch.uint8, pin_memory=True)
    data = pinned.numpy()
    synth.fill_many(args.seed + 5000, "mixture", sizes, out=data)
    bits = []
    for x in range(args.indexes):  # AND of three random bit strings: 12.5 % of the bits set
        r = [synth.random_bytes(args.seed + 5001, 3 * x + j, 64 << 20) for j in range(3)]
        bits.append(r[0] & r[1] & r[2])
    idx = [ctx.index_from_bits(b) for b in bits]
    n, nidx = nseg, len(idx)
    lens = np.ascontiguousarray(sizes, dtype=np.uint64)
    offs = np.ascontiguousarray(offs, dtype=np.uint64)
    cap = ctx.capacity(lens, dd)
    out_f = torch.empty(cap * 256, dtype=torch.uint8, pin_memory=True).numpy()
    out_c = np.zeros(cap, dtype=np.uint16)
    hits = np.zeros(cap * nidx, dtype=np.uint8)
    arr = (C.c_void_p * nidx)(*[x.h for x in idx])
    res = (DigestResult * n)()

    def call(with_index=True):
        if with_index:
            rc = lib().sdbfg_digest_batch_search(ctx.h, data.ctypes.data, _ptr(offs), _ptr(lens), n, dd,
                                                 out_f.ctypes.data, cap, out_c.ctypes.data, res, arr, nidx,
                                                 hits.ctypes.data)
        else:
            rc = lib().sdbfg_digest_batch(ctx.h, data.ctypes.data, _ptr(offs), _ptr(lens), n, dd, out_f.ctypes.data,
                                          cap, out_c.ctypes.data, res)
        ctx._check(rc)

    for _ in range(max(3, args.warmup)):
        call()
    torch.cuda.synchronize()
    clocks = ClockSampler(0)
    clocks.start()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        call()
    torch.cuda.synchronize()
    wall = (time.perf_counter() - t0) / args.steps
    clocks.stop()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        call(False)
    wall_plain = (time.perf_counter() - t0) / args.steps
    ctx.profile(True)
    l0 = ctx.launch_count
    for _ in range(args.steps):
        call()
    kd_ms, kd_n = ctx.kernel_time("k_block_digest")
    kq_ms, kq_n = ctx.kernel_time("k_index_query")
    launches = (ctx.launch_count - l0) // args.steps
    ctx.profile(False)
    dev_ms = (kd_ms + kq_ms) / args.steps
    nprobe_hits = int((hits > 4).sum())
    # parity and CPU baseline: the oracle on a sample of segments
    from oracle import Oracle
    O = Oracle()
    ncpu = os.cpu_count() or 1
    ks = list(range(0, n, max(1, n // 4)))[:4]
    sample = [data[int(offs[k]):int(offs[k]) + int(lens[k])] for k in ks]
    t1 = time.perf_counter()
    want = O.index_search(sample, dd, bits, ncpu)
    t_cpu = time.perf_counter() - t1
    for k, w in zip(ks, want):
        o = int(res[k].filter_offset)
        got = hits[o * nidx:(o + int(res[k].bf_count)) * nidx].reshape(-1, nidx)
        assert np.array_equal(got, w), "index-search hits differ from the oracle"
    hbm, src = peaks()
    alg = total  # each input byte read once by the block kernel
    line = {"metric": IX_METRIC, "value": total / (dev_ms / 1e3) / 1e9, "unit": "GB/s", "n_gpus": 1,
            "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": dev_ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
            "config": {"workload": "block-mode index search (sdhash --index-search)", "input_bytes": int(total),
                       "segments": n, "block": dd, "indexes": nidx, "index_bytes": 64 << 20,
                       "index_content": "seeded random bits at 12.5% density", "blocks": int(cap),
                       "l2": "inputs and indexes larger than L2 (no flush needed)"},
            "gpu_launches": int(launches), "clocks": clocks.summary(),
            "kernel_ms_per_step": {"k_block_digest": kd_ms / args.steps, "k_index_query": kq_ms / args.steps},
            "lookups_per_step": int(cap) * 48 * nidx,
            "blocks_with_hits_gt4": nprobe_hits,
            "roofline": {"bound": "hbm", "kernel": "k_block_digest", "achieved": alg / (kd_ms / args.steps / 1e3) / 1e9,
                         "peak": hbm, "unit": "GB/s", "frac": alg / (kd_ms / args.steps / 1e3) / 1e9 / hbm,
                         "traffic": None,
                         "peak_source": f"{src} hbm_gbs (MEASURED_PEAKS.json)", "algorithmic_bytes_per_step": alg},
            "plain_block_digest_e2e": {"value": total / wall_plain / 1e9, "unit": "GB/s",
                                       "path": "sdbfg_digest_batch, same input, no index"},
            "e2e": {"value": total / wall / 1e9, "unit": "GB/s", "h2d_bytes_per_step": int(total),
                    "d2h_bytes_per_step": int(cap) * (256 + 2 + nidx), "ms_per_step": wall * 1e3,
                    "path": "sdbfg_digest_batch_search from pinned host memory"},
            "cpu_baseline": {"value": sum(int(lens[k]) for k in ks) / t_cpu / 1e9, "unit": "GB/s", "cores": ncpu,
                             "kind": "port", "sample": f"{len(ks)} of {n} segments searched by the oracle",
                             "seconds": round(t_cpu, 3)}}
    print(json.dumps(line), flush=True)
    return 0


IB_METRIC = "index build input GB/s"
IB_KERNELS = ("k_stream_tiles", "k_stream_check", "k_stream_fix", "k_stream_commit_round", "k_stream_index_pred", "k_pred_dirty",
              "k_index_first_init", "k_stream_index_first", "k_stream_index_mark", "k_stream_commit_index",
              "k_scan_offsets", "k_pack_filters", "k_block_digest", "k_index_first", "k_index_mark")


def index_group_sizes(seed: int, lo: int, hi: int):
    """File sizes of one sdhash --index group: log-uniform lo..hi, up to the
    first file that takes the running total past 640 MiB (the group's end,
    sdhash_threads.cc:409,455)."""
    from sdhash_gb300 import synth
    sizes = synth.log_uniform_sizes(seed, 100000, lo, hi)
    k = int(np.searchsorted(np.cumsum(sizes.astype(np.int64)), 640 << 20, side="right")) + 1
    return sizes[:k]


def main_index_build(args):
    """sdhash --index on the GPU (sdbfg_digest_batch_index): one group of
    files below 16 MiB (sizes log-uniform 4 KiB..16 MiB, mixture content,
    just over 640 MiB -- the group sdhash --index closes) digested in stream
    mode into a fresh 64 MiB index, from pinned host memory, the index bits
    copied in and out.  Every file's digest depends on the index inserts of
    the files before it; the engine runs fixed-point rounds of the parallel
    commit (index_rounds).  value: summed device time of the call's kernels
    (CUDA events); e2e: the whole call.  Also measured: the same group cut
    from one shared 96 MiB pool (most features recur across files), the
    sequential one-warp commit, and a block-mode group (16 KiB blocks,
    64 MiB files).  cpu_baseline: the oracle's sequential index build (one
    core, as the reference builds a group with -p 1) on the first files of
    the group, which also checks the GPU's digests of those files.
    --quick leaves out the comparison runs (for profiling the main call)."""
    import ctypes as C
    import torch
    import sdhash_gb300 as g
    from sdhash_gb300 import DigestResult, lib, synth, _ptr
    torch.cuda.set_device(0)
    ctx = g.Context(0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)

    def group(sizes, fill):
        sizes = np.ascontiguousarray(sizes, dtype=np.uint64)
        offs, total = synth.packed_layout(sizes)
        data = torch.empty(max(16, total), dtype=torch.uint8, pin_memory=True).numpy()
        fill(data, offs, sizes)
        return data, np.ascontiguousarray(offs, dtype=np.uint64), sizes, int(sizes.sum())

    def fill_mixture(seed):
        def f(data, offs, sizes):
            synth.fill_many(seed, "mixture", sizes, out=data)
        return f

    def fill_pool(data, offs, sizes):
        pool = synth.mixture_bytes(args.seed + 6100, 0, 96 << 20)
        rng = np.random.default_rng(args.seed + 6100)
        for k in range(len(sizes)):
            n, o = int(sizes[k]), int(offs[k])
            a = int(rng.integers(0, pool.size - n + 1))
            data[o:o + n] = pool[a:a + n]
            m = min(n, 8192)
            data[o:o + m] = synth.random_bytes(args.seed + 6101, k, m)

    bits_host = torch.empty(64 << 20, dtype=torch.uint8, pin_memory=True).numpy()

    def runner(data, offs, lens, dd):
        n = len(lens)
        cap = ctx.capacity(lens, dd)
        out_f = torch.empty(max(1, cap) * 256, dtype=torch.uint8, pin_memory=True).numpy()
        out_c = np.zeros(max(1, cap), dtype=np.uint16)
        res = (DigestResult * n)()
        ec = np.zeros(1, dtype=np.uint64)

        def call():
            bits_host[:] = 0
            ec[0] = 0
            ctx._check(lib().sdbfg_digest_batch_index(ctx.h, data.ctypes.data, _ptr(offs), _ptr(lens), n, dd,
                                                      out_f.ctypes.data, cap, out_c.ctypes.data, res,
                                                      bits_host.ctypes.data, bits_host.size, _ptr(ec)))
            return int(ec[0])
        return call, res, out_f, cap

    def wall_of(call, steps):
        for _ in range(max(3, args.warmup)):
            call()
        t0 = time.perf_counter()
        for _ in range(steps):
            call()
        return (time.perf_counter() - t0) / steps

    sizes = index_group_sizes(args.seed + 6000, 4096, (16 << 20) - 1)
    data, offs, lens, total = group(sizes, fill_mixture(args.seed + 6000))
    call, res, out_f, cap = runner(data, offs, lens, 0)
    for _ in range(max(3, args.warmup)):
        call()
    torch.cuda.synchronize()
    clocks = ClockSampler(0)
    clocks.start()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ec = call()
    wall = (time.perf_counter() - t0) / args.steps
    clocks.stop()
    rounds = ctx.index_rounds
    ctx.profile(True)
    l0 = ctx.launch_count
    for _ in range(args.steps):
        call()
    kern = {}
    for k in IB_KERNELS:
        ms, cnt = ctx.kernel_time(k)
        if cnt:
            kern[k] = ms / args.steps
    launches = (ctx.launch_count - l0) // args.steps
    ctx.profile(False)
    dev_ms = sum(kern.values())
    # the sequential commit on the same group
    wall_seq = None
    if not args.quick:
        ctx.set_index_rounds(0)
        wall_seq = wall_of(call, 1)
        ctx.set_index_rounds(16)
    # parity + CPU baseline: the oracle's sequential build of the first files
    # (a prefix of the group has the same digests as in the whole group)
    from oracle import Oracle
    O = Oracle()
    call()
    pre = int(np.searchsorted(np.cumsum(lens.astype(np.int64)), int(args.cpu_sample_gib * 2 ** 30 / 24),
                              side="right")) + 1
    pre = min(pre, len(lens))
    sample = [data[int(offs[k]):int(offs[k]) + int(lens[k])] for k in range(pre)]
    obits = np.zeros(64 << 20, dtype=np.uint8)
    t1 = time.perf_counter()
    want, _ = O.index_build_stream(sample, [f"f{k}" for k in range(pre)], obits)
    t_cpu = time.perf_counter() - t1
    for k in range(pre):
        w = want[k]
        if w is None:
            assert res[k].status != 0
            continue
        o, nb = int(res[k].filter_offset), int(res[k].bf_count)
        assert (nb, int(res[k].last_count)) == (w.bf_count, w.last_count), f"index build: file {k} differs"
        assert out_f[o * 256:(o + nb) * 256].tobytes() == w.filters(), f"index build: file {k} filters differ"
    sample_bytes = int(lens[:pre].sum())
    extra = {}
    if not args.quick:
        # shared-pool content: the same sizes, features recurring across files
        pdata, poffs, plens, ptotal = group(sizes, fill_pool)
        pcall, _, _, _ = runner(pdata, poffs, plens, 0)
        pwall = wall_of(pcall, args.steps)
        prounds = ctx.index_rounds
        ctx.set_index_rounds(0)
        pwall_seq = wall_of(pcall, 1)
        ctx.set_index_rounds(16)
        del pdata
        # block-mode group: 64 MiB files
        bsizes = np.full(11, 64 << 20, dtype=np.uint64)
        bdata, boffs, blens, btotal = group(bsizes, fill_mixture(args.seed + 6200))
        bcall, _, _, _ = runner(bdata, boffs, blens, 16384)
        bwall = wall_of(bcall, args.steps)
        del bdata
        extra = {"sequential_commit_e2e": {"value": total / wall_seq / 1e9, "unit": "GB/s",
                                           "path": "the same call with index rounds off (one-warp commit)"},
                 "shared_pool_e2e": {"value": ptotal / pwall / 1e9, "unit": "GB/s", "index_rounds": prounds,
                                     "sequential_commit": ptotal / pwall_seq / 1e9,
                                     "content": "files cut from one 96 MiB mixture pool (first 8 KiB fresh)"},
                 "block_group_e2e": {"value": btotal / bwall / 1e9, "unit": "GB/s", "files": len(blens),
                                     "input_bytes": btotal, "block": 16384}}
    hbm, src = peaks()
    tiles_ms = kern.get("k_stream_tiles", 0.0)
    d2h = int(cap) * 256 + len(lens) * 24 + (64 << 20)
    line = {"metric": IB_METRIC, "value": total / (dev_ms / 1e3) / 1e9, "unit": "GB/s", "n_gpus": 1,
            "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": dev_ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
            "config": {"workload": "stream-mode index build (sdhash --index, one group)", "files": len(lens),
                       "input_bytes": total, "sizes": "log-uniform 4 KiB..16 MiB, up to the file past 640 MiB",
                       "content": "mixture, distinct per file", "index_bytes": 64 << 20,
                       "l2": "inputs larger than L2 (no flush needed)"},
            "gpu_launches": int(launches), "clocks": clocks.summary(), "index_rounds": rounds,
            "elements_inserted": ec, "kernel_ms_per_step": kern,
            "roofline": {"bound": "hbm", "kernel": "k_stream_tiles",
                         "achieved": total / (tiles_ms / 1e3) / 1e9 if tiles_ms else None, "peak": hbm,
                         "unit": "GB/s", "frac": total / (tiles_ms / 1e3) / 1e9 / hbm if tiles_ms else None,
                         "traffic": None, "peak_source": f"{src} hbm_gbs (MEASURED_PEAKS.json)",
                         "algorithmic_bytes_per_step": total},
            "e2e": {"value": total / wall / 1e9, "unit": "GB/s", "h2d_bytes_per_step": total + (64 << 20),
                    "d2h_bytes_per_step": d2h, "ms_per_step": wall * 1e3,
                    "path": "sdbfg_digest_batch_index from pinned host memory"},
            **extra,
            "cpu_baseline": {"value": sample_bytes / t_cpu / 1e9, "unit": "GB/s", "cores": 1, "kind": "port",
                             "sample": f"the group's first {pre} files ({sample_bytes} bytes), oracle index build",
                             "seconds": round(t_cpu, 3)}}
    print(json.dumps(line), flush=True)
    return 0


LD_METRIC = "SDBF text loaded GB/s"


def main_load(args):
    """Bulk load of a large SDBF reference set from its text form into a
    resident set (sdbf_set(const char* fname), sdbf/sdbf_set.cc:51-74): the
    serving workload's block-mode reference image written out with
    to_string, then loaded K times.  value: the device decode kernel over
    text already in HBM (k_text_decode, CUDA events); e2e: the whole
    Context.load_text call from host text (header scan, host->device copy,
    decode, checks); cpu_baseline: the oracle's line parser, one thread --
    the reference's loader reads and parses one line at a time."""
    import torch
    import sdhash_gb300 as g
    torch.cuda.set_device(0)
    ctx = g.Context(0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    refs, _, _ = serve_reference_set(args, ctx, stream, 0)
    text = "".join(d.to_string() for d in refs).encode()
    nfilt = sum(d.bf_count for d in refs)
    nb = len(text)
    for _ in range(max(3, args.warmup)):
        ctx.load_text(text).close()
    torch.cuda.synchronize()
    clocks = ClockSampler(0)
    clocks.start()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ds = ctx.load_text(text)
        ds.close()
    torch.cuda.synchronize()
    wall = (time.perf_counter() - t0) / args.steps
    clocks.stop()
    # device part: kernel time per launch (CUDA events on the launch stream)
    ctx.profile(True)
    launches0 = ctx.launch_count
    for _ in range(args.steps):
        ctx.load_text(text).close()
    ms, n = ctx.kernel_time("k_text_decode")
    n_launch = ctx.launch_count - launches0
    ctx.profile(False)
    kms = ms / max(1, n)
    # parity at size: a sample of loaded digests equals the digests written out
    ds = ctx.load_text(text)
    for i in range(0, len(refs), max(1, len(refs) // 8)):
        d = ds.digest(i)
        assert d.to_string() == refs[i].to_string(), "loaded digest differs"
    ds.close()
    # CPU: the oracle's parser over a sample of lines, one thread
    from oracle import Oracle
    O = Oracle()
    lines = text.splitlines(True)
    t1 = time.perf_counter()
    done = 0
    k = 0
    while time.perf_counter() - t1 < 10.0 and k < len(lines):
        O.parse(lines[k].decode())
        done += len(lines[k])
        k += 1
    t_cpu = time.perf_counter() - t1
    hbm, src = peaks()
    alg = nb + nfilt * (256 + 4)   # text read once, filters and (hamming, count) words written
    achieved = alg / (kms / 1e3) / 1e9
    line = {"metric": LD_METRIC, "value": nb / (kms / 1e3) / 1e9, "unit": "GB/s", "n_gpus": 1,
            "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": kms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u8 (base64 text)", "data": "synthetic",
            "config": {"workload": "bulk SDBF text load: block-mode reference set (serving image)",
                       "digests": len(refs), "filters": nfilt, "text_bytes": nb,
                       "l2": "text larger than L2 (no flush needed)"},
            "gpu_launches": int(n_launch // max(1, args.steps)),
            "clocks": clocks.summary(),
            "roofline": {"bound": "hbm", "kernel": "k_text_decode", "achieved": achieved, "peak": hbm,
                         "unit": "GB/s", "frac": achieved / hbm, "traffic": None,
                         "peak_source": f"{src} hbm_gbs (MEASURED_PEAKS.json)",
                         "algorithmic_bytes_per_launch": alg},
            "e2e": {"value": nb / wall / 1e9, "unit": "GB/s", "h2d_bytes_per_step": nb,
                    "d2h_bytes_per_step": 4 * len(refs), "ms_per_step": wall * 1e3,
                    "filters_per_s": nfilt / wall,
                    "path": "Context.load_text(host bytes) -> resident set (sdbfg_set_load_text)"},
            "cpu_baseline": {"value": done / t_cpu / 1e9, "unit": "GB/s", "cores": 1, "kind": "port",
                             "sample": f"{k} of {len(lines)} lines parsed by the oracle, one thread",
                             "seconds": round(t_cpu, 3)}}
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    if args.workload == "load":
        return main_load(args)
    if args.workload == "index":
        return main_index(args)
    if args.workload == "index-build":
        return main_index_build(args)
    if args.workload == "serve":
        return main_serve(args)
    if args.workload == "image":
        return main_image(args)
    if args.workload == "allpairs":
        return main_allpairs(args)
    if args.impl == "reference":
        return run_reference(args)
    rank, world, local = dist_setup(args.gpus)
    import torch
    import sdhash_gb300 as g
    torch.cuda.set_device(local)
    buf, data, offs, sizes, sizes_all = make_workload(args, rank, world, pinned=True)
    total_bytes = int(sizes.sum())
    ctx = g.Context(local)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    dev = torch.empty(max(16, len(data)), dtype=torch.uint8, device="cuda")
    dev.copy_(buf, non_blocking=True)
    cap = ctx.capacity(sizes, 0)
    out = torch.empty(max(1, cap) * 256, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()

    def step_device():
        return ctx.digest_device(dev.data_ptr(), offs, sizes, 0, out.data_ptr(), cap)

    for _ in range(args.warmup):
        step_device()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    launches0 = ctx.launch_count
    barrier(world)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    w0 = time.perf_counter()
    e0.record(stream)
    for _ in range(args.steps):
        res = step_device()
    e1.record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - w0
    barrier(world)
    clocks.stop()
    dev_ms = e0.elapsed_time(e1)
    launches = ctx.launch_count - launches0
    # the last timed step's device output and results, for the parity checks
    out_dev_host = out.cpu().numpy()

    # One more step, outside the timed region, with launch groups run one
    # after another and per-kernel CUDA events on the launch stream: the
    # kernels do not overlap, so each event pair brackets one kernel alone.
    depth0 = ctx.pipeline_depth
    ctx.set_pipeline_depth(1)
    ctx.profile(True)
    step_device()
    torch.cuda.synchronize()
    kern = {k: ctx.kernel_time(k) for k in KERNELS}
    ntile_ph = ctx.kernel_time("k_stream_tiles.count")[0] or 1.0
    phases = {k: ctx.kernel_time("k_stream_tiles." + k)[0] / ntile_ph
              for k in ("load", "ranks", "fres", "walk", "link", "compact", "sha1", "fixups")}
    commit_ph = {k: ctx.kernel_time("k_stream_commit." + k)[0] for k in ("wait", "busy", "groups", "loops", "max_file")}
    ctx.profile(False)
    ctx.set_pipeline_depth(depth0)
    tiles_ms, tiles_n = kern["k_stream_tiles"]
    ms_per_step = allmax(world, dev_ms / args.steps)
    bytes_all = allsum(world, total_bytes)
    value = bytes_all / (ms_per_step / 1e3) / 1e9
    out_filters = sum(int(r.bf_count) for r in res[: len(sizes)]) if len(sizes) else 0
    plain = plain_per_call(ctx, dev, offs, sizes, args.plain_gib) if args.plain_gib > 0 else None

    # e2e through the C ABI's host-buffer entry point (sdbfg_digest_batch):
    # the caller's pinned input in, the packed filters and per-file results
    # out into the caller's host buffers, every step
    e2e, e2e_bad = None, None
    if not args.no_e2e:
        import ctypes as C
        from sdhash_gb300 import DigestResult, lib, _ptr, _u64
        o64, l64 = _u64(offs), _u64(sizes)
        nf = len(sizes)
        cap_f = ctx.capacity(l64, 0)
        out_host = torch.empty(max(1, cap_f) * 256, dtype=torch.uint8, pin_memory=True).numpy()
        res_c = (DigestResult * max(1, nf))()

        def abi_call():
            ctx._check(lib().sdbfg_digest_batch(ctx.h, data.ctypes.data, _ptr(o64), _ptr(l64), nf, 0,
                                                out_host.ctypes.data, cap_f, None, res_c))

        abi_call()  # warm host staging
        barrier(world)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            abi_call()
        torch.cuda.synchronize()
        e2e_s = allmax(world, (time.perf_counter() - t0) / args.steps)
        d2h = sum(int(res_c[i].bf_count) for i in range(nf) if res_c[i].status == 0) * 256 + C.sizeof(res_c)
        e2e_bad = parity_host_vs_device(res, out_dev_host, res_c, out_host, nf)
        # the Python object API on the same batch, once (Digest objects built on the host)
        t1 = time.perf_counter()
        ds = ctx.digest_packed(data, offs, sizes, 0)
        py_s = allmax(world, time.perf_counter() - t1)
        del ds
        e2e = {"value": bytes_all / e2e_s / 1e9, "unit": UNIT, "h2d_bytes_per_step": int(total_bytes),
               "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_s * 1e3,
               "path": "C ABI sdbfg_digest_batch: pinned host input -> packed filters + results in host buffers",
               "python_api_value": bytes_all / py_s / 1e9}

    peak, peak_kind = peaks()
    ngroups = max(1, tiles_n)
    per_launch_bytes = total_bytes / ngroups
    tile_ms = tiles_ms / max(1, tiles_n)
    achieved = per_launch_bytes / (tile_ms / 1e3) / 1e9 if tile_ms > 0 else None
    tpb = profiled_traffic("k_stream_tiles")
    # the bound that holds: integer issue (warp instructions per input byte
    # from the committed ncu capture x achieved bytes/s, against one warp
    # instruction per scheduler per clock)
    wipb = profiled_value("k_stream_tiles", "warp_inst_per_input_byte")
    sm_mhz = clocks.summary().get("sm_mhz") or 2070.0
    issue_peak = 152 * 4 * sm_mhz * 1e6
    issue = None
    if wipb and achieved:
        issue = {"unit": "warp instructions/s", "warp_inst_per_input_byte": wipb,
                 "achieved": wipb * achieved * 1e9, "peak": issue_peak, "frac": wipb * achieved * 1e9 / issue_peak,
                 "ceiling_GBs_at_full_issue": issue_peak / wipb / 1e9,
                 "source": "profiles/k_stream_tiles_ncu.md (smsp__inst_executed per input byte); peak = 152 SMs x "
                           "4 schedulers x median SM clock"}
    # the rank kernel that runs ahead of each tile launch: input bytes per
    # second of its launches, and the same issue arithmetic
    ranks_ms, ranks_n = kern.get("k_stream_ranks", (0.0, 0))
    ranks = None
    if ranks_ms > 0:
        r_ach = total_bytes / (ranks_ms / 1e3) / 1e9
        r_wipb = profiled_value("k_stream_ranks", "warp_inst_per_input_byte")
        r_tpb = profiled_traffic("k_stream_ranks")
        ranks = {"kernel": "k_stream_ranks", "launches": ranks_n, "achieved_GBs": r_ach,
                 "frac_of_hbm": r_ach / peak if peak else None,
                 "traffic": (r_tpb * per_launch_bytes) if r_tpb else None,
                 "issue_frac": (r_wipb * r_ach * 1e9 / issue_peak) if r_wipb else None,
                 "warp_inst_per_input_byte": r_wipb}
    roofline = {"bound": "hbm", "kernel": "k_stream_tiles_pre", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "issue": issue, "ranks_kernel": ranks,
                "frac": (achieved / peak) if achieved else None,
                "traffic": (tpb * per_launch_bytes) if tpb else None,
                "peak_source": f"{peak_kind} hbm_gbs (MEASURED_PEAKS.json)",
                "algorithmic_bytes_per_launch": per_launch_bytes,
                "kernel_ms_unoverlapped_step": {k: v[0] for k, v in kern.items()},
                "tile_phase_cycles_per_tile": phases, "commit_phase_totals": commit_ph}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u8", "data": "synthetic",
            "config": dict(CONFIG_BASE, total_bytes=int(bytes_all), files_per_rank=len(sizes),
                           parallelism=f"files sharded over {world} GPU(s)", wall_s_timed=round(wall, 3),
                           out_filters_per_step=out_filters),
            "gpu_launches": launches, "clocks": clocks.summary(), "roofline": roofline, "e2e": e2e}
    if plain:
        line["plain_per_call"] = plain
        line["batched_over_plain"] = value / plain["value"]
    parity = {"files_checked": 0, "mismatches": 0}
    if rank == 0 and world == 1:
        cb, pick, ores = cpu_baseline(args, data, offs, sizes, keep=True)
        line["cpu_baseline"] = cb
        bad, nb = parity_vs_oracle(pick, ores, sizes, res, out_dev_host)
        del ores
        parity.update(files_checked=len(pick), mismatches=len(bad), bytes_checked=nb,
                      checked="oracle digests of the cpu_baseline sample against the last timed step's device "
                              "output (filters, bf_count, last_count)")
        if bad:
            parity["mismatched_files"] = bad[:16]
    if e2e_bad is not None:
        parity.update(e2e_files_checked=len(sizes), e2e_mismatches=len(e2e_bad),
                      e2e_checked="every file: sdbfg_digest_batch host output against the device-resident output")
        parity["mismatches"] += len(e2e_bad)
    line["parity"] = parity
    if rank == 0:
        print(json.dumps(line), flush=True)
    barrier(world)
    return 0


if __name__ == "__main__":
    sys.exit(main())
