#!/usr/bin/env python
"""Throughput benchmark of the chart-parsing hot path on one GB300.

Workload (one "step"): parse 20,000 sentences with the ~1,100-symbol split
grammar -- coarse (98-symbol) Viterbi inside/outside, pruning masks at a
log max-marginal of -9, fine Viterbi inside pass and on-device backtrace --
exactly the reference's ``CLParser.parse`` cascade.  Grammar and sentences are
seeded synthetic data with the published shapes (98 coarse symbols split into
1-16 subsymbols, ~1.5M binary rules with Gamma(0.3) weights, 40k-word Zipf(1.1)
vocabulary, lognormal lengths with mean 23 clipped to 1-40).

Reported (one JSON line on rank 0):
  value   sentences/s from the library's CUDA-event device time (first to last
          kernel of each batch; word ids already copied)
  e2e     sentences/s through the public C-ABI call with host buffers, host<->
          device copies included
  roofline  the fine-level inside span kernel (the dominant kernel)
  cpu_baseline  the CPU oracle (a port of the reference algorithm) on a
          bounded sample, all host threads
  plain   the same library run one sentence at a time (max_batch_sentences=1)
          on a bounded sample: the plain CUDA CKY path the batched and served
          paths are compared with
  serving the continuous-batching server under open-loop Poisson arrivals
          (lengths lognormal mean 23 clipped 1-60): achieved sentences/s and
          p50/p99 latency per offered rate

``--impl reference`` times the reference's algorithm on the host cores (the
oracle port: the reference's own JVM/OpenCL stack cannot run on this machine).
Under torchrun with N > 1 each rank parses its own 20,000 sentences (replicas,
weak scaling, no collective on the data path).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_SENT = 20000
MAX_LEN = 40
FINE_INSIDE_BYTES_PER_UNIT = 0.0813


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def workload(seed: int, n_sent: int, grammar_seed: int = 1, fine_semiring: str = "viterbi"):
    import numpy as np
    from puck_gb300 import grammar, grz, synth
    t0 = time.time()
    c, f = synth.split_grammar(seed=grammar_seed)
    levels = [grammar.compile_level(c, "viterbi"), grammar.compile_level(f, fine_semiring)]
    path = os.path.join(tempfile.gettempdir(),
                        f"puck_bench_split_{grammar_seed}_{fine_semiring}_{os.getpid()}.grz")
    grz.write_sequence(path, levels)
    sents = synth.lognormal_sentences(seed, n_sent, 23, 1, MAX_LEN, len(f.words))
    log(f"workload ready in {time.time() - t0:.1f}s: fine nt={levels[1].n_nt} t={levels[1].n_t} "
        f"rules={f.bin_rules.shape[0]} sentences={n_sent} mean_len={np.mean([len(s) for s in sents]):.2f}")
    return levels, path, sents


def long_workload(seed: int, n_sent: int):
    """Long-sentence stress grammar: ~2,000 fine symbols (splits up to 32),
    ~4M binaries; lengths uniform in 41-100."""
    import numpy as np
    from puck_gb300 import grammar, grz, synth
    t0 = time.time()
    c, f = synth.split_grammar(seed=5, max_split=32, mean_split=20.4, target_fine_rules=4_000_000)
    levels = [grammar.compile_level(c, "viterbi"), grammar.compile_level(f, "viterbi")]
    path = os.path.join(tempfile.gettempdir(), f"puck_bench_long_{os.getpid()}.grz")
    grz.write_sequence(path, levels)
    sents = synth.uniform_sentences(seed, n_sent, 41, 100, len(f.words))
    log(f"long workload ready in {time.time() - t0:.1f}s: fine nt={levels[1].n_nt} t={levels[1].n_t} "
        f"rules={f.bin_rules.shape[0]} sentences={n_sent} mean_len={np.mean([len(s) for s in sents]):.2f}")
    return levels, path, sents


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.path = tempfile.mktemp(suffix=".csv")
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        rows = []
        try:
            for line in open(self.path):
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9 and parts[0] == str(self.index):
                    rows.append(parts)
        except Exception:
            pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {}


def cpu_baseline(levels, sents, sample: int):
    import oracle
    import numpy as np
    sub = sents[:sample]
    threads = os.cpu_count() or 1
    L = [oracle.OracleLevel(l) for l in levels]
    r = oracle.OracleRun(L, sub, threads=threads)
    t0 = time.perf_counter()
    rc = r.run("parse")
    dt = time.perf_counter() - t0
    assert rc == 0
    return {"value": round(len(sub) / dt, 3), "unit": "sentences/s", "cores": threads, "kind": "port",
            "sample": f"first {len(sub)} sentences of the workload (mean length "
                      f"{np.mean([len(s) for s in sub]):.1f}), full cascade: coarse inside/outside, masks, "
                      f"fine inside, backtrace; {dt:.1f}s"}, r


def e2e_roofline(P, nlevels: int, dev_ms, fp32_peak: float) -> dict:
    """The end-to-end fraction: every level's binary-pass work of the last
    timed step (each step parses the same workload) at the FP32 lane peak,
    over the step's device time.  The HBM-bound kernels (lexicon, masks,
    decode) are a few percent of device time and are left out."""
    try:
        step_ops = 2.0 * sum(P.level_work(l)[0] for l in range(nlevels))
        step_s = sum(dev_ms) / len(dev_ms) / 1e3
        return {"frac": round(step_ops / (fp32_peak * 1e12) / step_s, 4), "ops_per_step": step_ops,
                "peak": round(fp32_peak, 2), "unit": "TFLOP/s",
                "note": "all levels' binary passes (2 ops per work unit) at the FP32 lane peak / device "
                        "time per step; HBM-bound kernels not counted"}
    except Exception as exc:  # a report, never a reason to lose the line
        return {"unavailable": str(exc)[:160]}


def reference_work(r, value: float) -> dict:
    """The reference's work measure on the CPU-baseline sample: (rule, split)
    applications its binary queues run in the last level's inside pass
    (rows queued per rule block times the block's rules, counted by the
    oracle), per sentence and at this run's sentences/s."""
    apps = r.rule_apps(len(r.levels) - 1, "inside") / max(len(r.lengths), 1)
    return {"rule_apps_per_sentence": round(apps), "rule_apps_per_s": float(f"{apps * value:.4g}"),
            "sample": f"the {len(r.lengths)} sentences of the CPU baseline",
            "note": "reference-equivalent CKY rule applications (fine inside, after pruning); "
                    "not the roofline's split-factored work"}


def parity(path, sents, batch_nodes, r, device: int):
    """The GPU's results on the CPU-baseline sample against the oracle's
    (the oracle run ``r`` of that sample): the sample's trees taken from the
    timed full-workload batch, and the sample parsed again as its own batch
    for its pruning masks and charts.  Viterbi results must be bit-identical;
    a tree that differs counts as explained only when its root score is
    within 1e-5 relative of the oracle's (a near-tie)."""
    import numpy as np
    from puck_gb300.parser import CLParser, pack_sentences
    sub = sents[:len(r.lengths)]
    lens = [len(s) for s in sub]
    k = sum(2 * n - 1 for n in lens)
    ref = r.trees()
    got = batch_nodes[:k]
    same, near, start = 0, 0, 0
    for n in lens:
        a, b = got[start:start + 2 * n - 1], ref[start:start + 2 * n - 1]
        start += 2 * n - 1
        if np.array_equal(a, b):
            same += 1
        else:
            sa, sb = float(a[0, 3:4].view(np.float32)[0]), float(b[0, 3:4].view(np.float32)[0])
            near += abs(sa - sb) <= 1e-5 * abs(sb)
    P = CLParser(path, max_alloc_size=8 << 30, device=device, max_length=MAX_LEN)
    w, o, _ = pack_sentences(sub)
    alone, st = P.parse_ids(w, o)
    assert (st == 0).all()
    bits = lambda x: np.ascontiguousarray(x).view(np.int32)
    masks_same = bool(np.array_equal(P.debug_copy(0, "masks"), r.masks(0)[0]))
    coarse_same = bool(np.array_equal(bits(P.debug_copy(0, "inside")), bits(r.chart(0, "inside"))) and
                       np.array_equal(bits(P.debug_copy(0, "outside")), bits(r.chart(0, "outside"))))
    fine_same = bool(np.array_equal(bits(P.debug_copy(1, "inside")), bits(r.chart(1, "inside"))))
    P.release()
    return {"sentences": len(sub), "trees_identical": same, "masks_identical": masks_same,
            "coarse_charts_identical": coarse_same, "fine_inside_chart_identical": fine_same,
            "alone_equals_batch": bool(np.array_equal(alone, got)),
            "divergences_within_1e-5": int(near), "divergences_unexplained": int(len(sub) - same - near),
            "oracle_corner_drops": int(r.corner_drops(1)),
            "note": "oracle = CPU restatement of the reference's cascade; trees from the timed batch"}


def plain_baseline(path, sents, sample: int, device: int):
    """The library one sentence at a time: every span launch covers the
    cells of a single sentence."""
    from puck_gb300.parser import CLParser, pack_sentences
    P = CLParser(path, max_alloc_size=8 << 30, profile=True, device=device, max_length=MAX_LEN,
                 max_batch_sentences=1)
    sub = sents[:sample]
    words, offsets, _ = pack_sentences(sub)
    P.parse_ids(*pack_sentences(sub[:4])[:2])  # warm-up
    t0 = time.perf_counter()
    nodes, st = P.parse_ids(words, offsets)
    dt = time.perf_counter() - t0
    assert (st == 0).all()
    s = P.stats()
    P.release()
    return {"value": round(len(sub) / (s["ms_device"] / 1e3), 2), "unit": "sentences/s",
            "e2e": round(len(sub) / dt, 2),
            "sample": f"first {len(sub)} sentences of the workload, one batch per sentence (device time)"}


def serving(path, levels, args, device: int):
    """Open-loop Poisson arrivals into the continuous-batching server."""
    import threading
    import numpy as np
    from puck_gb300 import synth
    from puck_gb300.parser import pack_sentences
    from puck_gb300.server import CLServer, now_ns
    n = args.serve_sentences
    sents = synth.lognormal_sentences(args.seed + 1000, n, 23, 1, 60, len(levels[1].lex_offsets) - 1)
    words, offsets, lens = pack_sentences(sents)
    S = CLServer(path, max_alloc_size=args.serve_mem_gb << 30, device=device, max_length=60, collect=False,
                 profile=True, lanes=args.serve_lanes)

    def drain(count, want):
        lat, done_at = [], []
        while len(lat) < count:
            for rid in S.poll(8192, 20):
                nodes, st, ln = S.take(int(rid), want[int(rid)])
                assert st == 0
                lat.append(ln)
        return np.array(lat, np.int64)

    # warm-up: a few hundred sentences at once
    w0, o0, l0 = pack_sentences(sents[:256])
    ids = S.submit_ids(w0, o0)
    drain(len(ids), {int(i): int(k) for i, k in zip(ids, l0)})
    rows = []
    rng = np.random.default_rng(args.seed + 2000)
    for rate in args.serve_rates:
        gaps = rng.exponential(1.0 / rate, n)
        st0 = S.stats()
        pm0 = [S.pass_ms(l) for l in range(len(levels))]
        t0 = now_ns() + 2_000_000
        sched = t0 + np.cumsum(gaps * 1e9).astype(np.int64)
        want = {}
        lock = threading.Lock()

        def gen():
            i = 0
            while i < n:
                t = now_ns()
                j = int(np.searchsorted(sched, t, side="right"))
                if j > i:
                    o = offsets[i:j + 1] - offsets[i]
                    w = words[offsets[i]:offsets[j]]
                    with lock:
                        rid = S.submit_ids(w, o, sched[i:j])
                        for k, r in enumerate(rid):
                            want[int(r)] = int(lens[i + k])
                    i = j
                else:
                    time.sleep(min(2e-4, max((sched[i] - t) / 1e9, 0)))

        th = threading.Thread(target=gen)
        th.start()
        lat, got = [], 0
        t_last = t0
        while got < n:
            for rid in S.poll(8192, 20):
                with lock:
                    ln_ = want[int(rid)]
                nodes, st, ln = S.take(int(rid), ln_)
                assert st == 0
                lat.append(ln)
                got += 1
            t_last = now_ns()
        th.join()
        st1 = S.stats()
        lat = np.array(lat, np.float64) / 1e6
        span_s = (t_last - t0) / 1e9
        rows.append({"offered": rate, "achieved": round(n / span_s, 1),
                     "p50_ms": round(float(np.percentile(lat, 50)), 2),
                     "p99_ms": round(float(np.percentile(lat, 99)), 2),
                     "resident_peak": int(st1["resident_peak"]),
                     "ticks": int(st1["ticks"] - st0["ticks"]),
                     "gpu_ms": round(st1["ms_device"] - st0["ms_device"], 1),
                     "pass_ms": {f"level{l}": [round(a - b, 1) for a, b in zip(S.pass_ms(l), pm0[l])]
                                 for l in range(len(levels))}})
        log(f"serving {rate}/s: {rows[-1]}")
    lanes = S.lanes()
    S.close()
    return {"sentences_per_rate": n, "lanes": lanes, "lengths": "lognormal mean 23 clipped 1-60",
            "arrivals": "open-loop Poisson, latency from scheduled arrival to result available on the host",
            "rates": rows}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(world, x: float) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_ours(args):
    import numpy as np
    import torch
    from puck_gb300.parser import CLParser, pack_sentences
    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    levels, path, sents = workload(args.seed + rank, args.sentences)
    words, offsets, lens = pack_sentences(sents)
    P = CLParser(path, max_alloc_size=args.mem_gb << 30, profile=True, device=local, max_length=MAX_LEN,
                 use_graphs=True)
    # the library's autotuner picks the split waves and, per level, the span
    # band of the flat-tile inside form on a sample of the workload, before
    # any timing
    tw, to, _ = pack_sentences(sents[:args.tune_sample]) if args.tune_sample > 0 else (None, None, None)
    tuned = P.autotune(tw, to) if args.tune_sample > 0 else None
    for _ in range(args.warmup):
        nodes, st = P.parse_ids(words, offsets)
    assert (st == 0).all(), "sentences failed to parse"
    dev_ms, api_ms, fine_in_ms, fine_in_launch, work, launches, h2d, d2h = [], [], 0.0, 0, 0, 0, 0, 0
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with ClockSampler(local) as clk:
        barrier(world)
        torch.cuda.synchronize()
        for k in range(args.steps):
            ev[k][0].record()
            nodes, st = P.parse_ids(words, offsets)
            ev[k][1].record()
            s = P.stats()
            dev_ms.append(s["ms_device"])
            work += P.level_work(len(levels) - 1)[0]
            launches += s["kernel_launches"]
            h2d, d2h = s["h2d_bytes"], s["d2h_bytes"]
            ms, n = P.pass_ms(len(levels) - 1)
            fine_in_ms += ms[0]
            fine_in_launch += n[0]
        torch.cuda.synchronize()
        barrier(world)
    api_ms = [ev[k][0].elapsed_time(ev[k][1]) for k in range(args.steps)]
    clocks = clk.summary()
    dev_total = allmax(world, sum(dev_ms) / 1e3)
    api_total = allmax(world, sum(api_ms) / 1e3)
    units = args.sentences * args.steps * world
    value = units / dev_total
    e2e = units / api_total
    # roofline of the dominant kernel: the fine inside span pass (FP32 max-plus on CUDA cores)
    pk = peaks()
    sm_max = float(pk.get("sm_max_mhz", 2070.0))
    fp32_peak = 152 * 128 * sm_max * 1e6 / 1e12                 # FP32 lane-ops/s in T
    # split-factored work units: each (live split, child pair) element of M and
    # each applied rule is one add and one max
    per_launch_ops = 2.0 * work / max(fine_in_launch, 1)
    avg_launch_s = fine_in_ms / 1e3 / max(fine_in_launch, 1)
    achieved = per_launch_ops / avg_launch_s / 1e12
    # DRAM traffic per work unit of the fine inside kernel, measured with ncu
    # on fine inside launches of a 2,000-sentence run of this workload, scaled
    # to this run's average launch
    traffic = FINE_INSIDE_BYTES_PER_UNIT * work / max(fine_in_launch, 1)
    out = {
        "metric": "sentences/sec, 1.1k-symbol grammar, len<=40 (batched/served vs plain); p50/p99 ms",
        "value": round(value, 2), "unit": "sentences/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(sum(dev_ms) / len(dev_ms), 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded split grammar and sentences with the published shapes)",
        "config": {"workload": "split-grammar Viterbi cascade: 98 coarse / "
                               f"{levels[1].n_nt + levels[1].n_t} fine symbols, "
                               f"{int(sum(l.shape[0] for l in levels[1].bucket_rules))} binary rules, "
                               f"{args.sentences} sentences lognormal(mean 23) clipped 1-40, prune -9",
                   "sentences_per_step": args.sentences, "prune_threshold": -9.0,
                   "l2": "inputs larger than L2 (coarse+fine charts of a step are ~18 GB)",
                   "parallelism": f"replicas x{world}", "autotuned": tuned, "cuda_graphs": True},
        "e2e": {"value": round(e2e, 2), "unit": "sentences/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": int(launches),
        "clocks": clocks,
        "roofline": {"bound": "alu", "kernel": "k_inside_span<viterbi> (fine level)",
                     "achieved": round(achieved, 3), "peak": round(fp32_peak, 2), "unit": "TFLOP/s",
                     "frac": round(achieved / fp32_peak, 4), "traffic": round(traffic),
                     "traffic_unit": "bytes per launch (ncu, scaled by work units)",
                     "traffic_gbs": round(traffic / avg_launch_s / 1e9, 1),
                     "note": "FP32 max-plus on CUDA cores: ops = 2 x (sum over cells of live splits x child "
                             "pairs + applied rules); peak = 152 SMs x 128 FP32 lanes x measured max SM clock",
                     "work_per_launch": round(work / max(fine_in_launch, 1)),
                     "avg_launch_ms": round(avg_launch_s * 1e3, 4)},
        "passes_ms_last_step": {
            f"level{l}": [round(v, 2) for v in P.pass_ms(l)[0]] for l in range(len(levels))},
        # chart cells of a step (bot and top halves) and those whose coarse
        # mask closes every fine symbol
        "pruning": {"cells": int(s["cells"]), "cells_pruned": int(s["cells_pruned"]),
                    "fraction": round(s["cells_pruned"] / max(s["cells"], 1), 4)},
    }
    out["e2e_roofline"] = e2e_roofline(P, len(levels), dev_ms, fp32_peak)
    P.release()
    if rank == 0 and world == 1:
        if args.cpu_sample > 0:
            out["cpu_baseline"], r_cpu = cpu_baseline(levels, sents, args.cpu_sample)
            try:
                out["reference_work"] = reference_work(r_cpu, value)
            except Exception as exc:  # a report, never a reason to lose the line
                out["reference_work"] = {"unavailable": str(exc)[:160]}
            out["parity"] = parity(path, sents, nodes, r_cpu, local)
            log(f"parity: {out['parity']}")
        if args.plain_sample > 0:
            out["plain"] = plain_baseline(path, sents, args.plain_sample, local)
            out["plain"]["batched_over_plain"] = round(value / out["plain"]["value"], 2)
        if args.serve_rates:
            out["serving"] = serving(path, levels, args, local)
    if rank == 0:
        print(json.dumps(out), flush=True)
    os.unlink(path)


def run_reference(args):
    world, rank, _ = dist_setup()
    if rank != 0:
        return
    import numpy as np
    import oracle
    levels, path, sents = workload(args.seed, args.sentences)
    os.unlink(path)
    threads = os.cpu_count() or 1
    L = [oracle.OracleLevel(l) for l in levels]
    sample = args.cpu_sample
    times = []
    for k in range(args.warmup + args.steps):
        sub = sents[(k * sample) % len(sents):(k * sample) % len(sents) + sample]
        r = oracle.OracleRun(L, sub, threads=threads)
        t0 = time.perf_counter()
        assert r.run("parse") == 0
        if k >= args.warmup:
            times.append(time.perf_counter() - t0)
    value = sample * len(times) / sum(times)
    out = {
        "impl": "reference",
        "metric": "sentences/sec, 1.1k-symbol grammar, len<=40 (batched/served vs plain); p50/p99 ms",
        "value": round(value, 3), "unit": "sentences/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(1e3 * sum(times) / len(times), 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded split grammar and sentences with the published shapes)",
        "config": {"workload": "split-grammar Viterbi cascade (same grammar and sentences as the GPU arm)",
                   "sentences_per_step": sample, "prune_threshold": -9.0},
        "cpu_baseline": {"value": round(value, 3), "unit": "sentences/s", "cores": threads, "kind": "port",
                         "sample": f"{sample} sentences per step; the reference's JVM/OpenCL stack is not "
                                   "runnable here, so its algorithm runs as the C++ port"},
        "e2e": {"value": round(value, 3), "unit": "sentences/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


def run_mbr(args):
    """Sum-product cascade with max-constituent (MBR) trees: throughput of the
    FP32 CUDA-core path, and its log-partition and posterior errors against
    the FP64 oracle on a subset."""
    import numpy as np
    import torch
    import oracle
    from puck_gb300.parser import CLParser, pack_sentences
    torch.cuda.set_device(0)
    levels, path, sents = workload(args.seed, args.sentences, fine_semiring="real")
    words, offsets, _ = pack_sentences(sents)
    P = CLParser(path, max_alloc_size=args.mem_gb << 30, profile=True, max_length=MAX_LEN, decode="mbr",
                 tensor_cores=args.tensor_cores)
    tc_on, tc_why = P.tensor_cores(len(levels) - 1)
    for _ in range(args.warmup):
        nodes, st = P.parse_ids(words, offsets)
        assert (st == 0).all()
    dev_ms, api_ms = [], []
    with ClockSampler(0) as clk:
        for _ in range(args.steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            _, st = P.parse_ids(words, offsets)
            api_ms.append(1e3 * (time.perf_counter() - t0))
            dev_ms.append(P.stats()["ms_device"])
            assert (st == 0).all()
    passes = {f"level{l}": [round(v, 2) for v in P.pass_ms(l)[0]] for l in range(len(levels))}
    if args.fp64_subset > 0:
        # errors on a subset, one batch, against FP64 with the GPU's own masks
        sub = sents[:args.fp64_subset]
        w2, o2, lens = pack_sentences(sub)
        z, st = P.partitions_ids(w2, o2)
        assert (st == 0).all()
        nodes, st = P.parse_ids(w2, o2)
        masks = P.debug_copy(0, "masks")
        isc, osc = P.debug_copy(0, "iscale"), P.debug_copy(0, "oscale")
        mbr = P.debug_copy(1, "mbr")
        P.release()
        t0 = time.time()
        r64 = oracle.OracleRun([oracle.OracleLevel(l) for l in levels], sub, precision=64)
        r64.set_final_masks(masks, isc, osc)
        assert r64.run("parse") == 0
        log(f"FP64 oracle on {len(sub)} sentences: {time.time() - t0:.1f}s")
        ins = r64.chart(1, "inside")
        pscale = r64.partition_scales(1)
        cell_off = r64.cell_off
        root = levels[1].root
        z64 = np.empty(len(sub))
        for i, n in enumerate(lens):
            n = int(n)
            top_root = cell_off[i] + n * (n + 1) // 2 + (n - 1) * n - (n - 1) * (n - 2) // 2
            z64[i] = np.log(ins[top_root, root]) + float(isc[top_root]) + pscale[i]
        rel = np.abs(z.astype(np.float64) - z64) / np.abs(z64)
        s64, y64 = r64.mbr_cells()
        sg = mbr[:, 0].astype(np.float64)
        yg = mbr[:, 1].view(np.int32)
        # cells whose FP64 best marginal is a normal FP32 number (the FP32 path
        # cannot represent smaller values to full precision)
        live = s64 > 1.2e-38
        nonfinite = int((~np.isfinite(sg[live])).sum())
        ok = live & np.isfinite(sg)
        post_err = np.abs(sg[ok] - s64[ok]) / np.abs(s64[ok])
        ref_nodes = r64.trees()
        same_tree = np.mean([np.array_equal(a[:, :3], b[:, :3]) for a, b in
                             zip(_blocks(nodes, lens), _blocks(ref_nodes, lens))])
    value = args.sentences * len(dev_ms) / (sum(dev_ms) / 1e3)
    out = {
        "metric": "MBR sentences/sec, 1.1k-symbol split grammar, sum-product (Real) fine level, len<=40",
        "value": round(value, 2), "unit": "sentences/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(sum(dev_ms) / len(dev_ms), 3), "higher_is_better": True,
        "dtype": "bf16 x bf16 -> f32 (inside binary sums), f32 elsewhere" if tc_on else "f32",
        "data": "synthetic (seeded split grammar and sentences with the published shapes)",
        "config": {"workload": "split-grammar cascade: coarse Viterbi, masks at -9, fine Real inside/outside, "
                               f"MBR trees; {args.sentences} sentences lognormal(mean 23) clipped 1-40",
                   "path": ("fine inside binary sums on tcgen05 tensor cores (BF16 operands, FP32 TMEM "
                            "accumulation); outside pass and the rest FP32 CUDA cores") if tc_on else
                           "FP32 CUDA cores (pair-factored sum-product)" + (f"; tensor cores: {tc_why}" if
                                                                           args.tensor_cores else "")},
        "e2e": {"value": round(args.sentences * len(api_ms) / (sum(api_ms) / 1e3), 2), "unit": "sentences/s"},
        "clocks": clk.summary(), "passes_ms_last_step": passes,
        "errors_vs_fp64": None if args.fp64_subset <= 0 else {
            "sentences": len(sub),
            "log_z_rel_max": float(rel.max()), "log_z_rel_median": float(np.median(rel)),
            "posterior_rel_max": float(post_err.max()), "posterior_rel_median": float(np.median(post_err)),
            "posterior_nonfinite_cells": nonfinite,
            "best_symbol_agreement": float(np.mean(yg[live] == y64[live])),
            "mbr_trees_identical": float(same_tree),
            "cells_compared": int(live.sum()),
            "note": "posterior = per-cell best coarse marginal (the MBR decode input), over cells whose FP64 "
                    "marginal is at least the smallest normal FP32 number; the FP64 oracle uses the GPU's "
                    "coarse masks and scales"},
    }
    print(json.dumps(out), flush=True)
    os.unlink(path)


def _blocks(nodes, lens):
    out, start = [], 0
    for n in lens:
        k = max(2 * int(n) - 1, 0)
        out.append(nodes[start:start + k])
        start += k
    return out


def run_long(args):
    """Long sentences (41-100 words) on a ~2,000-symbol grammar: Viterbi
    cascade throughput per pruning threshold."""
    import torch
    from puck_gb300.parser import CLParser, pack_sentences
    torch.cuda.set_device(0)
    levels, path, sents = long_workload(args.seed, args.long_sentences)
    words, offsets, _ = pack_sentences(sents)
    rows = []
    tune = min(len(sents), 200) if args.tune_sample > 0 else 0
    tw, to, _ = pack_sentences(sents[:tune]) if tune else (None, None, None)
    for thr in (-6.0, -9.0, -12.0):
        P = CLParser(path, max_alloc_size=args.mem_gb << 30, profile=True, max_length=100, prune_threshold=thr)
        tuned = P.autotune(tw, to) if tune else None
        nodes, st = P.parse_ids(words, offsets)  # warm-up
        assert (st == 0).all()
        t0 = time.perf_counter()
        P.parse_ids(words, offsets)
        api = time.perf_counter() - t0
        s = P.stats()
        rows.append({"prune_threshold": thr, "sentences_per_s": round(len(sents) / (s["ms_device"] / 1e3), 2),
                     "e2e_sentences_per_s": round(len(sents) / api, 2), "batches": int(s["batches"]),
                     "fine_work_units": P.level_work(1)[0], "autotuned": tuned,
                     "passes_ms": {f"level{l}": [round(v, 1) for v in P.pass_ms(l)[0]] for l in range(2)}})
        log(f"long, threshold {thr}: {rows[-1]}")
        P.release()
    out = {"metric": "sentences/sec, ~2k-symbol split grammar, len 41-100, Viterbi cascade",
           "unit": "sentences/s", "n_gpus": 1, "dtype": "f32", "data": "synthetic",
           "config": {"workload": f"{levels[1].n_nt + levels[1].n_t} fine symbols, "
                                  f"{int(sum(l.shape[0] for l in levels[1].bucket_rules))} binary rules, "
                                  f"{len(sents)} sentences uniform 41-100"},
           "thresholds": rows}
    print(json.dumps(out), flush=True)
    os.unlink(path)


def run_small(args):
    """The plain method on the small PCFG (64 nonterminals, 32 preterminals,
    20,000 binaries, 512 sentences of 5-20 words): FP32 inside and outside
    plus the Viterbi tree, no pruning -- the configuration the reference's
    own CPU path runs on."""
    import numpy as np
    import torch
    from puck_gb300 import grammar, grz, synth
    from puck_gb300.parser import CLParser, pack_sentences
    torch.cuda.set_device(0)
    g = synth.small_pcfg(0)
    levels = [grammar.compile_level(g, "viterbi")]
    path = os.path.join(tempfile.gettempdir(), f"puck_bench_small_{os.getpid()}.grz")
    grz.write_sequence(path, levels)
    sents = synth.uniform_sentences(args.seed, 512, 5, 20, len(g.words))
    words, offsets, _ = pack_sentences(sents)
    P = CLParser(path, max_alloc_size=8 << 30, profile=True, max_length=20)
    for _ in range(args.warmup):
        P.inside_outside_ids(words, offsets)
        P.parse_ids(words, offsets)
    io_ms, parse_ms = [], []
    for _ in range(args.steps):
        P.inside_outside_ids(words, offsets)
        io_ms.append(P.stats()["ms_device"])
        P.parse_ids(words, offsets)
        parse_ms.append(P.stats()["ms_device"])
    out = {"metric": "sentences/sec, small PCFG (64 NT + 32 PT, 20,000 binaries), len 5-20, no pruning",
           "unit": "sentences/s", "n_gpus": 1, "dtype": "f32", "data": "synthetic",
           "inside_outside": round(512 * len(io_ms) / (sum(io_ms) / 1e3), 1),
           "viterbi_parse": round(512 * len(parse_ms) / (sum(parse_ms) / 1e3), 1),
           "config": {"workload": "512 sentences uniform 5-20 words, Zipf(1.1) word ids"}}
    if args.cpu_sample > 0:
        import oracle
        t0 = time.perf_counter()
        r = oracle.run(levels, sents[:args.cpu_sample], mode="parse")
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": round(min(args.cpu_sample, 512) / dt, 2), "unit": "sentences/s",
                               "cores": os.cpu_count(), "kind": "port",
                               "sample": f"first {min(args.cpu_sample, 512)} sentences, Viterbi parse"}
    print(json.dumps(out), flush=True)
    P.release()
    os.unlink(path)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--sentences", type=int, default=N_SENT)
    ap.add_argument("--cpu-sample", type=int, default=32)
    ap.add_argument("--seed", type=int, default=2)
    ap.add_argument("--mem-gb", type=int, default=160)
    ap.add_argument("--plain-sample", type=int, default=100)
    ap.add_argument("--serve-rates", type=lambda v: [float(x) for x in v.split(",") if x], default="1000,2000,3000")
    ap.add_argument("--serve-sentences", type=int, default=6000)
    ap.add_argument("--serve-mem-gb", type=int, default=32)
    ap.add_argument("--serve-lanes", type=int, default=0, help="server request loops (0: the library's default)")
    ap.add_argument("--tensor-cores", action="store_true",
                    help="mbr config: the fine level's inside binary sums on tcgen05 tensor cores (BF16)")
    ap.add_argument("--config", default="viterbi", choices=["viterbi", "mbr", "long", "small"],
                    help="viterbi: the headline batched/served Viterbi cascade (default); mbr: sum-product "
                         "MBR throughput and errors against FP64; long: long sentences on a ~2k-symbol grammar; "
                         "small: the plain method on the small PCFG")
    ap.add_argument("--fp64-subset", type=int, default=500)
    ap.add_argument("--tune-sample", type=int, default=2000, help="sentences the autotuner parses (0: no tuning)")
    ap.add_argument("--long-sentences", type=int, default=5000)
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.config == "mbr":
        run_mbr(args)
    elif args.config == "long":
        run_long(args)
    elif args.config == "small":
        run_small(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
