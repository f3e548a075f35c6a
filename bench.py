#!/usr/bin/env python3
"""Benchmark of the batched transaction-processing hot path.

Default workload (N=1), the high-contention YCSB-style configuration:
2^24 rows x 10 int32 columns, 32 resident batches of 2^20 transactions x 16
ops, Zipf 0.99 keys over a seeded permutation of the rows, 80% reads / 20%
+1 read-modify-writes, ordered rule (every op on a cell in ascending TID
order, all transactions commit).  A step is one multi-batch call over all 32
batches (CUDA graph or persistent kernel, picked by the autotuner, as are the
kernel tilings per size bucket).  Inputs are far larger than L2 (201 MB of
ops per batch, 640 MB table).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--config zipf|plain|uneven|tpcc|serve]
  python bench.py --impl reference ...   (CPU baseline: the oracle's
                                           multi-threaded serial replay)

Under torchrun every rank drives its own GPU with an independent replica of
the workload (replicas only: no data-path collective); value = all ranks'
transactions / the slowest rank's time.
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

METRIC = "committed txn/s"
DEFAULT_STEPS = {"zipf": 20, "plain": 50, "uneven": 30, "serve": 1, "tpcc": 10, "ycsbe": 10, "gather": 1,
                 "refcuda": 5}
WORKLOAD_TEXT = {
    "zipf": "ycsb-zipf0.99: 2^24 rows x 10 int32, 32 batches x 2^20 txns x 16 ops, 80% read / 20% +1 RMW",
    "plain": "ycsb-uniform: 2^20 rows x 10 int32, 16 batches x 2^16 txns x 10 ops, 50% read / 50% +1 RMW",
    "uneven": "ycsb-uneven: 2^24 rows x 10 int32, 64 batches x 2^U[10,20] txns x U[1,32] ops, zipf U[0.5,0.99], "
              "70% read / 30% +1 RMW",
    "tpcc": "tpcc-shaped order entry: 64 warehouses (10 districts, 30,000 customers, 100,000 stock rows each; "
            "100,000 items), 4 batches x 2^18 txns, 50% new-order (5-15 lines, NURand items, 1% remote) / 50% payment "
            "(NURand customers, 15% remote, 60% by last name, int64 cents), 9 tables, int32/int64 columns",
    "ycsbe": "ycsb-e: 2^20 rows x 3 int32 (the reference YCSB schema's int attributes), 16 batches x 2^16 txns, "
             "each 9 scans of rows [r, r+2) (every int column read) + 1 insert, zipf0.99 rows",
    "refcuda": "the reference's own CUDA path (cuda/src, unchanged, sm_103a) on YCSB_A batches: 2^20 rows "
               "(3 int, 3 double, 4 string columns), 2^16 txns x 10 distinct uniform rows (5 selects, 5 updates)",
    "serve": "serving: 256 Poisson client streams, seeded 50/50 blend of zipf0.99 YCSB txns (2^24 rows x 10 int32, "
             "16 ops, 80/20) and tpcc-shaped new-order/payment txns (W=64, 9 tables, inserts), offered load swept "
             "1M-50M txn/s, 250 us batch deadline, 4 GB read/write-set budget, aborts re-queued",
}
# algorithmic bytes per kernel launch, from the batch's counters
KERNEL_BYTES = {  # st["key_bytes"]: 8, or 4 for batches loaded with 32-bit keys
    "mark": lambda st: (8 + st["key_bytes"]) * st["ops"],
    "ids": lambda st: 20 * st["touched_words"] + 32 * st["contended_cells"],  # id scan + pre-batch values
    "classify": lambda st: (20 + st["key_bytes"]) * st["ops"],
    "sort_pass0": lambda st: 16 * st["contended_ops"],
    "sort_pass1": lambda st: 16 * st["contended_ops"],
    "sort_pass2": lambda st: 16 * st["contended_ops"],
    "sort_pass3": lambda st: 16 * st["contended_ops"],
    "apply": lambda st: 16 * st["contended_ops"] + 12 * st["contended_cells"],
    "insert": lambda st: st.get("insert_bytes", 0),
    "finish": lambda st: 12 * st["touched_words"],
}
def kernels_per_batch(n_ops, has_payload):
    """Kernels one batch launches under the ordered rule: mark, ids, dbase,
    classify, one radix pass per 8 bits of the largest possible contended id
    (n_ops - 1), apply, the insert prefix and insert (only with a payload),
    finish."""
    passes = 1
    while passes < 4 and ((max(n_ops, 1) - 1) >> (8 * passes)) != 0:
        passes += 1
    return 4 + passes + 1 + (2 if has_payload else 0) + 1


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def reduce_max(x, world):
    """Max over ranks (identity at world 1)."""
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(x)], dtype=torch.float64)
    if dist.get_backend() == "nccl":
        t = t.cuda()
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


class ClockSampler:
    """nvidia-smi samples of SM clock / throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "50", "-i", str(self.device)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.th.join(timeout=2)
        sm = [float(r[1]) for r in self.rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows if len(r) >= 9 for i in range(4) if r[5 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(sm)}


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per unit of work,
# from one ncu capture of each kernel on one batch of the same workload
# (profiles/batch_kernels_zipf.md, profiles/k_mark_insert_tpcc.md,
# profiles/k_insert_tpcc.md);
# a launch's traffic is this figure times the units it processed
MEASURED_TRAFFIC = {
    ("zipf", "classify"): (37.4, "ops"),  # 32-bit keys
    ("zipf", "mark"): (13.3, "ops"),  # 32-bit keys
    ("zipf", "apply"): (30.3, "contended_ops"),
    ("zipf", "ids"): (6.9, "ops"),  # k_ids + k_dbase
    ("tpcc", "insert"): (55.5, "ops"),  # 32-bit keys
    ("tpcc", "mark"): (15.7, "ops"),  # 32-bit keys
}


# mark's L2 atomic and reduction sectors per op (lts__t_sectors_srcunit_tex_op_atom / _red
# over the batch's ops, from the same capture as MEASURED_TRAFFIC)
MEASURED_ATOMICS = {"zipf": (0.760, 0.581)}


def random_access_roof(G, device, sh, st, avg, config):
    """The random-access roofline of mark and classify: their random accesses
    at this GPU's measured rates (ltp_probe_random_access over arrays of the
    workload's table and conflict-word sizes) give a floor time; frac = floor
    over the measured kernel time."""
    table_b = sh["rows"] * sh["cols"] * 4
    words_b = max(4096, (sh["rows"] * sh["cols"] + 31) // 32 * 16)  # conflict words (mark's atomics)
    view_b = max(4096, (sh["rows"] * sh["cols"] + 31) // 32 * 8)  # their compact view (classify's reads)
    pr = G.lib.probe_random_access
    c = {"load_table": pr(device, table_b, G.lib.PROBE_LOAD), "load_views": pr(device, view_b, G.lib.PROBE_LOAD),
         "atomic_words": pr(device, words_b, G.lib.PROBE_ATOMIC),
         "reduce_words": pr(device, words_b, G.lib.PROBE_REDUCE)}
    out = {"ceilings_per_s": c, "array_bytes": {"table": table_b, "words": words_b, "views": view_b}}
    ops, unc = st["ops"], st["ops"] - st["contended_ops"]
    floor = ops / c["load_views"] + unc / c["load_table"]
    out["classify"] = {"random_reads": {"views": ops, "cells": unc}, "floor_ms": floor * 1e3,
                       "ms": avg["classify"], "frac": floor * 1e3 / avg["classify"]}
    if config in MEASURED_ATOMICS:
        a, r = MEASURED_ATOMICS[config]
        floor = a * ops / c["atomic_words"] + r * ops / c["reduce_words"]
        out["mark"] = {"atomics": a * ops, "reductions": r * ops, "floor_ms": floor * 1e3, "ms": avg["mark"],
                       "frac": floor * 1e3 / avg["mark"]}
    return out


def measured_traffic(config, kernel, stats):
    t = MEASURED_TRAFFIC.get((config, kernel))
    return None if t is None else t[0] * stats[t[1]]


def gen_batches(config, nb, rank):
    from ltpmg_gb300 import workloads as W

    return [W.generate(config, b, rank=rank) for b in range(nb)]


def cpu_baseline(config, host, budget_s=12.0):
    """Single-core serial replay (the oracle port) over whole batches until
    the time budget is spent; returns txn/s and what was sampled."""
    import numpy as np

    from ltpmg_gb300 import workloads as W

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    L = O.lib()
    sh = W.SHAPES[config]
    tab = O.table_init(sh["seed"], sh["rows"], sh["cols"])
    done_txns, done, t_used = 0, 0, 0.0
    for tf, keys, opw, n, _ in host:
        out = np.zeros(len(keys), np.int32)
        commit = np.zeros(n, np.uint8)
        t0 = time.perf_counter()
        rc = L.ltpo_replay(0, sh["rows"], sh["cols"], tab.ctypes.data, n, tf.ctypes.data, keys.ctypes.data,
                           opw.ctypes.data, commit.ctypes.data, out.ctypes.data)
        t_used += time.perf_counter() - t0
        assert rc == 0
        done += 1
        done_txns += n
        if t_used >= budget_s:
            break
    out = {"value": done_txns / t_used, "unit": "txn/s", "cores": 1, "kind": "port",
           "sample": f"{done} whole batch(es), {done_txns} txns, serial replay (ordered rule), {t_used:.1f} s"}
    gen = reference_generator_rate(config)
    if gen and "value" in gen:
        # (i) the reference's own generator/scheduler path, then (i)+(ii):
        # generating a transaction and replaying it, back to back
        out["generator"] = gen
        out["generator_plus_replay"] = {"value": 1.0 / (1.0 / gen["value"] + 1.0 / out["value"]), "unit": "txn/s",
                                        "cores": f"{gen['cores']} (generator) + 1 (replay)"}
    elif gen:
        out["generator"] = gen
    return out


def reference_generator_rate(config):
    """The reference's own host generator (Txn_Generator + Query::generate_txn,
    src/txn_generator.cpp:601-673, src/query.cpp:270-311) timed on this
    machine's host cores with hardware_concurrency() threads, as the reference
    runs it, at its closest settings to the workload (YCSB_A; its "zipf" is a
    100-rank truncated law, src/random.cpp:105-161); None when it was not
    built here."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    if not os.path.exists(O.REF_GEN):
        return None
    settings = {"zipf": ("YCSB_A", 16, 1 << 18, "zipf", 0.99), "uneven": ("YCSB_A", 16, 1 << 18, "zipf", 0.75),
                "plain": ("YCSB_A", 1, 1 << 16, "unif", 0.0)}.get(config)
    if settings is None:
        return None
    try:
        r = O.ref_gen_time(*settings, reps=2)
    except Exception as e:  # reported, not fatal: the baseline is informational
        return {"unavailable": str(e)[:200]}
    sec = min(r["seconds"])
    return {"value": r["txns"] / sec, "unit": "txn/s", "cores": r["threads"], "kind": "reference",
            "sample": f"{r['benchmark']} {r['txns']} txns over {r['rows']} rows, {r['distribution']} "
                      f"{r['zipf_config']}: Query::generate_txn, best of {len(r['seconds'])} calls ({sec:.3f} s)"}


def oracle_batches(config, nb, seed=None):
    """Batches of the workload drawn by the oracle's own generator
    (ltpo_gen_ycsb_batch), fingerprint-equal to the library's, so that the
    reference arm never loads the product library."""
    from ltpmg_gb300 import workloads as W  # shapes only: importing it loads no library

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    sh = W.SHAPES[config]
    s = sh["seed"] if seed is None else seed
    out = []
    for b in range(nb):
        n, omin, omax, rf, th = W.batch_params(config, b, s)
        tf, keys, opw = O.gen_ycsb_batch(O.ycsb_params(s, sh["rows"], sh["cols"], omin, omax, rf, th), b, n)
        out.append((tf, keys, opw, n))
    return out


def product_library_mapped():
    """Is libltpmg_gb300.so mapped into this process?"""
    try:
        return "libltpmg_gb300" in open("/proc/self/maps").read()
    except OSError:
        return False


def run_reference(args, config):
    """The reference arm: the reference's execution rule on the host cores.
    The reference has no executable CPU path for execution (execute_on_CPU is
    never called, cuda/src/gpulauncher.cu:771), so the oracle's
    cell-partitioned serial replay on every host thread stands in for it.
    Each step replays one whole batch of the workload (the same batches the
    GPU arm runs: for the default workload 2^20 transactions x 16 ops) on a
    table that carries every earlier step's effects.  Inputs come from the
    oracle's generator; the product library is never loaded."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import numpy as np

    from ltpmg_gb300 import workloads as W

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    threads = os.cpu_count() or 1
    sh = W.SHAPES[config]
    nb = min(sh["batches"], 4 if config == "zipf" else 8)
    host = oracle_batches(config, nb)
    tab = O.table_init(sh["seed"], sh["rows"], sh["cols"])
    L = O.lib()

    def step(i):
        tf, k, w, n = host[i % len(host)]
        commit = np.zeros(n, np.uint8)
        out = np.zeros(len(k), np.int32)
        rc = L.ltpo_replay_r0_mt(sh["rows"], sh["cols"], tab.ctypes.data, n, tf.ctypes.data, k.ctypes.data,
                                 w.ctypes.data, commit.ctypes.data, out.ctypes.data, threads)
        assert rc == 0
        return n

    for i in range(args.warmup):
        step(i)
    t0 = time.perf_counter()
    txns = sum(step(args.warmup + i) for i in range(args.steps))
    dt = time.perf_counter() - t0
    assert not product_library_mapped(), "the reference arm must not load the product library"
    value = txns / dt
    sizes = sorted({h[3] for h in host})
    line = {"metric": METRIC, "value": value, "unit": "txn/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic (seeded generator)",
            "config": {"workload": WORKLOAD_TEXT[config],
                       "step": "one whole batch of the workload (" + "/".join(str(x) for x in sizes) + " txns), "
                               f"cycling over its first {nb} batches",
                       "l2": "inputs larger than L2", "same_config": True},
            "impl": "reference",
            "cpu_baseline": {"value": value, "unit": "txn/s", "cores": threads, "kind": "port",
                             "sample": f"{args.steps} whole batches, cell-partitioned serial replay (ordered rule) "
                                       f"on {threads} threads; inputs from the oracle's generator"},
            "e2e": {"value": value, "unit": "txn/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args, config):
    import numpy as np
    import torch

    import ltpmg_gb300 as G
    from ltpmg_gb300 import autotune as AT
    from ltpmg_gb300 import workloads as W

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    sh = W.SHAPES[config]
    nb = args.batches or sh["batches"]
    host = gen_batches(config, nb, rank)
    ctx = G.Context(device=local, stage_timing=True)
    t = ctx.create_table(sh["rows"], sh["cols"])
    ctx.fill_seeded(t, sh["seed"] + rank)
    dev = []
    for tf, keys, opw, n, opt in host:
        b = ctx.batch(n, len(keys))
        # row ids below 2^32 load as 32-bit keys (the reference's row ids are 32-bit)
        b.load(None if opt else tf, keys.astype(np.uint32) if sh["rows"] <= (1 << 32) else keys, opw, ops_per_txn=opt)
        dev.append(b)
    ctx.sync()

    # autotuning (untimed): tilings per size bucket, then the multi-batch mode
    ctx.set_stage_timing(False)  # tune what the timed region runs: no event nodes
    # resident batches run from captured graphs: candidates are timed that way
    tiles = fixed_tiles(ctx, dev, args.tiles) if args.tiles else AT.tune_buckets(ctx, dev, reps=3, copies=4)
    if args.mode == "auto":
        mode, mode_ms = AT.tune_mode(ctx, dev)
    else:
        mode = {"graph": G.MODE_GRAPH, "persistent": G.MODE_PERSISTENT, "stream": G.MODE_STREAM}[args.mode]
        mode_ms = {}
    mode_name = {G.MODE_STREAM: "stream", G.MODE_GRAPH: "graph", G.MODE_PERSISTENT: "persistent"}[mode]
    if args.tuning_out:
        AT.save(args.tuning_out, tiles, mode_name)

    stream = torch.cuda.ExternalStream(ctx.stream)

    def timed_region(steps):
        for _ in range(args.warmup):
            ctx.execute_many(dev, mode=mode)
        ctx.sync()
        barrier(world)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            ctx.execute_many(dev, mode=mode)
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1)

    # headline: no per-kernel events in the launch sequence
    ctx.set_stage_timing(False)
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.15)
    ms = timed_region(args.steps)
    clk = clocks.stop()
    ms = reduce_max(ms, world)
    for b in dev:
        b.finish()
    # per-kernel times: the same steps again with an event after every kernel
    # (event nodes inside the captured graph); each batch's last run is read
    ctx.set_stage_timing(True)
    ms_timed = timed_region(max(1, min(args.steps, 5)))
    stats = [b.finish().as_dict() for b in dev]
    ctx.set_stage_timing(False)
    txns_per_step = sum(h[3] for h in host)
    ops_per_step = sum(len(h[1]) for h in host)
    value = args.steps * txns_per_step * world / (ms / 1e3)

    e2e = None
    if not args.no_e2e:
        # end to end through the C ABI's pipeline: every step copies one batch
        # from pinned host memory, executes it and copies its commit vector and
        # op values back into pinned host memory; copies of neighbouring steps
        # overlap execution (3-deep pipeline, three streams)
        depth = 3
        n_e2e = min(64, max(32, args.steps))
        hb = [max(range(nb), key=lambda i: host[i][3])]
        hb.append((hb[0] + 1) % nb)
        # row ids below 2^32 travel as 32-bit keys (ltp_pipe_submit32)
        key_t, key_b = (np.uint32, 4) if sh["rows"] <= (1 << 32) else (np.uint64, 8)
        pins = []
        for i in hb:
            tf, keys, opw, n, opt = host[i]
            pk, pw = G.PinnedArray((len(keys),), key_t), G.PinnedArray((len(opw),), np.uint32)
            pk.array[:] = keys
            pw.array[:] = opw
            ptf = G.PinnedArray((len(tf),), np.uint32)
            ptf.array[:] = tf
            pins.append((ptf, pk, pw, n, opt))
        maxn = max(p[3] for p in pins)
        maxops = max(len(p[1].array) for p in pins)
        outs = [(G.PinnedArray((maxn,), np.uint8), G.PinnedArray((maxops,), np.int32)) for _ in range(depth)]
        pipe = G.Pipe(ctx, depth, maxn, maxops)
        h2d = d2h = 0

        def e2e_submit(i):
            ptf, pk, pw, n, opt = pins[i % 2]
            pc, pv = outs[i % depth]
            tk = pipe.submit(None if opt else ptf.array, pk.array, pw.array, pc.array[:n], pv.array[:len(pk.array)],
                             ops_per_txn=opt)
            return tk, n, len(pk.array), opt

        for i in range(depth):
            pipe.wait(e2e_submit(i)[0])
        ctx.sync()
        barrier(world)
        t0 = time.perf_counter()
        e2e_txns, inflight = 0, []
        for i in range(n_e2e):
            tk, n, nops, opt = e2e_submit(i)
            inflight.append(tk)
            if len(inflight) >= depth:
                pipe.wait(inflight.pop(0))
            e2e_txns += n
            h2d += (key_b + 4) * nops + (0 if opt else 4 * (n + 1))
            d2h += 4 * nops + n
        for tk in inflight:
            pipe.wait(tk)
        e2e_s = reduce_max(time.perf_counter() - t0, world)
        pipe.close()
        e2e = {"value": e2e_txns * world / e2e_s, "unit": "txn/s", "h2d_bytes_per_step": h2d // n_e2e,
               "d2h_bytes_per_step": d2h // n_e2e, "steps": n_e2e,
               "note": "one batch per step through ltp_pipe (3 slots): H2D, execute, D2H overlapped across steps; "
                       f"{8 * key_b}-bit keys"}

    if rank != 0:
        return
    peak, peak_kind = load_peaks()
    key_bytes = 4 if sh["rows"] <= (1 << 32) else 8  # the batches were loaded with 32-bit keys
    alg = W.algorithmic_bytes(ops_per_step, txns_per_step, key_bytes)
    step_ms = ms / args.steps
    roof = {"bound": "hbm", "peak": peak, "unit": "GB/s", "peak_kind": peak_kind,
            "kernel_timing_pass_ms_per_step": ms_timed / max(1, min(args.steps, 5)),
            "pipeline": {"algorithmic_bytes_per_step": alg, "avg_step_ms": step_ms,
                         "achieved": alg / (step_ms / 1e3) / 1e9, "frac": alg / (step_ms / 1e3) / 1e9 / peak}}
    mean_stats = {k: sum(s[k] for s in stats) / len(stats) for k in ("ops", "touched_words", "contended_cells",
                                                                     "contended_ops")}
    mean_stats["key_bytes"] = key_bytes
    if mode != G.MODE_PERSISTENT:
        avg = {name: sum(s["ms_stage"][name] for s in stats) / len(stats) for name in KERNEL_BYTES}
        dom = max(avg, key=avg.get)
        dom_bytes = KERNEL_BYTES[dom](mean_stats)
        achieved = dom_bytes / (avg[dom] / 1e3) / 1e9
        traffic_b = measured_traffic(config, dom, mean_stats)
        roof.update({"kernel": dom, "achieved": achieved, "frac": achieved / peak, "traffic": traffic_b,
                     "algorithmic_bytes_per_launch": dom_bytes, "avg_launch_ms": avg[dom], "kernel_ms": avg,
                     "random_access": random_access_roof(G, local, sh, mean_stats, avg, config)})
    else:
        roof.update({"kernel": "k_persist (whole pipeline, one launch per step)", "achieved":
                     roof["pipeline"]["achieved"], "frac": roof["pipeline"]["frac"], "traffic": None,
                     "algorithmic_bytes_per_launch": alg, "avg_launch_ms": step_ms})
    launches = args.steps * (1 if mode == G.MODE_PERSISTENT else
                             sum(kernels_per_batch(len(h[1]), False) for h in host))
    line = {"metric": METRIC, "value": value, "unit": "txn/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic (seeded generator)",
            "config": {"workload": WORKLOAD_TEXT[config], "batches_per_step": nb, "txns_per_step": txns_per_step,
                       "rule": "ordered (ascending TID per cell, all commit)", "mode": mode_name,
                       "mode_ms": {str(k): v for k, v in mode_ms.items()},
                       "tuning": {str(k): f"{v['block']}x{v['ipt']}" + ("w64" if v.get("word_bits") == 64 else "") + ("+precheck" if v.get("flags") else "")
                                  for k, v in tiles.items()},
                       "l2": "inputs larger than L2", "parallelism": f"replicas x{world}"},
            "gpu_launches": launches, "roofline": roof, "clocks": clk, "e2e": e2e,
            "contention": {"contended_ops_per_batch": mean_stats["contended_ops"],
                           "contended_cells_per_batch": mean_stats["contended_cells"]}}
    if world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(config, host)
    if config == "zipf" and world == 1 and not args.no_serving:
        # the serving half of the metric (p50/p99/p99.9 and serving vs the
        # plain path), after the headline measurement, on a fresh context
        for b in dev:
            b.free()
        ctx.close()
        line["serving"] = serving_measure(args, local, rank, point_s=0.5)
    print(json.dumps(line), flush=True)


def fixed_tiles(ctx, dev, spec):
    from ltpmg_gb300 import autotune as AT

    import ltpmg_gb300 as G

    # BLOCKxIPT[w64][+precheck], e.g. 512x4, 256x2w64+precheck
    base, _, opt = spec.partition("+")
    base, _, wb = base.partition("w")
    blk, ipt = (int(x) for x in base.split("x"))
    word_bits = int(wb) if wb else 32
    flags = G.lib.TUNE_MARK_PRECHECK if opt == "precheck" else 0
    out = {}
    for b in dev:
        k = AT.bucket_of(b.n_ops)
        ctx.set_tuning(k, blk, ipt, word_bits=word_bits, flags=flags)
        out[k] = {"block": blk, "ipt": ipt, "word_bits": word_bits, "flags": flags}
    return out


def tpcc_setup(seed_offset=0):
    import ltpmg_gb300 as G
    from ltpmg_gb300 import workloads as W

    sh = W.SHAPES["tpcc"]
    return G.Tpcc(sh["warehouses"], seed=sh["seed"] + seed_offset), sh


def tpcc_cpu_tables(g, sample_inserts):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    tabs = []
    for t in range(9):
        n_cols, mask, rows = g.table(t)
        tabs.append((g.initial(t, rows + int(sample_inserts[t])), rows, mask))
    return O.TablesDB(tabs)


class TpccLoad:
    """The order-entry workload for the payload runner: 9 tables, batches of
    new-order / payment transactions with inserts."""
    config = "tpcc"
    dtype = "int32/int64"

    def __init__(self, rank):
        self.g, self.sh = tpcc_setup(rank)
        self.n_batches = self.sh["batches"]

    def batch(self, b):
        tf, keys, opw, pay, n_no, ins = self.g.gen(b, self.sh["batch"])
        return tf, keys, opw, pay, len(tf) - 1, ins

    def create_tables(self, ctx, extra):
        return self.g.create_tables(ctx, extra)

    def table_names(self):
        import ltpmg_gb300 as G

        return G.TPCC_TABLES

    def alg_bytes(self, h):
        from ltpmg_gb300 import workloads as W

        return W.tpcc_algorithmic_bytes(self.g, h[1], h[2], h[4], key_bytes=4)

    def insert_bytes(self, h):
        from ltpmg_gb300 import workloads as W

        return W.tpcc_insert_bytes(self.g, h[1], h[2], key_bytes=4)

    def cpu_tables(self, sample_inserts):
        return tpcc_cpu_tables(self.g, sample_inserts)


class YcsbeLoad:
    """The YCSB-E workload (9 scans of two rows + one insert per
    transaction, as the compatibility layer expands the reference's YCSB_E
    query) for the payload runner: one 3-column int32 table."""
    config = "ycsbe"
    dtype = "int32"

    def __init__(self, rank):
        from ltpmg_gb300 import workloads as W

        self.rank = rank
        self.sh = W.SHAPES["ycsbe"]
        self.n_batches = self.sh["batches"]

    def batch(self, b):
        from ltpmg_gb300 import workloads as W

        return W.ycsbe_batch(b, rank=self.rank)

    def create_tables(self, ctx, extra):
        sh = self.sh
        t = ctx.create_table(sh["rows"], sh["cols"], rows_cap=sh["rows"] + int(extra[0]))
        ctx.fill_seeded(t, sh["seed"] + self.rank)
        return [t]

    def table_names(self):
        return ["ycsb"]

    def alg_bytes(self, h):
        from ltpmg_gb300 import workloads as W

        return W.ycsbe_algorithmic_bytes(len(h[1]), h[4], int(h[5][0]), self.sh["cols"])

    def insert_bytes(self, h):
        from ltpmg_gb300 import workloads as W

        return W.ycsbe_insert_bytes(len(h[1]), int(h[5][0]), self.sh["cols"])

    def cpu_tables(self, sample_inserts):
        import numpy as np

        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O

        sh = self.sh
        data = np.zeros((sh["cols"], sh["rows"] + int(sample_inserts[0])), np.int32)
        data[:, :sh["rows"]] = O.table_init(sh["seed"] + self.rank, sh["rows"], sh["cols"])
        return O.TablesDB([(data, sh["rows"])])


def payload_load(config, rank):
    return TpccLoad(rank) if config == "tpcc" else YcsbeLoad(rank)


def tpcc_cpu_baseline(wl, host, budget_s=12.0, threads=0, slice_txns=1 << 16):
    """Replay of whole-batch slices of the workload by the oracle port; only
    the replay call is timed."""
    import numpy as np

    sample, t_used, done = [], 0.0, 0
    for tf, keys, opw, pay, n, ins in host:
        for lo in range(0, n, slice_txns):
            hi = min(n, lo + slice_txns)
            a, b = int(tf[lo]), int(tf[hi])
            sample.append(((tf[lo:hi + 1] - tf[lo]).astype(np.uint32), keys[a:b], opw[a:b], pay, hi - lo))
    # room for every slice's inserts (at most one row per op)
    per = np.zeros(9, np.int64)
    for tf, keys, opw, pay, n in sample:
        per += np.bincount(((opw >> 8) & 15)[(opw & 3) == 2], minlength=16)[:9]
    db = wl.cpu_tables(per)
    for tf, keys, opw, pay, n in sample:
        t0 = time.perf_counter()
        db.replay(0, tf, keys, opw, pay, threads=threads)
        t_used += time.perf_counter() - t0
        done += n
        if t_used >= budget_s:
            break
    return done / t_used, done, t_used


def run_payload(args, config):
    """Resident batches with inserts (the order-entry or the YCSB-E
    workload): device throughput, end to end with payload, roofline, CPU
    baseline."""
    import numpy as np
    import torch

    import ltpmg_gb300 as G
    from ltpmg_gb300 import autotune as AT
    from ltpmg_gb300 import workloads as W

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    wl = payload_load(config, rank)
    nb = args.batches or wl.n_batches
    host = [wl.batch(b) for b in range(nb)]
    # every execution appends its inserts: size the insert tables for all
    # executions this run makes (tuning, warm-up, timed steps, the kernel
    # timing pass and the end-to-end pass)
    timing_steps = max(1, min(args.steps, 5))
    n_e2e = max(32, min(64, args.steps))
    execs_all = (6 if args.mode == "auto" else 0) + args.warmup * 2 + args.steps + timing_steps
    per_batch = np.max([h[5] for h in host], axis=0)
    # tuning: ~17 executions of the first batch, then 4 candidates x 3 runs of the list
    extra = per_batch * (execs_all * nb + (0 if args.tiles else 40 + 12 * nb) + (0 if args.no_e2e else n_e2e + 3))
    ctx = G.Context(device=local, stage_timing=True)
    ctx_tables = wl.create_tables(ctx, extra)
    dev = []
    for tf, keys, opw, pay, n, _ in host:
        b = ctx.batch(n, len(keys))
        b.load(tf, keys.astype(np.uint32), opw)  # row ids and payload offsets are below 2^32
        b.load_payload(pay)
        dev.append(b)
    ctx.sync()
    ctx.set_stage_timing(False)  # tune what the timed region runs: no event nodes
    tiles = fixed_tiles(ctx, dev, args.tiles) if args.tiles else AT.tune_buckets(ctx, dev[:1], reps=1)
    if not args.tiles:  # the single-batch choice, checked on the batch list itself
        tiles = {k: AT.refine_pipeline(ctx, dev, v) for k, v in tiles.items()}
    if args.mode == "auto":
        mode, mode_ms = AT.tune_mode(ctx, dev)
    else:
        mode = {"graph": G.MODE_GRAPH, "persistent": G.MODE_PERSISTENT, "stream": G.MODE_STREAM}[args.mode]
        mode_ms = {}
    mode_name = {G.MODE_STREAM: "stream", G.MODE_GRAPH: "graph", G.MODE_PERSISTENT: "persistent"}[mode]
    stream = torch.cuda.ExternalStream(ctx.stream)

    def timed_region(steps):
        for _ in range(args.warmup):
            ctx.execute_many(dev, mode=mode)
        ctx.sync()
        barrier(world)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            ctx.execute_many(dev, mode=mode)
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1)

    ctx.set_stage_timing(False)
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.15)
    ms = timed_region(args.steps)
    clk = clocks.stop()
    ms = reduce_max(ms, world)
    for b in dev:
        b.finish()
    ctx.set_stage_timing(True)
    ms_timed = timed_region(timing_steps)
    stats = [b.finish().as_dict() for b in dev]
    ctx.set_stage_timing(False)
    txns_per_step = sum(h[4] for h in host)
    ops_per_step = sum(len(h[1]) for h in host)
    value = args.steps * txns_per_step * world / (ms / 1e3)

    e2e = None
    if not args.no_e2e:
        # end to end: one batch per step through the 3-slot pipeline (payload too)
        depth = 3
        pins = []
        for tf, keys, opw, pay, n, _ in host[:2]:
            arrs = []
            for a, dt in ((tf, np.uint32), (keys, np.uint32), (opw, np.uint32), (pay, np.int32)):
                p = G.PinnedArray((len(a),), dt)
                p.array[:] = a
                arrs.append(p)
            pins.append((arrs, n))
        maxn = max(p[1] for p in pins)
        maxops = max(len(p[0][1].array) for p in pins)
        outs = [(G.PinnedArray((maxn,), np.uint8), G.PinnedArray((maxops,), np.int32)) for _ in range(depth)]
        pipe = G.Pipe(ctx, depth, maxn, maxops)
        h2d = d2h = 0

        def e2e_submit(i):
            (ptf, pk, pw, pp), n = pins[i % len(pins)]
            pc, pv = outs[i % depth]
            tk = pipe.submit(ptf.array, pk.array, pw.array, pc.array[:n], pv.array[:len(pk.array)], payload=pp.array)
            return tk, n, len(pk.array), len(pp.array)

        for i in range(depth):
            pipe.wait(e2e_submit(i)[0])
        ctx.sync()
        barrier(world)
        t0 = time.perf_counter()
        e2e_txns, inflight = 0, []
        for i in range(n_e2e):
            tk, n, nops, npay = e2e_submit(i)
            inflight.append(tk)
            if len(inflight) >= depth:
                pipe.wait(inflight.pop(0))
            e2e_txns += n
            h2d += 8 * nops + 4 * (n + 1) + 4 * npay  # 32-bit keys
            d2h += 4 * nops + n
        for tk in inflight:
            pipe.wait(tk)
        e2e_s = reduce_max(time.perf_counter() - t0, world)
        pipe.close()
        e2e = {"value": e2e_txns * world / e2e_s, "unit": "txn/s", "h2d_bytes_per_step": h2d // n_e2e,
               "d2h_bytes_per_step": d2h // n_e2e, "steps": n_e2e,
               "note": "one batch (+ insert payload) per step through ltp_pipe (3 slots), copies overlapped"}
    if rank != 0:
        return
    peak, peak_kind = load_peaks()
    alg = sum(wl.alg_bytes(h) for h in host)  # 32-bit keys
    step_ms = ms / args.steps
    roof = {"bound": "hbm", "peak": peak, "unit": "GB/s", "peak_kind": peak_kind,
            "kernel_timing_pass_ms_per_step": ms_timed / timing_steps,
            "pipeline": {"algorithmic_bytes_per_step": alg, "avg_step_ms": step_ms,
                         "achieved": alg / (step_ms / 1e3) / 1e9, "frac": alg / (step_ms / 1e3) / 1e9 / peak}}
    mean_stats = {k: sum(s[k] for s in stats) / len(stats) for k in ("ops", "touched_words", "contended_cells",
                                                                     "contended_ops")}
    mean_stats["insert_bytes"] = sum(wl.insert_bytes(h) for h in host) / len(host)
    mean_stats["key_bytes"] = 4
    if mode != G.MODE_PERSISTENT:
        avg = {nm: sum(s["ms_stage"][nm] for s in stats) / len(stats) for nm in KERNEL_BYTES}
        dom = max(avg, key=avg.get)
        dom_bytes = KERNEL_BYTES[dom](mean_stats)
        achieved = dom_bytes / (avg[dom] / 1e3) / 1e9
        roof.update({"kernel": dom, "achieved": achieved, "frac": achieved / peak,
                     "traffic": measured_traffic(config, dom, mean_stats),
                     "algorithmic_bytes_per_launch": dom_bytes, "avg_launch_ms": avg[dom], "kernel_ms": avg})
    else:
        roof.update({"kernel": "k_persist (whole pipeline, one launch per step)",
                     "achieved": roof["pipeline"]["achieved"], "frac": roof["pipeline"]["frac"], "traffic": None,
                     "algorithmic_bytes_per_launch": alg, "avg_launch_ms": step_ms})
    launches = args.steps * (1 if mode == G.MODE_PERSISTENT else
                             sum(kernels_per_batch(len(h[1]), True) for h in host))
    rows = {wl.table_names()[t]: ctx.table_rows(tid) for t, tid in enumerate(ctx_tables)}
    line = {"metric": METRIC, "value": value, "unit": "txn/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": wl.dtype, "data": "synthetic (seeded generator)",
            "config": {"workload": WORKLOAD_TEXT[config], "batches_per_step": nb, "txns_per_step": txns_per_step,
                       "ops_per_step": ops_per_step, "rule": "ordered (ascending TID per cell, all commit)",
                       "mode": mode_name, "mode_ms": {str(k): v for k, v in mode_ms.items()},
                       "tuning": {str(k): f"{v['block']}x{v['ipt']}" + ("w64" if v.get("word_bits") == 64 else "") + ("+precheck" if v.get("flags") else "")
                                  for k, v in tiles.items()},
                       "l2": "inputs larger than L2", "parallelism": f"replicas x{world}"},
            "gpu_launches": launches, "roofline": roof, "clocks": clk, "e2e": e2e,
            "contention": {"contended_ops_per_batch": mean_stats["contended_ops"],
                           "contended_cells_per_batch": mean_stats["contended_cells"]},
            "table_rows_after": rows}
    if world == 1 and not args.no_cpu_baseline:
        v, done, t_used = tpcc_cpu_baseline(wl, host[:1])
        line["cpu_baseline"] = {"value": v, "unit": "txn/s", "cores": 1, "kind": "port",
                                "sample": f"{done} txns of batch 0 in slices of 2^16, serial replay of the "
                                          f"{len(ctx_tables)} table(s) (ordered rule), {t_used:.1f} s"}
    print(json.dumps(line), flush=True)


def run_reference_payload(args, config):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import numpy as np

    wl = payload_load(config, 0)
    threads = os.cpu_count() or 1
    tf, keys, opw, pay, n, ins = wl.batch(0)
    slice_txns = 1 << 16
    slices = []
    for lo in range(0, len(tf) - 1, slice_txns):
        hi = min(len(tf) - 1, lo + slice_txns)
        a, b = int(tf[lo]), int(tf[hi])
        slices.append(((tf[lo:hi + 1] - tf[lo]).astype(np.uint32), keys[a:b], opw[a:b], hi - lo))
    n_steps = args.warmup + args.steps
    per = np.zeros(9, np.int64)
    for i in range(n_steps):
        w = slices[i % len(slices)][2]
        per += np.bincount(((w >> 8) & 15)[(w & 3) == 2], minlength=16)[:9]
    db = wl.cpu_tables(per)

    def step(i):
        tfs, k, w, n = slices[i % len(slices)]
        db.replay(0, tfs, k, w, pay, threads=threads)
        return n

    for i in range(args.warmup):
        step(i)
    t0 = time.perf_counter()
    txns = sum(step(args.warmup + i) for i in range(args.steps))
    dt = time.perf_counter() - t0
    value = txns / dt
    line = {"metric": METRIC, "value": value, "unit": "txn/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": wl.dtype, "data": "synthetic (seeded generator)",
            "config": {"workload": WORKLOAD_TEXT[config], "step": f"up to {slice_txns} txns of the workload",
                       "l2": "inputs larger than L2"},
            "impl": "reference",
            "cpu_baseline": {"value": value, "unit": "txn/s", "cores": threads, "kind": "port",
                             "sample": f"{args.steps} slices of up to {slice_txns} txns of batch 0, "
                                       f"{len(wl.table_names())} table(s), cell-partitioned replay on {threads} "
                                       "threads (inserts split by table)"},
            "e2e": {"value": value, "unit": "txn/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def serving_measure(args, local, rank, point_s):
    """The serving half of the metric, on one GPU.  Two request pools over
    device-resident tables: the Zipf 0.99 YCSB transactions of the headline
    workload (batch 0, 2^20 transactions x 16 ops, 2^24 x 10 int32 table)
    and the seeded 50/50 blend of 2^18 of those with 2^18 TPC-C-shaped
    order-entry transactions (W=64, nine tables, inserts).  Per pool:
      - the plain batch path on the same tables: the whole pool as one batch,
        executed back to back;
      - the device-resident request log (ltp_ingest: requests in HBM, merged
        Poisson arrivals of the client streams admitted by the clock, 250 us
        deadline, 4 GB read/write-set budget, aborts re-queued) swept over
        offered loads, each point at least point_s seconds of arrivals;
    and for the blend the host submission API (ltp_serve: 256 client
    streams submitting from 8 load-generator threads) swept over
    args.loads.  Per point: p50/p99/p99.9 latency (arrival -> result) and
    committed txn/s; per pool: the best committed txn/s at p99 <= 2 ms and
    its ratio to the plain path.  Before each sweep the serving size buckets
    are autotuned (untimed)."""
    import numpy as np

    import ltpmg_gb300 as G
    from ltpmg_gb300 import autotune as AT
    from ltpmg_gb300 import workloads as W

    sh = W.SHAPES["zipf"]
    n_each = 1 << 18
    tf, keys, opw, n, _ = W.generate("zipf", 0, rank=rank)
    ycsb = (tf[:n_each + 1], keys[:16 * n_each], opw[:16 * n_each])
    g, tsh = tpcc_setup(rank)
    t_tf, t_k, t_w, t_pay, _, t_ins, t_pf = g.gen(0, n_each, with_pay_first=True)
    ptf, pk, pw, ppf, ppay, src = W.mixed_pool(ycsb, (t_tf, t_k, t_w, t_pay, t_pf), seed=sh["seed"] + rank)
    n_pool = len(ptf) - 1

    def k32(k):
        """Keys as 32-bit keys when they fit: the request log stores them so."""
        return k.astype(np.uint32) if len(k) and int(k.max()) < (1 << 32) else k

    def loads_of(spec, plain):
        """Offered loads in txn/s: "a,b,..." in M txn/s, or "xf1,f2,..." as
        multiples of the plain path's rate on the same tables (the knee of
        the p99 curve sits at a steady fraction of it)."""
        if not spec:
            return []
        if spec.startswith("x"):
            return [round(float(f) * plain / 1e6) * 1e6 for f in spec[1:].split(",")]
        return [float(x) * 1e6 for x in spec.split(",")]

    host_loads = loads_of(args.loads, 0.0)
    t_host = [max(point_s, min(2.0, 20e6 / r)) for r in host_loads]
    # insert-table room for the most transactions one point can run (a
    # relative blend grid is bounded with a plain rate of 600 M txn/s); the
    # insert tables are truncated between points
    blend_bound = loads_of(args.ingest_loads, 600e6)
    per_txn = np.asarray(t_ins, np.float64) / (2 * n_each)
    most = max([r * t for r, t in zip(host_loads, t_host)] + [r * point_s for r in blend_bound] +
               [13 * n_pool]) * 1.25 + n_pool
    ctx = G.Context(device=local)
    t = ctx.create_table(sh["rows"], sh["cols"])
    ctx.fill_seeded(t, sh["seed"] + rank)
    ids = g.create_tables(ctx, np.ceil(per_txn * most).astype(np.int64) + 16)
    base_rows = {tid: ctx.table_rows(tid) for tid in ids}

    def truncate():
        for tid, r in base_rows.items():
            ctx.truncate(tid, r)

    def plain_rate(tf_, k_, w_, pay_=None, reps=10):
        """The plain batch path on the same tables: the pool as one batch."""
        b = ctx.batch(len(tf_) - 1, len(k_))
        b.load(tf_, k32(k_), w_)
        if pay_ is not None:
            b.load_payload(pay_)
        for _ in range(3):
            b.execute()
        ctx.sync()
        t0 = time.perf_counter()
        for _ in range(reps):
            b.execute()
        ctx.sync()
        r = reps * (len(tf_) - 1) / (time.perf_counter() - t0)
        b.finish()
        del b
        truncate()
        return r

    def tune_for(tf_, k_, w_, pf_, pay_):
        """Autotunes the size buckets serving batches fall into, on leading
        slices of the pool (untimed; the tables are truncated after)."""
        chosen = {}
        for m in (1 << 12, 1 << 14, 1 << 16, 1 << 18):
            m = min(m, len(tf_) - 1)
            a, e = int(tf_[0]), int(tf_[m])
            bt = ctx.batch(m, e - a)
            bt.load((tf_[:m + 1] - tf_[0]).astype(np.uint32), k32(k_[a:e]), w_[a:e])
            if pf_ is not None:
                bt.load_payload(pay_[int(pf_[0]):int(pf_[m])])
            ch = AT.tune_tiles(ctx, bt, reps=2)
            chosen[ch["bucket"]] = f"{ch['block']}x{ch['ipt']}" + ("w64" if ch["word_bits"] == 64 else "") + \
                ("+precheck" if ch["flags"] else "")
            bt.finish()
            del bt
            truncate()
        return chosen

    def point(st, rate, requests=None):
        st["offered_txn_per_s"] = rate
        if requests is not None:
            st["requests"] = requests
        st["committed_per_s"] = st["committed"] / max(st["elapsed_s"], 1e-9)
        return {k: (round(v, 3) if isinstance(v, float) else v) for k, v in st.items()}

    def ingest_sweep(ing, loads, seed):
        out = []
        ing.run(G.lib.poisson_arrivals(1 << 20, 20e6, seed))  # untimed warm-up
        truncate()
        for i, rate in enumerate(loads):
            m = int(rate * point_s)
            st = ing.run(G.lib.poisson_arrivals(m, rate, seed + 1 + i))
            truncate()
            out.append(point(st, rate, m))
        return out

    def best_of(sweep):
        ok = [p for p in sweep if p["p99_us"] <= 2000.0]
        return max(ok, key=lambda p: p["committed_per_s"]) if ok else None

    def summary(sweep, plain):
        b = best_of(sweep)
        return {"committed_txn_per_s_at_p99_le_2ms": b["committed_per_s"] if b else 0.0,
                "p50_us": b["p50_us"] if b else None, "p99_us": b["p99_us"] if b else None,
                "p999_us": b["p999_us"] if b else None,
                "offered_txn_per_s": b["offered_txn_per_s"] if b else None,
                "plain_batch_txn_per_s": plain,
                "serving_over_plain": (b["committed_per_s"] / plain) if (b and plain) else 0.0}

    out = {"point_seconds": point_s, "p99_bound_us": 2000.0, "deadline_us": 250, "budget_bytes": 4 << 30,
           "client_streams": 256}
    t_start = time.perf_counter()
    # 1. Zipf YCSB alone, request log
    if args.ycsb_loads:
        ny = 1 << 20
        ytf, yk, yw = tf[:ny + 1], keys[:int(tf[ny])], opw[:int(tf[ny])]
        plain_y = plain_rate(ytf, yk, yw)
        ycsb_loads = loads_of(args.ycsb_loads, plain_y)
        tuning_y = tune_for(ytf, yk, yw, None, None)
        ing = G.Ingest(ctx, ytf, yk, yw, deadline_us=250, depth=2, budget_bytes=4 << 30, max_txns=1 << 20,
                       max_ops=1 << 24, eager=True, jit=bool(args.ingest_jit))
        sw = ingest_sweep(ing, ycsb_loads, sh["seed"] + 29 + rank)
        ing.close()
        out["ycsb_request_log"] = dict(summary(sw, plain_y), sweep=sw, tuning=tuning_y,
                                       pool_txns=ny, workload="zipf0.99 YCSB, 16 ops, 80/20")
    # 2. the 50/50 blend, request log
    plain_b = plain_rate(ptf, pk, pw, ppay)
    blend_loads = [min(r, b) for r, b in zip(loads_of(args.ingest_loads, plain_b), blend_bound)]
    if blend_loads:
        tuning_b = tune_for(ptf, pk, pw, ppf, ppay)
        ing = G.Ingest(ctx, ptf, pk, pw, ppf, ppay, deadline_us=250, depth=2, budget_bytes=4 << 30,
                       max_txns=1 << 20, max_ops=1 << 24, eager=True, jit=bool(args.ingest_jit))
        sw = ingest_sweep(ing, blend_loads, sh["seed"] + 17 + rank)
        ing.close()
        out["blend_request_log"] = dict(summary(sw, plain_b), sweep=sw, tuning=tuning_b, pool_txns=n_pool,
                                        workload="50/50 zipf0.99 YCSB + tpcc-shaped new-order/payment")
    # 3. the blend through the host submission API
    if host_loads:
        srv = G.Server(ctx, deadline_us=250, depth=3, budget_bytes=4 << 30, max_txns=1 << 18, max_ops=1 << 22,
                       keep_results=False, persistent=args.serve_mode == "persistent")
        srv.loadgen(1e6, 0.1, 256, ptf, pk, pw, seed=1, threads=8, pay_first=ppf, payload=ppay)  # untimed
        srv.close()
        truncate()
        sw = []
        for rate, t_load in zip(host_loads, t_host):
            srv = G.Server(ctx, deadline_us=250, depth=3, budget_bytes=4 << 30, max_txns=1 << 18,
                           max_ops=1 << 22, keep_results=False, persistent=args.serve_mode == "persistent")
            # eight load-generator threads (half the host cores of the GPU
            # machine): more busy-wait the dispatcher and completer off their cores
            srv.loadgen(rate, t_load, 256, ptf, pk, pw, seed=int(rate), threads=args.loadgen_threads,
                        pay_first=ppf, payload=ppay)
            st = srv.close()
            truncate()
            st["load_seconds"] = t_load
            sw.append(point(st, rate))
        out["blend_host_api"] = dict(summary(sw, plain_b), sweep=sw, pool_txns=n_pool,
                                     loadgen_threads=args.loadgen_threads)
    out["seconds"] = round(time.perf_counter() - t_start, 1)
    ctx.close()
    return out


def run_serve(args):
    """The serving sweeps alone (longer points than the default line's);
    value = the highest committed txn/s at p99 <= 2 ms over the blend's
    request-log and host-API sweeps."""
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    sv = serving_measure(args, local, rank, point_s=args.serve_point_s)
    cands = [sv[k] for k in ("blend_request_log", "blend_host_api") if k in sv]
    best = max(cands, key=lambda d: d["committed_txn_per_s_at_p99_le_2ms"]) if cands else None
    line = {"metric": METRIC, "value": best["committed_txn_per_s_at_p99_le_2ms"] if best else 0.0, "unit": "txn/s",
            "n_gpus": world, "steps": 1, "warmup": 0, "ms_per_step": None, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int32/int64", "data": "synthetic (seeded generator)",
            "config": {"workload": WORKLOAD_TEXT["serve"], "selection": "highest committed txn/s with p99 <= 2 ms",
                       "batch_execution": args.serve_mode},
            "serving": sv}
    print(json.dumps(line), flush=True)


def uniform_distinct_rows(rows, n, per, seed):
    """n x per row ids, uniform over rows and distinct within each row of
    the result (the reference's YCSB generator redraws repeats,
    src/txn_generator.cpp:627-642)."""
    import numpy as np

    rng = np.random.default_rng(seed)
    q = rng.integers(0, rows, size=(n, per), dtype=np.int64)
    while True:
        s = np.sort(q, axis=1)
        bad = (s[:, 1:] == s[:, :-1]).any(axis=1)
        if not bad.any():
            return q.astype(np.uint32)
        q[bad] = rng.integers(0, rows, size=(int(bad.sum()), per), dtype=np.int64)


def run_refcuda(args):
    """The reference's own CUDA path timed on this GPU (oracle/_ref/
    ltpmg_ref_cuda): its host-timed cost_gpu per epoch (txn_executor through
    txn_commit, cuda/src/gpulauncher.cu:1070-1099) on the same YCSB_A batch
    re-sent every epoch, as its Scheduler does.  Its updates do not write and
    it never aborts, so this is an ordering-only throughput: a reported
    reference number, not this build's arm."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    if not os.path.exists(O.REF_CUDA):
        print(json.dumps({"impl": "reference-cuda", "unavailable": "oracle/_ref/ltpmg_ref_cuda not built "
                          "(the reference sources were never staged)"}), flush=True)
        return
    rows, n = 1 << 20, 1 << 16
    q = uniform_distinct_rows(rows, n, 10, 0x4C54504D47)
    tab = O.table_init(0x4C54504D47, rows, 3)
    epochs = args.warmup + args.steps
    out = O.ref_cuda_run(rows, q, tab.T, epochs=epochs, timeout=1200)
    timed = out["cost_gpu"][args.warmup:]
    sec = sum(timed) / len(timed)
    line = {"metric": METRIC + " (reference CUDA path, ordering only)", "value": n / sec, "unit": "txn/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec * 1e3,
            "higher_is_better": True, "impl": "reference-cuda", "data": "synthetic (seeded generator)",
            "config": {"workload": WORKLOAD_TEXT["refcuda"], "timer": "the reference's own cost_gpu (host clock, "
                       "stream synchronisations between its kernels)"},
            "cost_gpu_s": out["cost_gpu"], "used_rows": out["used_rows"],
            "ops_per_step": 10 * n}
    print(json.dumps(line), flush=True)


def run_gather(args):
    """Random-access ceiling of this GPU: uniformly random 4-byte gathers
    (torch indexing kernel, not this library) from a table of the Zipf
    workload's size (640 MB, beyond L2) and of its conflict-word array's size
    (84 MB, L2-resident).  Every random read moves at least one 32-byte
    sector, so this -- not the copy bandwidth -- bounds kernels whose ops
    touch random cells."""
    import torch

    torch.manual_seed(0)
    out = {}
    n_idx = 1 << 24
    for name, nbytes in (("table_640MB", 10 << 26), ("words_84MB", 84 << 20)):
        src = torch.zeros(nbytes // 4, dtype=torch.int32, device="cuda")
        idx = torch.randint(0, src.numel(), (n_idx,), device="cuda")
        for _ in range(3):
            src[idx]
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        reps = 10
        for _ in range(reps):
            src[idx]
        e1.record()
        e1.synchronize()
        s_per = e0.elapsed_time(e1) / 1e3 / reps
        out[name] = {"gathers_per_s": n_idx / s_per, "sector_GBps": n_idx * 32 / s_per / 1e9}
        del src, idx
    # the library's own probe: random loads, atomicOr with result, reductions
    import ltpmg_gb300 as G

    probe = {}
    for name, nbytes in (("table_640MB", 10 << 26), ("words_84MB", 84 << 20)):
        probe[name] = {m: G.lib.probe_random_access(0, nbytes, k) for m, k in
                       (("load", G.lib.PROBE_LOAD), ("atomic", G.lib.PROBE_ATOMIC), ("reduce", G.lib.PROBE_REDUCE))}
    print(json.dumps({"metric": "random 4-byte accesses/s", "gather": out, "probe": probe}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=0)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="zipf", choices=sorted(DEFAULT_STEPS))
    ap.add_argument("--mode", default="auto", choices=["auto", "graph", "persistent", "stream"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--batches", type=int, default=0, help="resident batches (default: the config's)")
    ap.add_argument("--tuning-out", default="", help="write the autotuner's choices to this JSON file")
    ap.add_argument("--tiles", default="",
                    help="fixed BLOCKxIPT[w64][+precheck] tiling instead of the autotuner's (e.g. 512x4, 256x2w64)")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end pipeline pass")
    ap.add_argument("--loads", default="1,2,5,10,20,50", help="serving sweep: offered loads in M txn/s")
    ap.add_argument("--loadgen-threads", type=int, default=8, help="serving sweep: load-generator threads")
    ap.add_argument("--ycsb-loads", default="x0.94,0.955,0.97,0.975,0.98,0.99",
                    help="request-log serving of the Zipf YCSB transactions alone: offered loads in M txn/s, "
                         "or x-prefixed multiples of the plain batch path's rate on the same tables")
    ap.add_argument("--ingest-jit", type=int, default=1,
                    help="serve: request log queues a batch only once the one ahead is past its sort (1) or at once (0)")
    ap.add_argument("--ingest-loads", default="x0.92,0.935,0.943,0.95,0.957,0.965",
                    help="serving the blend from a device-resident request log: offered loads in M txn/s, or "
                         "x-prefixed multiples of the plain batch path's rate ('' = skip)")
    ap.add_argument("--serve-point-s", type=float, default=1.0, help="serve: seconds of arrivals per sweep point")
    ap.add_argument("--no-serving", action="store_true", help="default workload: skip the serving section")
    ap.add_argument("--serve-mode", default="persistent", choices=["persistent", "stream"],
                    help="serving: each batch as one persistent-kernel launch, or as a kernel sequence")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if not args.steps:
        args.steps = DEFAULT_STEPS[args.config]
    if args.impl == "reference":
        if args.config in ("tpcc", "ycsbe"):
            run_reference_payload(args, args.config)
        else:
            run_reference(args, "zipf" if args.config in ("serve", "gather", "refcuda") else args.config)
    elif args.config == "serve":
        run_serve(args)
    elif args.config in ("tpcc", "ycsbe"):
        run_payload(args, args.config)
    elif args.config == "gather":
        run_gather(args)
    elif args.config == "refcuda":
        run_refcuda(args)
    else:
        run_ours(args, args.config)


if __name__ == "__main__":
    main()
