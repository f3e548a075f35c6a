#!/usr/bin/env python3
"""Benchmark of the batched transaction-processing hot path.

Default workload (N=1): the high-contention YCSB-style configuration --
2^24 rows x 10 int32 columns, 32 resident batches of 2^20 transactions x 16
ops, Zipf 0.99 keys over a seeded permutation of the rows, 80% reads / 20% +1
read-modify-writes, ordered rule (every op on a cell in ascending TID order,
all transactions commit).  A step is one batch; steps cycle over the 32
batches, so the table evolves exactly as a serial replay would evolve it.
Inputs are far larger than L2 (201 MB of ops per batch, 640 MB table).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--config zipf|plain]
  python bench.py --impl reference ...   (CPU baseline: the oracle's
                                           multi-threaded serial replay)

Under torchrun every rank drives its own GPU with an independent replica of
the workload (the path does not shard on one GPU per process: replicas only);
value = all ranks' transactions / the slowest rank's time.
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

SEED = 0x4C54504D47
CONFIGS = {
    "zipf": dict(workload="ycsb-zipf0.99: 2^24 rows x 10 int32, 32 batches x 2^20 txns x 16 ops, 80% read / 20% +1 RMW",
                 rows=1 << 24, cols=10, txns=1 << 20, ops=16, read=0.8, theta=0.99, batches=32, seed=SEED + 2),
    "plain": dict(workload="ycsb-uniform: 2^20 rows x 10 int32, 16 batches x 2^16 txns x 10 ops, 50% read / 50% +1 RMW",
                  rows=1 << 20, cols=10, txns=1 << 16, ops=10, read=0.5, theta=0.0, batches=16, seed=SEED),
}
METRIC = "committed txn/s"
# per-kernel algorithmic bytes: key 8 + opword 4 + bitmap word 4
KERNEL_BYTES = {
    "mark": lambda st: 16 * st["ops"],
    "ids": lambda st: 20 * st["touched_words"] + 16 * st["contended_cells"],
    "classify": lambda st: 28 * st["ops"],
    "sort_hist": lambda st: 8 * st["contended_ops"],
    "sort_pass0": lambda st: 16 * st["contended_ops"],
    "sort_pass1": lambda st: 16 * st["contended_ops"],
    "sort_pass2": lambda st: 16 * st["contended_ops"],
    "sort_pass3": lambda st: 16 * st["contended_ops"],
    "apply": lambda st: 16 * st["contended_ops"] + 12 * st["contended_cells"],
    "finish": lambda st: 12 * st["touched_words"],
}


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


def load_traffic():
    p = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    return json.load(open(p)) if os.path.exists(p) else {}


def gen_batches(cfg, nb, rank):
    import ltpmg_gb300 as G

    out = []
    for b in range(nb):
        tf, k, w = G.gen_ycsb(cfg["seed"] + rank, cfg["rows"], cfg["cols"], cfg["ops"], cfg["ops"], cfg["read"],
                              cfg["theta"], batch=b, n_txns=cfg["txns"])
        out.append((k, w))
    return out


def cpu_baseline(cfg, batches, budget_s=12.0):
    """Single-core serial replay (the oracle port) over whole batches until
    the time budget is spent; returns txn/s and what was sampled."""
    import ctypes

    import numpy as np

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    L = O.lib()
    tab = O.table_init(cfg["seed"], cfg["rows"], cfg["cols"])
    tf = (np.arange(cfg["txns"] + 1, dtype=np.uint32) * cfg["ops"]).astype(np.uint32)
    commit = np.zeros(cfg["txns"], np.uint8)
    done, t_used = 0, 0.0
    for k, w in batches:
        out = np.zeros(len(k), np.int32)
        t0 = time.perf_counter()
        rc = L.ltpo_replay(0, cfg["rows"], cfg["cols"], tab.ctypes.data, cfg["txns"], tf.ctypes.data, k.ctypes.data,
                           w.ctypes.data, commit.ctypes.data, out.ctypes.data)
        t_used += time.perf_counter() - t0
        assert rc == 0
        done += 1
        if t_used >= budget_s:
            break
    _ = ctypes
    return {"value": done * cfg["txns"] / t_used, "unit": "txn/s", "cores": 1, "kind": "port",
            "sample": f"{done} full batch(es) of {cfg['txns']} txns x {cfg['ops']} ops, serial replay (ordered rule), "
                      f"{t_used:.1f} s"}


def run_reference(args, cfg):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import ctypes

    import numpy as np

    import ltpmg_gb300 as G  # host generator only (no GPU use)

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    threads = os.cpu_count() or 1
    nb = min(cfg["batches"], 4)
    batches = gen_batches(cfg, nb, 0)
    tab = O.table_init(cfg["seed"], cfg["rows"], cfg["cols"])
    sample_txns = min(cfg["txns"], 1 << 16)
    per_batch = cfg["txns"] // sample_txns
    tf = (np.arange(sample_txns + 1, dtype=np.uint32) * cfg["ops"]).astype(np.uint32)
    commit = np.zeros(sample_txns, np.uint8)
    out = np.zeros(sample_txns * cfg["ops"], np.int32)
    L = O.lib()

    def step(i):
        k, w = batches[(i // per_batch) % nb]
        j = i % per_batch
        lo, hi = j * sample_txns * cfg["ops"], (j + 1) * sample_txns * cfg["ops"]
        kk, ww = k[lo:hi], w[lo:hi]
        rc = L.ltpo_replay_r0_mt(cfg["rows"], cfg["cols"], tab.ctypes.data, sample_txns, tf.ctypes.data,
                                 kk.ctypes.data, ww.ctypes.data, commit.ctypes.data, out.ctypes.data, threads)
        assert rc == 0

    for i in range(args.warmup):
        step(i)
    t0 = time.perf_counter()
    for i in range(args.steps):
        step(args.warmup + i)
    dt = time.perf_counter() - t0
    value = args.steps * sample_txns / dt
    _ = (ctypes, G)
    line = {"metric": METRIC, "value": value, "unit": "txn/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic (seeded generator)",
            "config": {"workload": cfg["workload"], "step": f"{sample_txns} txns x {cfg['ops']} ops",
                       "l2": "inputs larger than L2"},
            "impl": "reference",
            "cpu_baseline": {"value": value, "unit": "txn/s", "cores": threads, "kind": "port",
                             "sample": f"{args.steps} slices of {sample_txns} txns from {nb} batches, "
                                       f"cell-partitioned serial replay on {threads} threads"},
            "e2e": {"value": value, "unit": "txn/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args, cfg):
    import numpy as np
    import torch

    import ltpmg_gb300 as G

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    nb = cfg["batches"]
    host = gen_batches(cfg, nb, rank)
    ctx = G.Context(device=local, stage_timing=True)
    if args.tune:
        blk, ipt = (int(x) for x in args.tune.split(","))
        for bucket in range(64):
            ctx.set_tuning(bucket, blk, ipt)
    t = ctx.create_table(cfg["rows"], cfg["cols"])
    ctx.fill_seeded(t, cfg["seed"] + rank)
    dev = []
    for k, w in host:
        b = ctx.batch(cfg["txns"], len(k))
        b.load(None, k, w, ops_per_txn=cfg["ops"])
        dev.append(b)
    ctx.sync()
    stream = torch.cuda.ExternalStream(ctx.stream)
    for i in range(args.warmup):
        dev[i % nb].execute()
    ctx.sync()
    barrier(world)
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.15)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for i in range(args.steps):
        dev[(args.warmup + i) % nb].execute()
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    clk = clocks.stop()
    ms = reduce_max(ms, world)
    # per-kernel times of the last execution of every batch (events on the launching stream)
    stats = [b.finish().as_dict() for b in dev]
    total_txns = args.steps * cfg["txns"] * world
    value = total_txns / (ms / 1e3)

    # end to end through the C ABI: pinned host inputs, H2D, execute, D2H of
    # the commit vector and per-op values, every step
    n_e2e = min(args.steps, 64)
    pk = [G.PinnedArray((len(host[i][0]),), np.uint64) for i in range(2)]
    pw = [G.PinnedArray((len(host[i][1]),), np.uint32) for i in range(2)]
    for i in range(2):
        pk[i].array[:] = host[i][0]
        pw[i].array[:] = host[i][1]
    pc = G.PinnedArray((cfg["txns"],), np.uint8)
    pv = G.PinnedArray((cfg["txns"] * cfg["ops"],), np.int32)
    eb = dev[0]
    for i in range(2):
        eb.load(None, pk[i].array, pw[i].array, ops_per_txn=cfg["ops"])
        eb.execute()
        eb.fetch(pc.array, pv.array)
    ctx.sync()
    barrier(world)
    t0 = time.perf_counter()
    for i in range(n_e2e):
        eb.load(None, pk[i % 2].array, pw[i % 2].array, ops_per_txn=cfg["ops"])
        eb.execute()
        eb.fetch(pc.array, pv.array)
    ctx.sync()
    e2e_s = reduce_max(time.perf_counter() - t0, world)
    eb.finish()
    n_ops = cfg["txns"] * cfg["ops"]
    e2e = {"value": n_e2e * cfg["txns"] * world / e2e_s, "unit": "txn/s", "h2d_bytes_per_step": 12 * n_ops,
           "d2h_bytes_per_step": 4 * n_ops + cfg["txns"], "steps": n_e2e}

    if rank != 0:
        return
    peak, peak_kind = load_peaks()
    avg = {}
    for name in KERNEL_BYTES:
        vals = [s["ms_stage"][name] for s in stats]
        avg[name] = sum(vals) / len(vals)
    dom = max(avg, key=avg.get)
    mean_stats = {k: sum(s[k] for s in stats) / len(stats) for k in ("ops", "touched_words", "contended_cells",
                                                                     "contended_ops")}
    dom_bytes = KERNEL_BYTES[dom](mean_stats)
    achieved = dom_bytes / (avg[dom] / 1e3) / 1e9
    traffic = load_traffic().get(dom)
    traffic_b = None
    if traffic:
        units = mean_stats["contended_ops"] if traffic.get("unit") == "contended_op" else mean_stats["ops"]
        traffic_b = traffic["bytes_per_unit"] * units
    batch_ms = statistics.mean(s["ms_stage"]["total"] for s in stats)
    alg_batch = 28 * n_ops + 4 * cfg["txns"]
    line = {"metric": METRIC, "value": value, "unit": "txn/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic (seeded generator)",
            "config": {"workload": cfg["workload"], "rule": "ordered (ascending TID per cell, all commit)",
                       "l2": "inputs larger than L2 (201 MB ops/batch, 640 MB table)",
                       "parallelism": f"replicas x{world}"},
            "gpu_launches": 10 * args.steps,
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic_b, "peak_kind": peak_kind,
                         "algorithmic_bytes_per_launch": dom_bytes, "avg_launch_ms": avg[dom],
                         "pipeline": {"algorithmic_bytes_per_batch": alg_batch, "avg_batch_ms": batch_ms,
                                      "achieved": alg_batch / (batch_ms / 1e3) / 1e9,
                                      "frac": alg_batch / (batch_ms / 1e3) / 1e9 / peak},
                         "kernel_ms": avg},
            "clocks": clk, "e2e": e2e,
            "contention": {"contended_ops_per_batch": mean_stats["contended_ops"],
                           "contended_cells_per_batch": mean_stats["contended_cells"]}}
    if world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(cfg, host)
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="zipf", choices=sorted(CONFIGS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--batches", type=int, default=0, help="resident batches to cycle (default: the config's)")
    ap.add_argument("--tune", default="", help="block,ipt for every size bucket (default: library tuning)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    cfg = dict(CONFIGS[args.config])
    if args.batches:
        cfg["batches"] = args.batches
    if args.impl == "reference":
        run_reference(args, cfg)
    else:
        run_ours(args, cfg)


if __name__ == "__main__":
    main()
