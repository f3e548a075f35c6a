"""Project-written autotuner for the batch kernels.

Per size bucket (floor(log2(ops in the batch))) it times every candidate
tiling of the streaming kernels -- threads per block x ops per thread, the
knobs that set how many ops a tile stages in shared memory -- then 64-cell
conflict words (bitmap word granularity) for the fastest tilings, then the
mark kernel's hot-word pre-check, on a representative batch with CUDA
events, and keeps the fastest.  For a list of
batches it also times the multi-batch execution modes (CUDA graph vs the
persistent cooperative kernel) and keeps the faster one.  Choices persist as
JSON and are applied with Context.set_tuning.

Tuning runs execute real batches: they advance the table they run on, so
run them on a context whose table may change (a scratch copy, or before the
workload's measured or checked part).
"""
import json
import math
import time

from . import lib as L

BLOCKS = (128, 256, 512)
IPTS = (1, 2, 4, 8)


def bucket_of(n_ops):
    return max(0, int(math.floor(math.log2(n_ops)))) if n_ops > 0 else 0


def _time_batch(ctx, batch, reps, copies=1):
    """Median over reps of one execution's time.  copies > 1: the batch runs
    that many times back to back in one captured graph per rep (the way
    resident batches run), so host launch gaps do not blur small batches."""
    import torch

    stream = torch.cuda.ExternalStream(ctx.stream)
    if copies > 1:
        ctx.execute_many([batch] * copies, mode=L.MODE_GRAPH)  # captures this tuning's graph
    ms = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        if copies > 1:
            ctx.execute_many([batch] * copies, mode=L.MODE_GRAPH)
        else:
            batch.execute()
        e1.record(stream)
        e1.synchronize()
        ms.append(e0.elapsed_time(e1) / copies)
    batch.finish()
    ms.sort()
    return ms[len(ms) // 2]


def tune_tiles(ctx, batch, reps=3, blocks=BLOCKS, ipts=IPTS, copies=1):
    """Times every (block, ipt) on one loaded batch; sets and returns the best
    for the batch's size bucket as {"block", "ipt", "ms", "candidates"}.
    copies > 1 times graph-captured back-to-back executions (see _time_batch);
    a batch with insert payload is always timed one execution at a time, so
    that tuning appends as few rows as possible."""
    bucket = bucket_of(batch.n_ops)
    if getattr(batch, "_keep_payload", None) is not None or batch.n_ops >= (1 << 22):
        copies = 1  # (a batch of 2^22 ops runs long enough to time alone)
    results = {}
    batch.execute()  # warm-up
    batch.finish()
    for blk in blocks:
        for ipt in ipts:
            ctx.set_tuning(bucket, blk, ipt)
            results[f"{blk}x{ipt}"] = _time_batch(ctx, batch, reps, copies)
    # conflict-word granularity: 64-cell words for the three fastest tilings
    # that have them (tiles of at most 2048 ops)
    for name in sorted(results, key=results.get)[:6]:
        blk, ipt = (int(x) for x in name.split("x"))
        if blk * ipt <= 2048 and len([k for k in results if k.endswith("w64")]) < 3:
            ctx.set_tuning(bucket, blk, ipt, word_bits=64)
            results[f"{name}w64"] = _time_batch(ctx, batch, reps, copies)
    best = min(results, key=results.get)
    base, _, wb = best.partition("w")
    blk, ipt = (int(x) for x in base.split("x"))
    word_bits = int(wb) if wb else 32
    # then, for the best tiling, the mark kernel's hot-word pre-check
    ctx.set_tuning(bucket, blk, ipt, word_bits=word_bits, flags=L.TUNE_MARK_PRECHECK)
    pre_ms = _time_batch(ctx, batch, reps, copies)
    results[f"{best}+precheck"] = pre_ms
    flags = L.TUNE_MARK_PRECHECK if pre_ms < results[best] else 0
    ctx.set_tuning(bucket, blk, ipt, word_bits=word_bits, flags=flags)
    return {"bucket": bucket, "block": blk, "ipt": ipt, "word_bits": word_bits, "flags": flags,
            "ms": min(results[best], pre_ms), "candidates": results}


def tune_mode(ctx, batches, reps=2, modes=(L.MODE_GRAPH, L.MODE_PERSISTENT)):
    """Times whole multi-batch calls in each mode; returns (best_mode, {mode: ms})."""
    import torch

    stream = torch.cuda.ExternalStream(ctx.stream)
    out = {}
    for m in modes:
        ctx.execute_many(batches, mode=m)  # warm-up (captures the graph)
        ctx.sync()
        ms = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            ctx.execute_many(batches, mode=m)
            e1.record(stream)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        out[m] = min(ms)
    for b in batches:
        b.finish()
    return min(out, key=out.get), out


def parse_choice(name):
    """(block, ipt, word_bits, flags) of a candidate name such as 512x4,
    512x2w64 or 512x4+precheck."""
    base, _, opt = name.partition("+")
    base, _, wb = base.partition("w")
    blk, ipt = (int(x) for x in base.split("x"))
    return blk, ipt, int(wb) if wb else 32, L.TUNE_MARK_PRECHECK if opt == "precheck" else 0


def _time_list(ctx, batches, reps, mode=L.MODE_GRAPH):
    """Best over reps of one multi-batch call over the list (after a warm-up
    call that captures the graph)."""
    import torch

    stream = torch.cuda.ExternalStream(ctx.stream)
    ctx.execute_many(batches, mode=mode)
    ctx.sync()
    ms = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ctx.execute_many(batches, mode=mode)
        e1.record(stream)
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    for b in batches:
        b.finish()
    return min(ms)


def refine_pipeline(ctx, batches, choice, top=2, reps=2, mode=L.MODE_GRAPH):
    """Re-times a size bucket's `top` fastest single-batch tilings, each with
    and without the mark pre-check, on the whole list of batches executed the
    way the workload runs them (one captured graph by default), and keeps the
    fastest there.  One batch repeated in isolation misjudges tilings whose
    L2 footprint differs when different batches follow each other (order
    entry: 512x2 with 64-cell words looks as fast as 512x4 alone, and is 2%
    slower over four batches).  Every candidate runs reps + 1 times over the
    list: a payload workload needs 2 * top * (reps + 1) executions' worth of
    insert capacity."""
    bases = []
    for name in sorted(choice["candidates"], key=choice["candidates"].get):
        base = name.partition("+")[0]
        if base not in bases:
            bases.append(base)
        if len(bases) == top:
            break
    ranked = [b + sfx for b in bases for sfx in ("", "+precheck")]
    timed = {}
    for name in ranked:
        blk, ipt, wb, flags = parse_choice(name)
        ctx.set_tuning(choice["bucket"], blk, ipt, word_bits=wb, flags=flags)
        timed[name] = _time_list(ctx, batches, reps, mode)
    best = min(timed, key=timed.get)
    blk, ipt, wb, flags = parse_choice(best)
    ctx.set_tuning(choice["bucket"], blk, ipt, word_bits=wb, flags=flags)
    out = dict(choice)
    out.update({"block": blk, "ipt": ipt, "word_bits": wb, "flags": flags, "pipeline_ms": timed})
    return out


def tune_buckets(ctx, batches, reps=3, copies=1):
    """One representative batch per size bucket; returns {bucket: choice}."""
    seen = {}
    for b in batches:
        k = bucket_of(b.n_ops)
        if k not in seen or b.n_ops > seen[k].n_ops:
            seen[k] = b
    return {k: tune_tiles(ctx, b, reps, copies=copies) for k, b in sorted(seen.items())}


def save(path, choices, mode=None):
    doc = {"buckets": {str(k): {"block": v["block"], "ipt": v["ipt"], "word_bits": v.get("word_bits", 32),
                                "flags": v.get("flags", 0), "ms": v["ms"]}
                       for k, v in choices.items()},
           "mode": mode, "when": time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime())}
    with open(path, "w") as f:
        json.dump(doc, f, indent=1)


def load(ctx, path):
    """Applies a saved tuning file to a context; returns its multi-batch mode."""
    doc = json.load(open(path))
    for k, v in doc["buckets"].items():
        ctx.set_tuning(int(k), int(v["block"]), int(v["ipt"]), word_bits=int(v.get("word_bits", 32)),
                       flags=int(v.get("flags", 0)))
    return doc.get("mode")
