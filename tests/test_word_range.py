"""Batches that touch part of a multi-table context, against the oracle.

The ids and finish kernels stream over the conflict words between the
lowest and the highest word a batch touched when that range is densely
touched, so a batch on a table that is not the context's first starts its
scan at a nonzero word.  Apply scans in 32 bits for a batch that touches no
int64 cell even when the context has int64 columns (the 64-bit outputs of
int32 ops are then widened on fetch).  Under the ordered rule an insert's
slot comes from mark's per-tile insert counts; mark tiles of every size
from 128 to 4096 ops add into the same 4096-op insert tiles.  Every case
compares commit vectors, 64- and 32-bit op values and every table bit for
bit with the oracle's multi-table replay.
"""
import numpy as np
import pytest

import ltpmg_gb300 as G
import oracle as O

pytestmark = pytest.mark.gpu
READ, ADD, INS = 0, 1, 2


def _batch(rng, shapes, tables, n_txns, ops, hot=8, p_ins=0.0):
    """Transactions of `ops` ops on the listed tables: half on a few hot
    rows, reads and RMWs (+ inserts with probability p_ins)."""
    tf, keys, opw, payload = [0], [], [], []
    for _ in range(n_txns):
        for _ in range(ops):
            tb = int(tables[int(rng.integers(0, len(tables)))])
            rows, cols, mask = shapes[tb]
            if rng.random() < p_ins:
                keys.append(len(payload))
                opw.append(O.opword(INS, 0, tb, 0))
                for c in range(cols):
                    v = int(rng.integers(-2**40, 2**40)) if (mask >> c) & 1 else int(rng.integers(-2**31, 2**31))
                    payload += [v & 0xFFFFFFFF, (v >> 32) & 0xFFFFFFFF] if (mask >> c) & 1 else [v & 0xFFFFFFFF]
                continue
            r = int(rng.integers(0, hot) if rng.random() < 0.5 else rng.integers(0, rows))
            keys.append(r)
            opw.append(O.opword(int(rng.random() < 0.4), int(rng.integers(0, cols)), tb,
                                int(rng.integers(-2**19, 2**19))))
        tf.append(len(keys))
    pl = np.array(payload or [0], np.uint32).view(np.int32)
    return np.array(tf, np.uint32), np.array(keys, np.uint64), np.array(opw, np.uint32), pl


def _context(ctx, rng, shapes, caps):
    ids, ref = [], []
    for (rows, cols, mask), cap in zip(shapes, caps):
        tid = ctx.create_table(rows, cols, rows_cap=cap, wide=[c for c in range(cols) if (mask >> c) & 1])
        d = np.zeros((cols, cap), np.int64)
        for c in range(cols):
            hi = 2**50 if (mask >> c) & 1 else 2**31
            d[c, :rows] = rng.integers(-hi, hi, rows)
        ctx.upload(tid, d[:, :rows])
        ids.append(tid)
        ref.append((d if mask else d.astype(np.int32), rows, mask))
    return ids, ref


def _check(ctx, ids, ref, rule, batches, bs):
    for (tf, keys, opw, pl), b in zip(batches, bs):
        commit, vals, st = b.results64()
        ref, rc, ro = O.replay_tables(rule, ref, tf, keys, opw, pl)
        assert np.array_equal(commit, rc)
        bad = np.nonzero(vals != ro)[0]
        assert len(bad) == 0, (bad[:5], vals[bad[:5]], ro[bad[:5]])
        _, vals32, _ = b.results()
        assert np.array_equal(vals32, ro.astype(np.int32))
    for k, tid in enumerate(ids):
        assert ctx.table_rows(tid) == ref[k][1]
        assert np.array_equal(ctx.download(tid), ref[k][0][:, :ref[k][1]])
    return ref


@pytest.mark.parametrize("mode", ["single", G.MODE_GRAPH])
def test_batches_on_part_of_a_multi_table_context(mode):
    """Table 0 (int32), table 1 (int32, small: a batch on it alone touches
    most of its words, which start past table 0's), table 2 (an int64
    column, large capacity: the context's word space is ~90x table 1's).
    Batches on table 1 alone (enough ops that mark builds no touched-word
    list), on table 0 alone, on tables 0 and 2 (64-bit scan), then on table
    1 again (mark builds the list; ids and finish still stream the range)."""
    rng = np.random.default_rng(7)
    shapes = [(1 << 13, 6, 0), (1 << 10, 4, 0), (1 << 12, 5, 0b00100)]
    caps = [1 << 13, 1 << 10, 1 << 16]
    plan = [([1], 1 << 11, 12), ([0], 1 << 12, 8), ([0, 2], 1 << 11, 8), ([1], 1 << 10, 16)]
    with G.Context(device=0) as ctx:
        ids, ref = _context(ctx, rng, shapes, caps)
        batches = [_batch(rng, shapes, tabs, n, ops) for tabs, n, ops in plan]
        bs = [ctx.batch(n, n * ops) for _, n, ops in plan]
        for (tf, keys, opw, pl), b in zip(batches, bs):
            b.load(tf, keys, opw)
        if mode == "single":
            for b in bs:
                b.execute()
        else:
            ctx.execute_many(bs, mode=mode)
        _check(ctx, ids, ref, 0, batches, bs)


@pytest.mark.parametrize("block,ipt,word_bits", [(128, 1, 32), (256, 2, 32), (512, 4, 32), (512, 8, 32),
                                                 (256, 4, 64), (512, 2, 64)])
def test_insert_slots_from_mark_counts_every_tiling(block, ipt, word_bits):
    """Inserts into three tables spread over several 4096-op insert tiles,
    with mark tiles of 128 to 4096 ops: the slots, the rows and every op
    value equal the oracle's, over two batches (the second starts from the
    first's row counts)."""
    rng = np.random.default_rng(block * 10 + ipt + word_bits)
    shapes = [(1 << 12, 4, 0), (600, 3, 0b010), (300, 2, 0)]
    n_txns, ops = 1500, 12
    caps = [s[0] + 2 * n_txns * ops for s in shapes]
    with G.Context(device=0) as ctx:
        for bucket in range(64):
            ctx.set_tuning(bucket, block, ipt, word_bits=word_bits)
        ids, ref = _context(ctx, rng, shapes, caps)
        batches, bs = [], []
        for _ in range(2):
            tf, keys, opw, pl = _batch(rng, shapes, [0, 1, 2], n_txns, ops, p_ins=0.3)
            b = ctx.batch(n_txns, n_txns * ops)
            b.load(tf, keys, opw)
            b.load_payload(pl)
            b.execute()
            batches.append((tf, keys, opw, pl))
            bs.append(b)
        ref = _check(ctx, ids, ref, 0, batches, bs)
        assert ref[0][1] > shapes[0][0]  # rows were inserted
