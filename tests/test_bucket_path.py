"""The cell-bucket path (LTP_TUNE_BUCKET) against the oracle, bit for bit.

With the flag set on every size bucket, ordered-rule batches without
inserts run as: hot-cell sampling and selection, op records, one radix pass
into 256 buckets of consecutive cells, one block per bucket (local sort by
cell, segmented scan, write-back), and the hot cells by a radix pass of
their ids and the segmented scan.  Same results as the conflict-word path
and the serial replay: the commit vector, every op value and the table --
at full size (the Zipf and uniform workloads), with int64 columns and two
tables, at every chunk and tile edge, with adversarial keys (one cell, all
distinct, two hot cells, enough hot cells to overflow the hot set),
immediates too wide for the record, and batches that fall back to the
conflict-word path (inserts, the priority rule, the persistent kernel).
"""
import numpy as np
import pytest

import ltpmg_gb300 as G
import oracle as O
from test_gpu_parity import SEED, _pattern_batch, gen, run_and_check

pytestmark = pytest.mark.gpu
BUCKET = (512, 4, 32, G.lib.TUNE_BUCKET)


@pytest.fixture(scope="module")
def lib_loaded():
    return G.load()


def test_full_size_zipf_batches_on_the_bucket_path(lib_loaded):
    rows, cols = 1 << 24, 10
    batches = [gen(SEED + 2, rows, cols, 16, 16, 0.8, 0.99, b, 1 << 20) for b in range(2)]
    stats = run_and_check(0, rows, cols, batches, seed=SEED + 2, fixed=16, threads=8, tuning=BUCKET)
    for st in stats:
        assert st["path"] == 1 and st["bucket_ops"] > 0 and st["contended_cells"] > 0
        assert st["bucket_ops"] + st["contended_ops"] == st["ops"]


def test_full_size_plain_batches_on_the_bucket_path(lib_loaded):
    rows, cols = 1 << 20, 10
    batches = [gen(SEED, rows, cols, 10, 10, 0.5, 0.0, b, 1 << 16) for b in range(4)]
    stats = run_and_check(0, rows, cols, batches, fixed=10, threads=8, tuning=BUCKET)
    assert all(st["path"] == 1 for st in stats)


@pytest.mark.parametrize("shape", [(1 << 14, 10, 1, 32, 0.99, 3000), (300, 3, 1, 8, 1.2, 5000),
                                   (1 << 16, 4, 16, 16, 0.0, 4096), (7, 2, 1, 4, 0.5, 1000)])
def test_seeded_sequences_on_the_bucket_path(lib_loaded, shape):
    rows, cols, omin, omax, th, n = shape
    batches = [gen(SEED + 7, rows, cols, omin, omax, 0.6, th, b, n) for b in range(3)]
    stats = run_and_check(0, rows, cols, batches, seed=SEED + 7, tuning=BUCKET)
    assert all(st["path"] == 1 for st in stats)


@pytest.mark.parametrize("n_ops", [1, 31, 32, 2047, 2048, 2049, 3072, 4095, 4096, 4097, 8193, 40000])
@pytest.mark.parametrize("pattern", ["same_cell", "distinct", "skewed", "hot_pair"])
def test_chunk_edges_and_adversarial_keys(lib_loaded, n_ops, pattern):
    """Sizes around the 2048-op record tile, the 3072-record radix tile and
    the 4096-record bucket chunk; keys on one cell (a hot cell, or with few
    ops a cold one), all distinct, Zipf 1.3, two hot cells; random
    immediates in [-3, 3]."""
    rows, cols = 1 << 12, 4
    rng = np.random.default_rng(n_ops * 17 + len(pattern))
    tf, keys, opw = _pattern_batch(pattern, n_ops, rows, cols, rng)
    stats = run_and_check(0, rows, cols, [(tf, keys, opw)], seed=5, tuning=BUCKET)
    assert stats[0]["path"] == 1


def test_wide_immediates_and_many_hot_cells(lib_loaded):
    """Immediates beyond the record's 11 bits (read from the opword) and
    more hot-cell candidates than the hot set holds (the rest stay in their
    buckets): 600 cells with ~4000 ops each."""
    rows, cols = 1 << 14, 10
    rng = np.random.default_rng(3)
    n = 600 * 4000
    cells = rng.integers(0, 600, n) * 97 % (rows * cols)
    keys = (cells // cols).astype(np.uint64)
    col = (cells % cols).astype(np.uint32)
    kind = (rng.random(n) < 0.3).astype(np.uint32)
    imm = rng.integers(-(1 << 19), 1 << 19, n)
    opw = (kind | (col << 2) | ((np.where(kind == 1, imm, 0).astype(np.int64) & 0xFFFFF) << 12)).astype(np.uint32)
    tf = np.arange(0, n + 1, 8, dtype=np.uint32)
    stats = run_and_check(0, rows, cols, [(tf, keys, opw)], seed=9, tuning=BUCKET)
    assert stats[0]["path"] == 1 and 0 < stats[0]["contended_cells"] <= 256


def test_int64_columns_and_two_tables(lib_loaded):
    """Two tables, one with int64 columns, sums beyond 2^32, on the bucket
    path (the 64-bit segmented scan)."""
    rng = np.random.default_rng(11)
    with G.Context(device=0) as ctx:
        for bucket in range(64):
            ctx.set_tuning(bucket, *BUCKET)
        a = ctx.create_table(5000, 3)
        w = ctx.create_table(2000, 4, wide=[1, 3])
        ctx.fill_seeded(a, 1)
        ctx.fill_seeded(w, 2)
        ta = O.table_init(1, 5000, 3)
        tw = np.zeros((4, 2000), np.int64)
        tw[:] = O.table_init(2, 2000, 4)
        n = 60000
        tb = rng.integers(0, 2, n)
        keys = np.where(tb == 0, rng.integers(0, 64, n), rng.integers(0, 40, n)).astype(np.uint64)
        col = np.where(tb == 0, rng.integers(0, 3, n), rng.integers(0, 4, n)).astype(np.uint32)
        kind = (rng.random(n) < 0.5).astype(np.uint32)
        imm = rng.integers(400000, 500000, n)
        opw = (kind | (col << 2) | (tb.astype(np.uint32) << 8) |
               ((np.where(kind == 1, imm, 0) & 0xFFFFF) << 12)).astype(np.uint32)
        tf = np.arange(0, n + 1, 4, dtype=np.uint32)
        for _ in range(2):
            b = ctx.batch(len(tf) - 1, n)
            b.load(tf, keys, opw)
            b.execute()
            commit, vals, st = b.results64()
            assert st.path == 1
            after, rc, ro = O.replay_tables(0, [(ta, 5000), (tw, 2000, 0b1010)], tf, keys, opw)
            ta, tw = after[0][0], after[1][0]
            assert np.array_equal(commit, rc) and np.array_equal(vals, ro)
        assert np.array_equal(ctx.download(a), ta)
        assert np.array_equal(ctx.download(w), tw)


def test_ineligible_batches_fall_back(lib_loaded):
    """The priority rule and batches with inserts take the conflict-word
    path even where the bucket flag is set; results equal the oracle."""
    rows, cols = 1 << 12, 4
    batches = [gen(SEED + 3, rows, cols, 1, 16, 0.7, 0.9, b, 2000) for b in range(2)]
    stats = run_and_check(1, rows, cols, batches, seed=SEED + 3, tuning=BUCKET)
    assert all(st["path"] == 0 for st in stats)


@pytest.mark.parametrize("mode", [G.MODE_STREAM, G.MODE_GRAPH, G.MODE_PERSISTENT])
def test_multi_batch_modes_on_the_bucket_path(lib_loaded, mode):
    """Uneven batches through one multi-batch call (the persistent kernel
    keeps the conflict-word path), twice, against the oracle."""
    rows, cols, seed = 1 << 14, 10, 99
    shapes = [(1 << 10, 1, 32, 0.5), (3000, 1, 32, 0.99), (200, 4, 4, 0.8), (1 << 12, 16, 16, 0.7), (1, 1, 1, 0.9)]
    with G.Context(device=0) as ctx:
        for bucket in range(64):
            ctx.set_tuning(bucket, *BUCKET)
        t = ctx.create_table(rows, cols)
        ctx.fill_seeded(t, seed)
        ref = O.table_init(seed, rows, cols)
        bs = [ctx.batch(n, n * omax) for n, omin, omax, th in shapes]
        for rep in range(2):
            data = []
            for k, ((n, omin, omax, th), b) in enumerate(zip(shapes, bs)):
                tf, keys, opw = gen(seed + rep, rows, cols, omin, omax, 0.7, th, k, n)
                b.load(tf, keys, opw)
                data.append((tf, keys, opw))
            ctx.execute_many(bs, mode=mode)
            for (tf, keys, opw), b in zip(data, bs):
                commit, vals, st = b.results()
                ref, rc, ro = O.replay(0, ref, tf, keys, opw)
                assert np.array_equal(commit, rc) and np.array_equal(vals, ro)
                assert st.path == (0 if mode == G.MODE_PERSISTENT else 1)
            assert np.array_equal(ctx.download(t), ref)
