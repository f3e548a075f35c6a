"""int64 columns and linked inserts.

CPU tests check the oracle's int64 / link semantics on hand-made batches;
GPU tests compare the CUDA path with the oracle bit for bit: 64-bit sums
beyond 2^32 on one hot cell, int32 columns wrapping at 32 bits inside a
context that has int64 columns, linked inserts taking a read's or an RMW's
output, and the malformed-link error path.
"""
import numpy as np
import pytest

import ltpmg_gb300 as G
import oracle as O

READ, ADD, INS = 0, 1, 2


def link(col, table, d):
    return O.opword(INS, col, table, d & 0x3FF)


def test_oracle_int64_sum_and_int32_wrap():
    # table 0: col 0 int32, col 1 int64
    data = np.zeros((2, 4), np.int64)
    data[0, 0] = 2**31 - 1
    data[1, 0] = 2**40
    ops = [(0, O.opword(ADD, 0, 0, 1)), (0, O.opword(ADD, 1, 0, -5)), (0, O.opword(READ, 1, 0, 0))]
    tf = np.array([0, 3], np.uint32)
    keys = np.array([k for k, _ in ops], np.uint64)
    opw = np.array([w for _, w in ops], np.uint32)
    after, commit, out = O.replay_tables(0, [(data, 4, 0b10)], tf, keys, opw)
    assert list(out) == [-(2**31), 2**40 - 5, 2**40 - 5]
    assert after[0][0][0, 0] == -(2**31) and after[0][0][1, 0] == 2**40 - 5


def test_oracle_linked_insert():
    counter = np.array([[10, 20]], np.int32)
    rows = np.zeros((2, 8), np.int64)
    # txn 0: counter[1] += 1 -> 21, insert row linked to it in column 0;
    # txn 1: read counter[1] (21), insert linked (distance 1) in column 1
    tf = np.array([0, 2, 4], np.uint32)
    keys = np.array([1, 0, 1, 3], np.uint64)
    opw = np.array([O.opword(ADD, 0, 0, 1), link(0, 1, 1), O.opword(READ, 0, 0, 0), link(1, 1, 1)], np.uint32)
    payload = np.array([0, 7, 0, 9, 0, 0], np.int32)  # row images: int32 col 0, int64 col 1 (2 slots)
    after, commit, out = O.replay_tables(0, [(counter, 2), (rows, 0, 0b10)], tf, keys, opw, payload)
    assert list(out) == [21, 0, 21, 1]
    assert after[1][1] == 2
    assert after[1][0][:, :2].tolist() == [[21, 9], [7, 21]]


def test_oracle_rejects_bad_links():
    t = np.zeros((1, 4), np.int32)
    pl = np.zeros(4, np.int32)
    for tf, keys, opw in (
        ([0, 1], [0], [link(0, 0, 1)]),                               # before the transaction
        ([0, 1, 2], [0, 0], [O.opword(READ, 0, 0, 0), link(0, 0, 1)]),  # other transaction
        ([0, 2], [0, 0], [link(0, 0, 0), link(0, 0, 1)]),             # names an insert
        ([0, 2], [0, 0], [O.opword(READ, 0, 0, 0), link(3, 0, 1)]),   # no such column
    ):
        with pytest.raises(ValueError):
            O.replay_tables(0, [(t, 1)], np.array(tf, np.uint32), np.array(keys, np.uint64),
                            np.array(opw, np.uint32), pl)


def _wide_batch(rng, shapes, n_txns, hot=4, p_ins=0.2, max_ops=10):
    """Random multi-table batch over int32/int64 columns: reads, RMWs with
    large immediates, plain and linked inserts."""
    tf, keys, opw, payload = [0], [], [], []
    for _ in range(n_txns):
        first = len(keys)
        for _ in range(int(rng.integers(1, max_ops + 1))):
            tb = int(rng.integers(0, len(shapes)))
            rows, cols, mask = shapes[tb]
            if rng.random() < p_ins:
                keys.append(len(payload))
                prior = [j for j in range(first, len(keys) - 1) if (opw[j] & 3) != INS]
                if prior and rng.random() < 0.6:
                    j = prior[int(rng.integers(0, len(prior)))]
                    opw.append(link(int(rng.integers(0, cols)), tb, len(keys) - 1 - j))
                else:
                    opw.append(O.opword(INS, 0, tb, 0))
                for c in range(cols):
                    v = int(rng.integers(-2**40, 2**40)) if (mask >> c) & 1 else int(rng.integers(-2**31, 2**31))
                    payload += [v & 0xFFFFFFFF, (v >> 32) & 0xFFFFFFFF] if (mask >> c) & 1 else [v & 0xFFFFFFFF]
                continue
            r = int(rng.integers(0, hot) if rng.random() < 0.5 else rng.integers(0, rows))
            keys.append(r)
            opw.append(O.opword(int(rng.random() < 0.7), int(rng.integers(0, cols)), tb,
                                int(rng.integers(-2**19, 2**19))))
        tf.append(len(keys))
    pl = np.array(payload or [0], np.uint32).view(np.int32)
    return np.array(tf, np.uint32), np.array(keys, np.uint64), np.array(opw, np.uint32), pl


def _initial(rng, rows, cols, mask, cap):
    d = np.zeros((cols, cap), np.int64)
    for c in range(cols):
        hi = 2**50 if (mask >> c) & 1 else 2**31
        d[c, :rows] = rng.integers(-hi, hi, rows)
    return d


@pytest.mark.gpu
@pytest.mark.parametrize("rule", [0, 1])
@pytest.mark.parametrize("mode", ["single", G.MODE_GRAPH, G.MODE_PERSISTENT])
def test_wide_columns_and_links_match_oracle(rule, mode):
    rng = np.random.default_rng(100 + rule)
    shapes = [(300, 4, 0b1010), (50, 3, 0b001), (40, 2, 0)]
    n_batches, n_txns = 3, 3000
    with G.Context(device=0, rule=rule) as ctx:
        ids, ref = [], []
        for rows, cols, mask in shapes:
            cap = rows + n_batches * n_txns * 10
            tid = ctx.create_table(rows, cols, rows_cap=cap, wide=[c for c in range(cols) if (mask >> c) & 1])
            d = _initial(rng, rows, cols, mask, cap)
            ctx.upload(tid, d[:, :rows])
            ids.append(tid)
            ref.append((d if mask else d.astype(np.int32), rows, mask))
        cur = list(shapes)
        batches = []
        for _ in range(n_batches):
            # rows named by later batches must exist at their start: use the
            # row counts before any of this sequence's inserts
            batches.append(_wide_batch(rng, cur, n_txns))
        bs = [ctx.batch(n_txns, n_txns * 10) for _ in batches]
        for (tf, keys, opw, pl), b in zip(batches, bs):
            b.load(tf, keys, opw)
            b.load_payload(pl)
        if mode == "single":
            for b in bs:
                b.execute()
        else:
            ctx.execute_many(bs, mode=mode)
        for (tf, keys, opw, pl), b in zip(batches, bs):
            commit, vals, _ = b.results64()
            ref, rc, ro = O.replay_tables(rule, ref, tf, keys, opw, pl)
            assert np.array_equal(commit, rc)
            bad = np.nonzero(vals != ro)[0]
            assert len(bad) == 0, (bad[:5], vals[bad[:5]], ro[bad[:5]])
            _, vals32, _ = b.results()
            assert np.array_equal(vals32, ro.astype(np.int32))
        for k, tid in enumerate(ids):
            assert ctx.table_rows(tid) == ref[k][1]
            got = ctx.download(tid)
            assert np.array_equal(got, ref[k][0][:, :ref[k][1]])


@pytest.mark.gpu
def test_int64_hot_cell_sum_beyond_32_bits():
    """2^16 RMWs of +500000 on one int64 cell (sum ~3.3e10) next to one
    int32 cell that wraps, in a single batch."""
    n = 1 << 16
    with G.Context(device=0) as ctx:
        t = ctx.create_table(4, 2, wide=[1])
        ctx.upload(t, np.array([[2**31 - 10, 0, 0, 0], [2**45, 0, 0, 0]], np.int64))
        keys = np.zeros(2 * n, np.uint64)
        opw = np.empty(2 * n, np.uint32)
        opw[0::2] = O.opword(ADD, 1, 0, 500000)
        opw[1::2] = O.opword(ADD, 0, 0, 3)
        b = ctx.batch(n, 2 * n)
        b.load(None, keys, opw, ops_per_txn=2)
        b.execute()
        commit, vals, st = b.results64()
        steps = np.arange(1, n + 1, dtype=np.int64)
        assert np.array_equal(vals[0::2], 2**45 + 500000 * steps)
        assert np.array_equal(vals[1::2], ((2**31 - 10 + 3 * steps + 2**31) % 2**32) - 2**31)
        fin = ctx.download(t)
        assert fin[1, 0] == 2**45 + 500000 * n
        assert st.contended_cells == 2


@pytest.mark.gpu
def test_bad_link_reported():
    with G.Context(device=0) as ctx:
        t = ctx.create_table(4, 2, rows_cap=16, wide=[1])
        b = ctx.batch(2, 4)
        # the second transaction's insert links across the transaction boundary
        b.load(np.array([0, 1, 2], np.uint32), np.array([0, 0], np.uint64),
               np.array([O.opword(READ, 0, 0, 0), link(0, 0, 1)], np.uint32))
        b.load_payload(np.zeros(4, np.int32))
        b.execute()
        with pytest.raises(G.LtpError) as e:
            b.results64()
        assert "index 1" in str(e.value)
        assert ctx.table_rows(t) == 4


@pytest.mark.gpu
@pytest.mark.parametrize("rule", [0, 1])
def test_repeated_cells_in_one_transaction_and_int32_wrap(rule):
    """A transaction that RMWs one cell twice and reads it in between (the
    cell is contended: the batch's smallest writing TID is this transaction,
    later transactions touch it too), and uncontended int32 RMWs that wrap."""
    with G.Context(device=0, rule=rule) as ctx:
        t = ctx.create_table(8, 2, wide=[1])
        init = np.array([[5, 2**31 - 2, -(2**31) + 1, 0, 0, 0, 0, 0], [2**40, 7, 0, 0, 0, 0, 0, 0]], np.int64)
        ctx.upload(t, init)
        tf = np.array([0, 5, 7, 8], np.uint32)
        keys = np.array([0, 0, 0, 0, 1, 0, 0, 2], np.uint64)
        opw = np.array([O.opword(ADD, 1, 0, 3), O.opword(READ, 1, 0, 0), O.opword(ADD, 1, 0, -7),
                        O.opword(ADD, 0, 0, 2), O.opword(ADD, 0, 0, 5),
                        O.opword(READ, 1, 0, 0), O.opword(ADD, 1, 0, 1),
                        O.opword(ADD, 0, 0, -9)], np.uint32)
        b = ctx.batch(3, 8)
        b.load(tf, keys, opw)
        b.execute()
        commit, vals, _ = b.results64()
        ref, rc, ro = O.replay_tables(rule, [(init, 8, 0b10)], tf, keys, opw)
        assert np.array_equal(commit, rc) and np.array_equal(vals, ro)
        assert np.array_equal(ctx.download(t), ref[0][0])
        assert ro[4] == -(2**31) + 3 and ro[7] == 2**31 - 8
