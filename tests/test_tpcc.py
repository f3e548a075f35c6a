"""TPC-C-shaped order-entry workload (new-order / payment).

CPU: the generator's batches have the documented op shapes, links, input
ranges and payload contents, the same for any thread count; the initial
tables follow their documented values and the last-name index picks the
middle customer.  GPU: whole-database parity with the oracle -- every
table, every op value (64-bit), the commit vector -- for sequences of
batches under both rules and the multi-batch modes, and a W=8 batch of
2^16 transactions.
"""
import numpy as np
import pytest

import ltpmg_gb300 as G
import oracle as O
from ltpmg_gb300 import lib as L

READ, ADD, INS = 0, 1, 2


def _fields(opw):
    imm = (opw.astype(np.uint32) >> 12).astype(np.int64)
    imm = np.where(imm >= 1 << 19, imm - (1 << 20), imm)
    return opw & 3, (opw >> 2) & 63, (opw >> 8) & 15, imm


@pytest.fixture(scope="module")
def small():
    return G.Tpcc(3, seed=11, customers=3000, items=100000)


def test_schema_and_initial_values(small):
    n_cols, mask, rows = small.table(L.TPCC_CUSTOMER)
    assert (n_cols, rows) == (16, 3 * 10 * 3000) and mask == (1 << 6) | (1 << 7)
    assert small.table(L.TPCC_ORDER_LINE)[2] == 0
    last = small.column(L.TPCC_CUSTOMER, 3)
    c = np.arange(len(last)) % 3000
    assert np.array_equal(last[c < 1000], c[c < 1000])
    assert last.min() >= 0 and last.max() <= 999
    assert np.all(small.column(L.TPCC_DISTRICT, 4) == 3000)
    price = small.column(L.TPCC_ITEM, 2)
    assert price.min() >= 100 and price.max() <= 10000
    q = small.column(L.TPCC_STOCK, 2)
    assert q.min() >= 10 and q.max() <= 100
    assert small.column(L.TPCC_WAREHOUSE, 2).dtype == np.int64


def test_generator_shapes_links_and_payload(small):
    tf, keys, opw, pay, n_no, ins = small.gen(3, 4000)
    kind, col, tb, imm = _fields(opw)
    price = small.column(L.TPCC_ITEM, 2)
    sdist = [small.column(L.TPCC_STOCK, 6 + q) for q in range(6)]
    lines = 0
    remote_lines = 0
    for t in range(4000):
        a, b = int(tf[t]), int(tf[t + 1])
        if tb[a] == L.TPCC_WAREHOUSE and kind[a] == READ:  # new-order
            n = b - a
            assert (n - 5) % 3 == 0 and 5 <= (n - 5) // 3 <= 15
            assert kind[a + 1] == ADD and tb[a + 1] == L.TPCC_DISTRICT and col[a + 1] == 4 and imm[a + 1] == 1
            w, dist = int(keys[a]), int(keys[a + 1])
            assert dist // 10 == w
            assert int(keys[a + 2]) // 3000 == dist
            for j in range(a + 3, b):
                if kind[j] == INS:
                    assert a + 1 == j - (imm[j] & 0x3FF), "insert not linked to the order-id draw"
            for line in range((n - 5) // 3):
                j = a + 5 + 3 * line
                assert tb[j] == L.TPCC_ORDER_LINE and kind[j] == INS
                p = int(keys[j])
                qty, item, supply = int(pay[p + 6]), int(pay[p + 4]) - 1, int(pay[p + 5]) - 1
                assert 1 <= qty <= 10 and int(pay[p + 3]) == line + 1
                amount = int(np.uint32(pay[p + 7])) | (int(pay[p + 8]) << 32)
                assert amount == qty * int(price[item])
                srow = supply * 100000 + item
                assert [int(pay[p + 9 + q]) for q in range(6)] == [int(s[srow]) for s in sdist]
                assert int(keys[j + 1]) == srow and imm[j + 1] == -qty and imm[j + 2] == qty
                lines += 1
                remote_lines += supply != w
        else:  # payment
            assert b - a == 7
            assert [int(x) for x in tb[a:b]] == [0, 1, 2, 2, 2, 2, 3]
            h = int(imm[a])
            assert 100 <= h <= 500000 and imm[a + 1] == h and imm[a + 3] == -h and imm[a + 5] == 1
            p = int(keys[a + 6])
            assert int(np.uint32(pay[p + 5])) | (int(pay[p + 6]) << 32) == h
    assert n_no == ins[L.TPCC_ORDER] == ins[L.TPCC_NEW_ORDER] and ins[L.TPCC_ORDER_LINE] == lines
    assert 0.45 < n_no / 4000 < 0.55
    assert remote_lines / lines < 0.03
    # thread count does not change the batch
    tf2, keys2, opw2, pay2, _, _ = small.gen(3, 4000, threads=1)
    assert np.array_equal(keys, keys2) and np.array_equal(opw, opw2) and np.array_equal(pay, pay2)


def test_last_name_payments_pick_the_middle_customer(small):
    """A by-name payment's customer has a last name that some draw produced;
    with many batches every resolved customer must be the middle one (by id)
    among the district's customers with that name."""
    last = small.column(L.TPCC_CUSTOMER, 3).reshape(30, 3000)
    middle = {}
    for d in range(30):
        for name in np.unique(last[d]):
            ids = np.nonzero(last[d] == name)[0]
            middle[(d, int(name))] = int(ids[(len(ids) - 1) // 2])
    tf, keys, opw, pay, n_no, ins = small.gen(9, 20000)
    kind, col, tb, imm = _fields(opw)
    pay_rows = [int(keys[int(tf[t]) + 2]) for t in range(20000) if tb[int(tf[t])] == L.TPCC_WAREHOUSE
                and kind[int(tf[t])] == ADD]
    by_middle = sum(1 for r in pay_rows if middle[(r // 3000, int(last[r // 3000, r % 3000]))] == r % 3000)
    # by-id draws hit a middle customer only by chance (about 1 in 2-3 for
    # the first 1000 ids); by-name draws always do: at least 60% overall
    assert by_middle / len(pay_rows) > 0.6


def _tables_for(g, extra):
    ref = []
    for t in range(9):
        n_cols, mask, rows = g.table(t)
        ref.append((g.initial(t, rows + int(extra[t])), rows, mask))
    return ref


def _run_tpcc(g, rule, n_batches, n_txns, mode="single", tuning=None):
    batches = [g.gen(b, n_txns) for b in range(n_batches)]
    extra = np.sum([x[5] for x in batches], axis=0)
    with G.Context(device=0, rule=rule) as ctx:
        if tuning:
            for bucket in range(64):
                ctx.set_tuning(bucket, *tuning)
        ids = g.create_tables(ctx, extra)
        bs = []
        for tf, keys, opw, pay, _, _ in batches:
            b = ctx.batch(len(tf) - 1, len(keys))
            b.load(tf, keys, opw)
            b.load_payload(pay)
            bs.append(b)
        if mode == "single":
            for b in bs:
                b.execute()
        else:
            ctx.execute_many(bs, mode=mode)
        ref = _tables_for(g, extra)
        for (tf, keys, opw, pay, _, _), b in zip(batches, bs):
            commit, vals, st = b.results64()
            ref, rc, ro = O.replay_tables(rule, ref, tf, keys, opw, pay)
            assert np.array_equal(commit, rc)
            bad = np.nonzero(vals != ro)[0]
            assert len(bad) == 0, (bad[:5], vals[bad[:5]], ro[bad[:5]])
        for t, tid in enumerate(ids):
            assert ctx.table_rows(tid) == ref[t][1], G.TPCC_TABLES[t]
            got = ctx.download(tid)
            assert np.array_equal(got, ref[t][0][:, :ref[t][1]]), G.TPCC_TABLES[t]
        return [b.finish() for b in bs]


@pytest.mark.gpu
@pytest.mark.parametrize("rule", [0, 1])
def test_tpcc_sequence_matches_oracle(small, rule):
    stats = _run_tpcc(small, rule, 3, 5000)
    if rule == 1:
        assert all(s.aborted > 0 for s in stats)


@pytest.mark.gpu
@pytest.mark.parametrize("rule", [0, 1])
def test_tpcc_sequence_with_64_cell_words(small, rule):
    _run_tpcc(small, rule, 2, 4000, tuning=(256, 2, 64))


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [G.MODE_GRAPH, G.MODE_PERSISTENT])
def test_tpcc_multi_batch_modes(small, mode):
    _run_tpcc(small, 0, 3, 3000, mode=mode)


@pytest.mark.gpu
def test_tpcc_w8_batch_2_16():
    g = G.Tpcc(8, seed=23)
    stats = _run_tpcc(g, 0, 2, 1 << 16)
    assert stats[0].contended_cells > 0


@pytest.mark.gpu
def test_checkpoint_and_resume_replays_to_the_same_state(small):
    """Checkpoint = every table's rows (ltp_table_download) after batch k;
    resume = a fresh context with those rows uploaded, then the batches after
    k.  Execution is deterministic, so the resumed run's op values, commit
    vectors and final tables equal the uninterrupted run's (both rules)."""
    for rule in (0, 1):
        batches = [small.gen(b, 3000) for b in range(4)]
        extra = np.sum([x[5] for x in batches], axis=0)
        outs, snap = [], None
        with G.Context(device=0, rule=rule) as ctx:
            ids = small.create_tables(ctx, extra)
            for k, (tf, keys, opw, pay, _, _) in enumerate(batches):
                b = ctx.batch(len(tf) - 1, len(keys))
                b.load(tf, keys, opw)
                b.load_payload(pay)
                b.execute()
                outs.append(b.results64()[:2])
                if k == 1:
                    snap = [ctx.download(t) for t in ids]
            final = [ctx.download(t) for t in ids]
        with G.Context(device=0, rule=rule) as ctx:
            ids2 = []
            for t in range(9):
                n_cols, mask, rows0 = small.table(t)
                rows = snap[t].shape[1]
                tid = ctx.create_table(rows, n_cols, rows_cap=max(1, rows0 + int(extra[t])),
                                       wide=[c for c in range(n_cols) if (mask >> c) & 1])
                if rows:
                    for c in range(n_cols):
                        ctx.upload_column(tid, c, snap[t][c])
                ids2.append(tid)
            for k in (2, 3):
                tf, keys, opw, pay, _, _ = batches[k]
                b = ctx.batch(len(tf) - 1, len(keys))
                b.load(tf, keys, opw)
                b.load_payload(pay)
                b.execute()
                commit, vals = b.results64()[:2]
                assert np.array_equal(commit, outs[k][0]) and np.array_equal(vals, outs[k][1]), (rule, k)
            for t, tid in enumerate(ids2):
                assert np.array_equal(ctx.download(tid), final[t]), (rule, G.TPCC_TABLES[t])
