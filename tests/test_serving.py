"""The continuous-batching request loop (ltp_server).

Every committed transaction's result must equal its result in the serial
replay of the committed history in (batch, position) order -- the result it
would get alone at its place in the sequence -- bit for bit; a stream's
transactions must commit in submission order; under the priority rule,
aborted transactions are re-queued and commit later.
"""
import numpy as np
import pytest

import ltpmg_gb300 as G
import oracle as O

pytestmark = pytest.mark.gpu


def _verify_history(results, pool, rows, cols, seed, rule):
    tf, keys, opw = pool
    committed = sorted([r for r in results if r.committed], key=lambda r: (r.batch_seq, r.pos))
    # the committed history, serially, from the initial table
    htf, hk, hw = [0], [], []
    for r in committed:
        a, b = int(tf[r.tag]), int(tf[r.tag + 1])
        hk.extend(keys[a:b])
        hw.extend(opw[a:b])
        htf.append(len(hk))
    tab, commit, out = O.replay(0, O.table_init(seed, rows, cols), np.array(htf, np.uint32),
                                np.array(hk, np.uint64), np.array(hw, np.uint32))
    for i, r in enumerate(committed):
        n = htf[i + 1] - htf[i]
        assert r.n_ops == n
        assert list(r.vals[:n]) == out[htf[i]:htf[i + 1]].tolist(), (r.tag, r.batch_seq, r.pos)
    return committed, tab


def _pool(seed, rows, cols, n, theta=0.99, omax=16):
    return G.gen_ycsb(seed, rows, cols, 1, omax, 0.7, theta, batch=0, n_txns=n)


@pytest.mark.parametrize("eager,persistent", [(True, False), (False, False), (True, True)])
def test_serving_ordered_rule_loadgen(eager, persistent):
    rows, cols, seed = 1 << 12, 10, 31
    pool = _pool(seed, rows, cols, 20000)
    with G.Context(device=0) as ctx:
        t = ctx.create_table(rows, cols)
        ctx.fill_seeded(t, seed)
        srv = G.Server(ctx, deadline_us=250, depth=3, max_txns=4096, max_ops=4096 * 16, eager=eager,
                       persistent=persistent)
        srv.loadgen(rate=400000.0, seconds=0.04, n_streams=64, txn_first=pool[0], keys=pool[1], opw=pool[2],
                    seed=7, threads=4)
        got = []
        while True:
            got.extend(srv.poll())
            if len(got) >= srv.stats()["submitted"]:
                break
        st = srv.close()
        final = ctx.download(t)
    assert st["submitted"] > 1000 and st["completed"] == st["submitted"] and st["committed"] == st["completed"]
    assert st["batches"] > 1 and st["p99_us"] > 0
    committed, tab = _verify_history(got, pool, rows, cols, seed, 0)
    assert np.array_equal(final, tab)
    # each stream's pool indices (tags) were drawn in time order: commit order keeps them increasing
    by_stream = {}
    for r in committed:
        by_stream.setdefault(r.stream, []).append(r.tag)
    assert all(v == sorted(v) for v in by_stream.values())


def test_serving_results_equal_serial_history():
    rows, cols, seed = 1 << 12, 10, 32
    pool = _pool(seed, rows, cols, 5000)
    with G.Context(device=0) as ctx:
        t = ctx.create_table(rows, cols)
        ctx.fill_seeded(t, seed)
        srv = G.Server(ctx, deadline_us=100, depth=3, max_txns=1024, max_ops=1024 * 16)
        tf, keys, opw = pool
        order = {}
        for k in range(len(tf) - 1):
            stream = k % 7
            srv.submit(stream, keys[tf[k]:tf[k + 1]], opw[tf[k]:tf[k + 1]], tag=k)
            order.setdefault(stream, []).append(k)
        got = []
        while len(got) < len(tf) - 1:
            got.extend(srv.poll())
        st = srv.close()
        final = ctx.download(t)
    assert st["committed"] == len(tf) - 1
    committed, tab = _verify_history(got, pool, rows, cols, seed, 0)
    assert np.array_equal(final, tab)
    # per-stream submission order is the commit order
    for stream, tags in order.items():
        seen = [r.tag for r in committed if r.stream == stream]
        assert seen == tags


def test_serving_priority_rule_requeues_aborts():
    rows, cols, seed = 256, 4, 33
    tf, keys, opw = _pool(seed, rows, cols, 3000, theta=1.3, omax=8)
    with G.Context(device=0, rule=G.RULE_PRIORITY) as ctx:
        t = ctx.create_table(rows, cols)
        ctx.fill_seeded(t, seed)
        srv = G.Server(ctx, deadline_us=200, depth=2, max_txns=512, max_ops=512 * 8, max_attempts=10000)
        for k in range(len(tf) - 1):
            srv.submit(k % 5, keys[tf[k]:tf[k + 1]], opw[tf[k]:tf[k + 1]], tag=k)
        got = []
        while len(got) < len(tf) - 1:
            got.extend(srv.poll())
        st = srv.close()
        final = ctx.download(t)
    assert st["committed"] == len(tf) - 1 and st["aborted_attempts"] > 0
    assert max(r.attempts for r in got) > 1
    committed, tab = _verify_history(got, (tf, keys, opw), rows, cols, seed, 1)
    assert np.array_equal(final, tab)


def test_serving_mix_of_ycsb_and_tpcc_transactions():
    """A seeded 50/50 blend of YCSB transactions (table 0) and TPC-C
    new-order / payment transactions with inserts and int64 columns (tables
    1-9) through the load generator: every committed transaction's 64-bit
    values equal its values in the serial replay of the committed history,
    and so do all ten tables."""
    from ltpmg_gb300 import workloads as W

    rows, cols, seed = 1 << 12, 10, 41
    g = G.Tpcc(2, seed=seed)
    ycsb = _pool(seed, rows, cols, 3000)
    tf_t, k_t, w_t, pay_t, _, _, pf_t = g.gen(0, 3000, with_pay_first=True)
    tf, keys, opw, pay_first, payload, src = W.mixed_pool(ycsb, (tf_t, k_t, w_t, pay_t, pf_t), seed=5)
    extra = np.zeros(9, np.int64)
    for t, n in enumerate(np.bincount(((w_t >> 8) & 15)[(w_t & 3) == 2], minlength=9)[:9]):
        extra[t] = n
    with G.Context(device=0) as ctx:
        t0 = ctx.create_table(rows, cols)
        ctx.fill_seeded(t0, seed)
        ids = g.create_tables(ctx, extra)
        assert ids == list(range(1, 10)) and ctx.wide
        srv = G.Server(ctx, deadline_us=200, depth=3, max_txns=2048, max_ops=2048 * 48, persistent=True)
        srv.loadgen(rate=300000.0, seconds=0.02, n_streams=32, txn_first=tf, keys=keys, opw=opw, seed=3, threads=4,
                    pay_first=pay_first, payload=payload)
        got = []
        while True:
            got.extend(srv.poll())
            if len(got) >= srv.stats()["submitted"]:
                break
        st = srv.close()
        finals = [ctx.download(t) for t in [t0] + ids]
    assert st["submitted"] > 1000 and st["committed"] == st["submitted"]
    assert {int(src[r.tag]) for r in got} == {0, 1}
    committed = sorted(got, key=lambda r: (r.batch_seq, r.pos))
    # the committed history as one serial batch (insert keys rebased to its payload)
    htf, hk, hw, hp = [0], [], [], []
    for r in committed:
        a, b = int(tf[r.tag]), int(tf[r.tag + 1])
        pa, pb = int(pay_first[r.tag]), int(pay_first[r.tag + 1])
        k = keys[a:b].copy()
        ins = (opw[a:b] & 3) == 2
        k[ins] = k[ins] - np.uint64(pa) + np.uint64(len(hp))
        hk.extend(k)
        hw.extend(opw[a:b])
        hp.extend(payload[pa:pb])
        htf.append(len(hk))
    tabs = [(O.table_init(seed, rows, cols), rows)]
    for t in range(9):
        n_cols, mask, r0 = g.table(t)
        tabs.append((g.initial(t, r0 + int(extra[t])), r0, mask))
    after, rc, out = O.replay_tables(0, tabs, np.array(htf, np.uint32), np.array(hk, np.uint64),
                                     np.array(hw, np.uint32), np.array(hp or [0], np.int32))
    for i, r in enumerate(committed):
        n = htf[i + 1] - htf[i]
        assert r.n_ops == n
        assert list(r.vals[:n]) == out[htf[i]:htf[i + 1]].tolist(), (r.tag, r.batch_seq, r.pos)
    for t, fin in enumerate(finals):
        data, n = after[t][0], after[t][1]
        assert np.array_equal(fin, data[:, :n]), t
