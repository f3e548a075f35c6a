"""Serving from a device-resident request log (ltp_ingest).

Every request's values must equal its values in the serial replay of the
committed history in (batch, position) order, bit for bit, and so must the
tables: under the ordered rule that history is the log order; under the
priority rule aborted requests are re-queued at the head of a later batch
and commit there.  A log longer than its pool (requests wrap around it)
must leave the tables equal to the serial replay of the whole log.
"""
import numpy as np
import pytest

import ltpmg_gb300 as G
import oracle as O

pytestmark = pytest.mark.gpu


def _arrivals(n, rate, seed):
    gaps = np.random.default_rng(seed).exponential(1e9 / rate, n)
    return np.cumsum(gaps).astype(np.uint64)


def _blend(seed, rows, cols, n_each):
    from ltpmg_gb300 import workloads as W

    g = G.Tpcc(2, seed=seed)
    ycsb = G.gen_ycsb(seed, rows, cols, 1, 16, 0.7, 0.99, batch=0, n_txns=n_each)
    tf_t, k_t, w_t, pay_t, _, _, pf_t = g.gen(0, n_each, with_pay_first=True)
    tf, keys, opw, pf, pay, _ = W.mixed_pool(ycsb, (tf_t, k_t, w_t, pay_t, pf_t), seed=seed + 1)
    ins_per_table = np.bincount(((w_t >> 8) & 15)[(w_t & 3) == 2], minlength=9)[:9]
    return g, tf, keys, opw, pf, pay, ins_per_table


def _tables(ctx, g, seed, rows, cols, extra):
    t0 = ctx.create_table(rows, cols)
    ctx.fill_seeded(t0, seed)
    ids = g.create_tables(ctx, extra)
    return [t0] + ids


def _oracle_tables(g, seed, rows, cols, extra):
    tabs = [(O.table_init(seed, rows, cols), rows)]
    for t in range(9):
        _, mask, r0 = g.table(t)
        tabs.append((g.initial(t, r0 + int(extra[t])), r0, mask))
    return tabs


def _history(order, tf, keys, opw, pf, pay):
    """The requests of `order` (pool indices) as one serial batch, insert keys
    rebased onto its payload."""
    htf, hk, hw, hp = [0], [], [], []
    for r in order:
        a, b = int(tf[r]), int(tf[r + 1])
        pa, pb = int(pf[r]), int(pf[r + 1])
        k = keys[a:b].copy()
        ins = (opw[a:b] & 3) == 2
        k[ins] = k[ins] - np.uint64(pa) + np.uint64(len(hp))
        hk.extend(k)
        hw.extend(opw[a:b])
        hp.extend(pay[pa:pb])
        htf.append(len(hk))
    return (np.array(htf, np.uint32), np.array(hk, np.uint64), np.array(hw, np.uint32),
            np.array(hp or [0], np.int32))


@pytest.mark.parametrize("eager,jit", [(True, False), (False, False), (True, True), (False, True)])
def test_ingest_ordered_blend_equals_log_order_replay(eager, jit):
    rows, cols, seed = 1 << 12, 10, 51
    g, tf, keys, opw, pf, pay, ins = _blend(seed, rows, cols, 6000)
    n = len(tf) - 1
    arr = _arrivals(n, 2e6, seed)  # 12,000 requests over ~6 ms: many batches
    with G.Context(device=0) as ctx:
        tabs = _tables(ctx, g, seed, rows, cols, ins)
        ing = G.Ingest(ctx, tf, keys, opw, pf, pay, deadline_us=250, depth=3, max_txns=2048, max_ops=2048 * 48,
                       eager=eager, keep_results=True, jit=jit)
        st = ing.run(arr)
        committed, seq, pos, att, vals = ing.results(values=True)
        ing.close()
        finals = [ctx.download(t) for t in tabs]
    assert st["submitted"] == n and st["committed"] == n and st["batches"] > 5
    assert committed.all() and (att == 1).all()
    # batches hold consecutive requests in log order
    order = np.lexsort((pos, seq))
    assert np.array_equal(order, np.arange(n))
    after, rc, out = O.replay_tables(0, _oracle_tables(g, seed, rows, cols, ins), *_history(range(n), tf, keys, opw,
                                                                                             pf, pay))
    assert np.array_equal(vals, out[:len(vals)])
    for t, fin in enumerate(finals):
        assert np.array_equal(fin, after[t][0][:, :after[t][1]]), t
    assert st["p99_us"] > 0 and st["p50_us"] <= st["p99_us"] <= st["max_us"] + 1


@pytest.mark.parametrize("ops", [(1, 8), (8, 8)])
def test_ingest_priority_rule_requeues_aborts(ops):
    rows, cols, seed = 256, 4, 52
    tf, keys, opw = G.gen_ycsb(seed, rows, cols, ops[0], ops[1], 0.7, 1.3, batch=0, n_txns=4000)
    n = len(tf) - 1
    arr = _arrivals(n, 1e6, seed)
    with G.Context(device=0, rule=G.RULE_PRIORITY) as ctx:
        t = ctx.create_table(rows, cols)
        ctx.fill_seeded(t, seed)
        ing = G.Ingest(ctx, tf, keys, opw, deadline_us=200, depth=2, max_txns=512, max_ops=512 * 8,
                       max_attempts=10000, keep_results=True)
        st = ing.run(arr)
        committed, seq, pos, att, vals = ing.results(values=True)
        ing.close()
        final = ctx.download(t)
    assert st["committed"] == n and st["aborted_attempts"] > 0 and att.max() > 1
    assert committed.all() and att.sum() == n + st["aborted_attempts"]
    order = np.lexsort((pos, seq))
    # no two requests share a (batch, position)
    assert len(set(zip(seq.tolist(), pos.tolist()))) == n
    htf, hk, hw, _ = _history(order, tf, keys, opw, np.zeros(n + 1, np.uint64), np.zeros(1, np.int32))
    tab, rc, out = O.replay(0, O.table_init(seed, rows, cols), htf, hk, hw)
    for i, r in enumerate(order):
        a, b = int(tf[r]), int(tf[r + 1])
        assert np.array_equal(vals[a:b], out[htf[i]:htf[i + 1]]), (r, seq[r], pos[r])
    assert np.array_equal(final, tab)


def test_ingest_priority_rule_gives_up_after_max_attempts():
    rows, cols, seed = 64, 2, 53
    tf, keys, opw = G.gen_ycsb(seed, rows, cols, 4, 8, 0.0, 1.5, batch=0, n_txns=3000)
    n = len(tf) - 1
    arr = np.zeros(n, np.uint64)  # everything arrives at once
    with G.Context(device=0, rule=G.RULE_PRIORITY) as ctx:
        t = ctx.create_table(rows, cols)
        ctx.fill_seeded(t, seed)
        ing = G.Ingest(ctx, tf, keys, opw, deadline_us=50, depth=2, max_txns=1024, max_ops=1024 * 8, max_attempts=2)
        st = ing.run(arr)
        committed, seq, pos, att = ing.results()
        ing.close()
    lost = int((committed == 0).sum())
    assert lost > 0 and st["completed"] == n and st["committed"] == n - lost
    assert (att[committed == 0] == 2).all() and att.max() <= 2


def test_ingest_log_wraps_its_pool():
    rows, cols, seed = 1 << 12, 10, 54
    g, tf, keys, opw, pf, pay, ins = _blend(seed, rows, cols, 2000)
    n_pool = len(tf) - 1
    n = n_pool * 5 // 2  # requests wrap the pool twice and a half
    arr = _arrivals(n, 3e6, seed)
    with G.Context(device=0) as ctx:
        tabs = _tables(ctx, g, seed, rows, cols, ins * 3)
        ing = G.Ingest(ctx, tf, keys, opw, pf, pay, deadline_us=150, depth=3, max_txns=1536, max_ops=1536 * 48)
        st = ing.run(arr)
        ing.close()
        finals = [ctx.download(t) for t in tabs]
    assert st["committed"] == n and st["batches"] > 3
    order = [i % n_pool for i in range(n)]
    after, rc, out = O.replay_tables(0, _oracle_tables(g, seed, rows, cols, ins * 3),
                                     *_history(order, tf, keys, opw, pf, pay))
    for t, fin in enumerate(finals):
        assert np.array_equal(fin, after[t][0][:, :after[t][1]]), t


@pytest.mark.parametrize("keys64", [False, True])
def test_ingest_fixed_length_pool_wraps_in_place(keys64):
    """A pool of equal-length transactions runs fixed-length batches; windows
    that wrap the pool execute in place from the doubled log; 32- and 64-bit
    log keys give the same tables and values."""
    rows, cols, seed = 1 << 14, 10, 56
    tf, keys, opw = G.gen_ycsb(seed, rows, cols, 16, 16, 0.8, 0.99, batch=0, n_txns=3000)
    n_pool = len(tf) - 1
    n = n_pool * 7 // 2  # requests wrap the pool three and a half times
    arr = _arrivals(n, 4e6, seed)
    with G.Context(device=0) as ctx:
        t = ctx.create_table(rows, cols)
        ctx.fill_seeded(t, seed)
        # first the kept values of one pool's worth of requests
        ing = G.Ingest(ctx, tf, keys, opw, deadline_us=120, depth=2, max_txns=1024, max_ops=1024 * 16,
                       keep_results=True, keys64=keys64)
        st = ing.run(arr[:n_pool])
        committed, seq, pos, att, vals = ing.results(values=True)
        ing.close()
        mid = ctx.download(t)
        # then a log that wraps the pool, with batches of up to the whole pool
        ing = G.Ingest(ctx, tf, keys, opw, deadline_us=300, depth=2, max_txns=n_pool, max_ops=n_pool * 16,
                       keys64=keys64, jit=True)
        st2 = ing.run(arr[n_pool:] - arr[n_pool])
        ing.close()
        mid2 = ctx.download(t)
        # a burst larger than the pool: batches of more than n_pool requests are gathered
        n3 = n_pool * 5 // 2
        ing = G.Ingest(ctx, tf, keys, opw, deadline_us=300, depth=2, max_txns=2 * n_pool, max_ops=2 * n_pool * 16,
                       keys64=keys64)
        st3 = ing.run(np.zeros(n3, np.uint64))
        ing.close()
        final = ctx.download(t)
    assert st["committed"] == n_pool and committed.all() and st["batches"] > 2
    tab, rc, out = O.replay(0, O.table_init(seed, rows, cols), tf, keys, opw)
    assert np.array_equal(vals, out) and np.array_equal(mid, tab)
    assert st2["committed"] == n - n_pool and st2["batches"] > 3
    order = [i % n_pool for i in range(n_pool, n)]
    htf, hk, hw, _ = _history(order, tf, keys, opw, np.zeros(n_pool + 1, np.uint64), np.zeros(1, np.int32))
    tab2, rc2, _ = O.replay(0, tab, htf, hk, hw)
    assert np.array_equal(mid2, tab2)
    assert st3["committed"] == n3 and st3["batches"] >= 2
    htf, hk, hw, _ = _history([i % n_pool for i in range(n3)], tf, keys, opw, np.zeros(n_pool + 1, np.uint64),
                              np.zeros(1, np.int32))
    tab3, rc3, _ = O.replay(0, tab2, htf, hk, hw)
    assert np.array_equal(final, tab3)


def test_ingest_rejects_bad_pools_and_arrivals():
    rows, cols, seed = 1 << 10, 4, 55
    tf, keys, opw = G.gen_ycsb(seed, rows, cols, 1, 8, 0.5, 0.5, batch=0, n_txns=100)
    with G.Context(device=0) as ctx:
        t = ctx.create_table(rows, cols)
        ctx.fill_seeded(t, seed)
        with pytest.raises(G.LtpError):  # a transaction larger than a batch
            G.Ingest(ctx, tf, keys, opw, max_txns=16, max_ops=4)
        ing = G.Ingest(ctx, tf, keys, opw, keep_results=True)
        with pytest.raises(G.LtpError):  # arrivals must not decrease
            ing.run(np.array([5, 3] + [9] * 98, np.uint64))
        with pytest.raises(G.LtpError):  # kept values need n <= pool
            ing.run(np.zeros(200, np.uint64))
        ing.close()
