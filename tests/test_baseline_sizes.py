"""Parity at the full sizes of the benchmark configurations.

Each test runs one configuration the way the benchmark does and compares
every batch's commit vector, every op value and the final tables with the
oracle's serial replay (its multi-threaded ordered-rule replay where the
batches are large), bit for bit:

  - high contention: all 32 Zipf 0.99 batches of 2^20 transactions x 16 ops
    on the 2^24 x 10 int32 table, chained, from one captured graph, 32-bit
    keys (the benchmark's step);
  - order entry: one batch of 2^18 new-order / payment transactions over the
    W=64 TPC-C-shaped tables (nine tables, int64 money, inserts);
  - uneven batching: the 64 batches of 2^U[10,20] transactions with 1-32 ops
    and per-batch Zipf skew, through one captured graph and through the
    persistent kernel;
  - serving: the 50/50 blend of the Zipf YCSB and order-entry transactions on
    full-size tables of both shapes (2^24 x 10 and W=64), served from the
    device-resident request log at the merged arrivals of 256 Poisson client
    streams; every request's values and the tables equal the serial replay
    of the log.
"""
import os

import numpy as np
import pytest

import ltpmg_gb300 as G
import oracle as O
from ltpmg_gb300 import workloads as W

pytestmark = pytest.mark.gpu
THREADS = os.cpu_count() or 1


def _load(b, tf, keys, opw, fixed, rows):
    k = keys.astype(np.uint32) if rows <= (1 << 32) else keys
    if fixed:
        b.load(None, k, opw, ops_per_txn=fixed)
    else:
        b.load(tf, k, opw)


def _check_chain(ctx, t, sh, name, bs, n_batches, seed):
    """Each resident batch against the oracle's replay, in order, on one
    oracle table carried from batch to batch; then the final table."""
    ref = O.table_init(seed, sh["rows"], sh["cols"])
    for k in range(n_batches):
        tf, keys, opw, n, _ = W.generate(name, k)
        commit, vals, _ = bs[k].results()
        ref, rc, ro = O.replay(0, ref, tf, keys, opw, threads=THREADS)
        assert np.array_equal(commit, rc), k
        bad = np.nonzero(vals != ro)[0]
        assert len(bad) == 0, (k, len(bad), bad[:5])
    assert np.array_equal(ctx.download(t), ref)


def test_zipf_all_32_batches_from_one_graph():
    name = "zipf"
    sh = W.SHAPES[name]
    with G.Context(device=0) as ctx:
        t = ctx.create_table(sh["rows"], sh["cols"])
        ctx.fill_seeded(t, sh["seed"])
        bs = []
        for k in range(sh["batches"]):
            tf, keys, opw, n, fixed = W.generate(name, k)
            b = ctx.batch(n, len(keys))
            _load(b, tf, keys, opw, fixed, sh["rows"])
            bs.append(b)
        ctx.execute_many(bs, mode=G.MODE_GRAPH)
        _check_chain(ctx, t, sh, name, bs, sh["batches"], sh["seed"])


@pytest.mark.parametrize("mode", [G.MODE_GRAPH, G.MODE_PERSISTENT])
def test_uneven_64_batches(mode):
    name = "uneven"
    sh = W.SHAPES[name]
    with G.Context(device=0) as ctx:
        t = ctx.create_table(sh["rows"], sh["cols"])
        ctx.fill_seeded(t, sh["seed"])
        bs = []
        for k in range(sh["batches"]):
            tf, keys, opw, n, fixed = W.generate(name, k)
            b = ctx.batch(n, len(keys))
            _load(b, tf, keys, opw, fixed, sh["rows"])
            bs.append(b)
        ctx.execute_many(bs, mode=mode)
        _check_chain(ctx, t, sh, name, bs, sh["batches"], sh["seed"])


def test_order_entry_w64_batch_2_18():
    sh = W.SHAPES["tpcc"]
    g = G.Tpcc(sh["warehouses"], seed=sh["seed"])
    tf, keys, opw, pay, n_no, ins = g.gen(0, sh["batch"])
    with G.Context(device=0) as ctx:
        ids = g.create_tables(ctx, ins)
        b = ctx.batch(len(tf) - 1, len(keys))
        b.load(tf, keys.astype(np.uint32), opw)
        b.load_payload(pay)
        b.execute()
        commit, vals, st = b.results64()
        tabs = []
        for k in range(9):
            _, mask, r0 = g.table(k)
            tabs.append((g.initial(k, r0 + int(ins[k])), r0, mask))
        after, rc, ro = O.replay_tables(0, tabs, tf, keys, opw, pay, threads=THREADS)
        assert np.array_equal(commit, rc)
        bad = np.nonzero(vals != ro)[0]
        assert len(bad) == 0, (len(bad), bad[:5])
        for k, tid in enumerate(ids):
            assert ctx.table_rows(tid) == after[k][1], G.TPCC_TABLES[k]
            assert np.array_equal(ctx.download(tid), after[k][0][:, :after[k][1]]), G.TPCC_TABLES[k]
    assert st.contended_cells > 0


def test_serving_blend_full_size_tables_256_streams():
    """The serving configuration's blend on full-size tables: 2^17 Zipf 0.99
    YCSB transactions (2^24 x 10 table) and 2^17 order-entry transactions
    (W=64), served from the request log at 300 M txn/s offered (the merged
    arrivals of 256 Poisson streams), 250 us deadline, 4 GB budget."""
    zs = W.SHAPES["zipf"]
    ts = W.SHAPES["tpcc"]
    n_each = 1 << 17
    ycsb = G.gen_ycsb(zs["seed"], zs["rows"], zs["cols"], 16, 16, 0.8, 0.99, batch=0, n_txns=n_each)
    g = G.Tpcc(ts["warehouses"], seed=ts["seed"])
    tf_t, k_t, w_t, pay_t, _, ins_t, pf_t = g.gen(0, n_each, with_pay_first=True)
    tf, keys, opw, pf, pay, _ = W.mixed_pool(ycsb, (tf_t, k_t, w_t, pay_t, pf_t), seed=zs["seed"] + 1)
    n = len(tf) - 1
    extra = np.asarray(ins_t, np.int64)
    arr = G.lib.poisson_arrivals(n, 300e6, 7)
    with G.Context(device=0) as ctx:
        t0 = ctx.create_table(zs["rows"], zs["cols"])
        ctx.fill_seeded(t0, zs["seed"])
        ids = g.create_tables(ctx, extra)
        ing = G.Ingest(ctx, tf, keys, opw, pf, pay, deadline_us=250, depth=2, budget_bytes=4 << 30,
                       max_txns=1 << 20, max_ops=1 << 24, eager=True, keep_results=True, jit=True)
        st = ing.run(arr)
        committed, seq, pos, att, vals = ing.results(values=True)
        ing.close()
        finals = [ctx.download(t) for t in [t0] + ids]
    assert st["submitted"] == n and st["committed"] == n and committed.all()
    assert st["batches"] > 1
    # under the ordered rule the committed history is the log order
    assert np.array_equal(np.lexsort((pos, seq)), np.arange(n))
    tabs = [(O.table_init(zs["seed"], zs["rows"], zs["cols"]), zs["rows"])]
    for k in range(9):
        _, mask, r0 = g.table(k)
        tabs.append((g.initial(k, r0 + int(extra[k])), r0, mask))
    # the pool as one serial batch (its insert keys already index the whole payload)
    after, rc, out = O.replay_tables(0, tabs, tf, keys, opw, pay, threads=THREADS)
    bad = np.nonzero(vals != out[:len(vals)])[0]
    assert len(bad) == 0, (len(bad), bad[:5])
    for k, fin in enumerate(finals):
        assert np.array_equal(fin, after[k][0][:, :after[k][1]]), k
