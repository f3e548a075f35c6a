"""The YCSB-E workload (ltpmg_gb300/workloads.py): the reference's YCSB_E
query -- 9 scans of rows [r, r+2) and one insert -- expanded into reads of
every int column of the scanned rows and an insert whose columns hold the
tenth row id, as the compatibility layer expands it.  CPU: the shape of the
generated transactions.  GPU: two batches (the second scans a table the
first grew) equal the oracle's serial replay, values and table."""
import numpy as np
import pytest

from ltpmg_gb300 import workloads as W


def test_ycsbe_transactions_have_the_reference_shape():
    sh = W.SHAPES["ycsbe"]
    tf, keys, opw, pay, n, ins = W.ycsbe_batch(3, n_txns=500)
    cols = sh["cols"]
    assert n == 500 and ins[0] == 500 and len(pay) == 500 * cols
    for t in range(n):
        a, b = int(tf[t]), int(tf[t + 1])
        k, w = keys[a:b], opw[a:b]
        assert (w[-1] & 3) == 2 and int(k[-1]) == t * cols  # the insert and its payload row
        reads = k[:-1].reshape(-1, cols)
        assert np.all((w[:-1] & 3) == 0) and np.all((w[:-1].reshape(-1, cols) >> 2) == np.arange(cols))
        assert len(reads) <= 18 and np.all(reads == reads[:, :1])  # every column of each scanned row
        firsts = reads[:, 0]
        assert np.all(firsts < sh["rows"])
        # scans of [r, r+2): pairs (r, r+1), a row past the end dropped
        assert len(set(int(x) for x in firsts)) >= len(firsts) // 2
        assert np.all(pay[t * cols:(t + 1) * cols] == pay[t * cols])


@pytest.mark.gpu
@pytest.mark.parametrize("rule", [0, 1])
def test_ycsbe_batches_match_oracle(rule):
    import ltpmg_gb300 as G
    import oracle as O

    sh = W.SHAPES["ycsbe"]
    batches = [W.ycsbe_batch(b, n_txns=2000) for b in range(2)]
    cap = sh["rows"] + sum(int(x[5][0]) for x in batches)
    with G.Context(device=0, rule=rule) as ctx:
        t = ctx.create_table(sh["rows"], sh["cols"], rows_cap=cap)
        ctx.fill_seeded(t, sh["seed"])
        data = np.zeros((sh["cols"], cap), np.int32)
        data[:, :sh["rows"]] = O.table_init(sh["seed"], sh["rows"], sh["cols"])
        ref = [(data, sh["rows"])]
        for tf, keys, opw, pay, n, ins in batches:
            b = ctx.batch(n, len(keys))
            b.load(tf, keys.astype(np.uint32), opw)
            b.load_payload(pay)
            b.execute()
            commit, vals, st = b.results()
            ref, rc, ro = O.replay_tables(rule, ref, tf, keys, opw, pay)
            assert np.array_equal(commit, rc[:n]) and np.array_equal(vals, ro)
        assert ctx.table_rows(t) == ref[0][1]
        assert np.array_equal(ctx.download(t), ref[0][0][:, :ref[0][1]])
