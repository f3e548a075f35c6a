"""CUDA path vs the CPU oracle, through the C ABI (libltpmg_gb300.so).

Bit-exact comparison of the commit vector, every per-op value and the final
table for seeded workloads at reduced sizes, the full-size plain batch
(2^20 rows, 16 batches of 2^16 transactions x 10 ops) and full-size Zipf
batches (2^24 rows, 2^20 transactions x 16 ops), plus the edge cases the
reference's per-row ordering implies (one hot row, one hot cell, read-only,
write-only, single transaction, empty batch) and error paths.
"""
import json
import os

import numpy as np
import pytest

import ltpmg_gb300 as G
import oracle as O

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "seeded_workloads.json")
SEED = 0x4C54504D47


@pytest.fixture(scope="module")
def lib_loaded():
    return G.load()


def run_and_check(rule, rows, cols, batches, seed=SEED, fixed=0, ctx_kwargs=None, tab0=None, threads=0):
    """Executes the batches in order on a fresh context and compares each
    batch's outputs and the final table with the oracle."""
    with G.Context(device=0, rule=rule, **(ctx_kwargs or {})) as ctx:
        t = ctx.create_table(rows, cols)
        if tab0 is None:
            ctx.fill_seeded(t, seed)
            ref = O.table_init(seed, rows, cols)
        else:
            ctx.upload(t, tab0)
            ref = tab0.copy()
        maxops = max([len(k) for _, k, _ in batches] + [1])
        maxtx = max([len(tf) - 1 for tf, _, _ in batches] + [1])
        b = ctx.batch(maxtx, maxops)
        stats = []
        for tf, keys, opw in batches:
            if fixed:
                b.load(None, keys, opw, ops_per_txn=fixed)
            else:
                b.load(tf, keys, opw)
            b.execute()
            commit, vals, st = b.results()
            ref, rc, ro = O.replay(rule, ref, tf, keys, opw, threads=threads)
            assert np.array_equal(commit, rc), "commit vector differs"
            bad = np.nonzero(vals != ro)[0]
            assert len(bad) == 0, f"{len(bad)} op values differ, first at {bad[:5]}: {vals[bad[:5]]} vs {ro[bad[:5]]}"
            stats.append(st.as_dict())
        final = ctx.download(t)
        assert np.array_equal(final, ref), f"final table differs in {(final != ref).sum()} cells"
        return stats


def gen(seed, rows, cols, omin, omax, rf, th, b, n):
    return G.gen_ycsb(seed, rows, cols, omin, omax, rf, th, batch=b, n_txns=n)


@pytest.mark.parametrize("rule", [0, 1])
def test_golden_workloads(lib_loaded, rule):
    doc = json.load(open(GOLDEN))
    for w in doc["workloads"]:
        tf, keys, opw = gen(w["seed"], w["rows"], w["cols"], w["ops_min"], w["ops_max"], w["read_frac"], w["theta"],
                            w["batch"], w["txns"])
        assert O.fnv1a(keys) == w["fnv_keys"] and O.fnv1a(opw) == w["fnv_opw"]
        with G.Context(device=0, rule=rule) as ctx:
            t = ctx.create_table(w["rows"], w["cols"])
            ctx.fill_seeded(t, w["seed"])
            assert O.fnv1a(ctx.download(t)) == w["fnv_table_init"]
            b = ctx.batch(w["txns"], len(keys))
            b.load(tf, keys, opw)
            b.execute()
            commit, vals, st = b.results()
            exp = w[f"r{rule}"]
            assert O.fnv1a(commit) == exp["fnv_commit"], w["name"]
            assert O.fnv1a(vals) == exp["fnv_out"], w["name"]
            assert O.fnv1a(ctx.download(t)) == exp["fnv_table"], w["name"]
            assert st.committed == exp["committed"]


@pytest.mark.parametrize("rule", [0, 1])
@pytest.mark.parametrize("shape", [
    # rows, cols, ops_min, ops_max, read_frac, theta, txns, batches
    (1 << 12, 10, 10, 10, 0.5, 0.0, 4096, 3),
    (1 << 14, 10, 16, 16, 0.8, 0.99, 4096, 3),
    (1 << 14, 10, 1, 32, 0.7, 0.75, 3000, 3),
    (64, 4, 1, 32, 0.3, 1.2, 2000, 2),
    (1 << 16, 1, 8, 8, 0.5, 0.99, 8192, 2),
    (1 << 10, 64, 4, 12, 0.2, 0.9, 5000, 2),
])
def test_seeded_sequences(lib_loaded, rule, shape):
    rows, cols, omin, omax, rf, th, txns, nb = shape
    batches = [gen(SEED + 11, rows, cols, omin, omax, rf, th, b, txns) for b in range(nb)]
    run_and_check(rule, rows, cols, batches, seed=SEED + 11)


@pytest.mark.parametrize("rule", [0, 1])
def test_fixed_length_path(lib_loaded, rule):
    rows, cols = 1 << 13, 10
    batches = [gen(3, rows, cols, 16, 16, 0.8, 0.99, b, 4096) for b in range(2)]
    run_and_check(rule, rows, cols, batches, seed=3, fixed=16)


def _manual(txn_ops):
    """txn_ops: list of transactions, each a list of (key, kind, col, imm)."""
    tf = [0]
    keys, opw = [], []
    for ops in txn_ops:
        for key, kind, col, imm in ops:
            keys.append(key)
            opw.append(O.opword(kind, col, 0, imm))
        tf.append(len(keys))
    return np.array(tf, np.uint32), np.array(keys, np.uint64), np.array(opw, np.uint32)


@pytest.mark.parametrize("rule", [0, 1])
def test_edge_cases(lib_loaded, rule):
    rows, cols = 256, 3
    rng = np.random.default_rng(5)
    cases = []
    # one hot cell: every op of every transaction on (row 7, col 1)
    cases.append(_manual([[(7, int(rng.random() < 0.5), 1, int(rng.integers(-5, 6)))] for _ in range(5000)]))
    # one hot row, all columns, all RMW
    cases.append(_manual([[(3, 1, c, 1) for c in range(3)] for _ in range(3000)]))
    # read only
    cases.append(_manual([[(int(r), 0, int(r) % 3, 0) for r in rng.choice(rows, 8, replace=False)] for _ in range(500)]))
    # write only, large immediates (wrap-around)
    cases.append(_manual([[(int(r), 1, 0, 524287 if r % 2 else -524288) for r in rng.choice(rows, 4, replace=False)]
                          for _ in range(2000)]))
    # a single transaction
    cases.append(_manual([[(1, 1, 0, 3), (2, 0, 1, 0), (3, 1, 2, -1)]]))
    # transactions with no ops in between
    cases.append(_manual([[], [(5, 1, 0, 1)], [], [(5, 0, 0, 0)], []]))
    tab0 = np.arange(rows * cols, dtype=np.int64).reshape(cols, rows).astype(np.int32) * 7 - 100
    tab0[0, 10] = 2 ** 31 - 1
    run_and_check(rule, rows, cols, cases, tab0=tab0)


def test_empty_batch(lib_loaded):
    with G.Context(device=0) as ctx:
        t = ctx.create_table(100, 2)
        ctx.fill_seeded(t, 1)
        before = ctx.download(t)
        b = ctx.batch(4, 16)
        b.load(np.zeros(1, np.uint32), np.zeros(0, np.uint64), np.zeros(0, np.uint32))
        b.execute()
        commit, vals, st = b.results()
        assert len(commit) == 0 and len(vals) == 0 and st.ops == 0
        assert np.array_equal(before, ctx.download(t))


@pytest.mark.parametrize("block,ipt,flags,word_bits",
                         [(b, i, 0, 32) for b in (128, 256, 512) for i in (1, 2, 4, 8)] +
                         [(b, i, 0, 64) for b in (128, 256, 512) for i in (1, 2, 4, 8) if b * i <= 2048] +
                         [(512, 4, G.lib.TUNE_MARK_PRECHECK, 32), (128, 1, G.lib.TUNE_MARK_PRECHECK, 32),
                          (256, 4, G.lib.TUNE_MARK_PRECHECK, 64)])
def test_tuning_variants(lib_loaded, block, ipt, flags, word_bits):
    rows, cols = 1 << 12, 10
    with G.Context(device=0) as ctx:
        t = ctx.create_table(rows, cols)
        ctx.fill_seeded(t, 21)
        for bucket in range(64):
            ctx.set_tuning(bucket, block, ipt, word_bits=word_bits, flags=flags)
        assert ctx.get_tuning(5) == (block, ipt, word_bits, flags)
        b = ctx.batch(3000, 3000 * 32)
        ref_tab = O.table_init(21, rows, cols)
        for batch in range(2):  # the second batch sees hot words already marked by the first's tiles
            tf, keys, opw = gen(21, rows, cols, 1, 32, 0.7, 0.95, batch, 3000)
            ref_tab, rc, ro = O.replay(0, ref_tab, tf, keys, opw)
            b.load(tf, keys, opw)
            b.execute()
            commit, vals, st = b.results()
            assert np.array_equal(vals, ro)
        assert np.array_equal(ctx.download(t), ref_tab)


@pytest.mark.parametrize("rule", [0, 1])
def test_word_widths_alternate_on_one_context(lib_loaded, rule):
    """Batches of two size buckets, one tuned to 32-cell and one to 64-cell
    conflict words, alternate on one context (both widths share the conflict
    state buffer, each batch leaves it clean), under both rules; a table of
    2^16 + 5 rows x 7 columns puts cells of one 64-cell word in two rows'
    tails and the last word partly past the table."""
    rows, cols = (1 << 16) + 5, 7
    with G.Context(device=0, rule=rule) as ctx:
        t = ctx.create_table(rows, cols)
        ctx.fill_seeded(t, 23)
        small, large = 2000, 20000
        ctx.set_tuning(int(np.log2(small * 8)), 256, 2, word_bits=64)
        ctx.set_tuning(int(np.log2(large * 8)), 512, 4, word_bits=32)
        ref_tab = O.table_init(23, rows, cols)
        for batch in range(6):
            n = small if batch % 2 == 0 else large
            tf, keys, opw = gen(23, rows, cols, 8, 8, 0.6, 1.1, batch, n)
            ref_tab, rc, ro = O.replay(rule, ref_tab, tf, keys, opw)
            b = ctx.batch(n, len(keys))
            b.load(tf, keys, opw)
            b.execute()
            commit, vals, st = b.results()
            assert np.array_equal(commit, rc[:n]) and np.array_equal(vals, ro), batch
            if rule == 1:
                assert st.aborted > 0
        assert np.array_equal(ctx.download(t), ref_tab)


def test_tuning_rejects_unbuilt_tilings(lib_loaded):
    with G.Context(device=0) as ctx:
        with pytest.raises(G.LtpError):  # 64-cell words fit tiles of at most 2048 ops
            ctx.set_tuning(3, 512, 8, word_bits=64)
        with pytest.raises(G.LtpError):
            ctx.set_tuning(3, 256, 4, word_bits=16)
        ctx.set_tuning(3, 512, 4, word_bits=64)
        assert ctx.get_tuning(3) == (512, 4, 64, 0)


def test_malformed_op_rejected_and_context_survives(lib_loaded):
    rows, cols = 128, 2
    with G.Context(device=0) as ctx:
        t = ctx.create_table(rows, cols)
        ctx.fill_seeded(t, 9)
        before = ctx.download(t)
        b = ctx.batch(8, 64)
        tf, keys, opw = _manual([[(1, 1, 0, 1), (rows + 5, 1, 1, 1)], [(2, 1, 1, 1)]])
        b.load(tf, keys, opw)
        b.execute()
        with pytest.raises(G.LtpError) as ei:
            b.results()
        assert ei.value.status == G.lib.LTP_E_BADARG and "index 1" in str(ei.value)
        assert np.array_equal(before, ctx.download(t)), "a rejected batch must not change the table"
        tf, keys, opw = _manual([[(1, 1, 0, 1)], [(1, 0, 0, 0)]])
        b.load(tf, keys, opw)
        b.execute()
        commit, vals, _ = b.results()
        assert vals.tolist() == [int(before[0, 1]) + 1, int(before[0, 1]) + 1]


@pytest.mark.parametrize("rule", [0, 1])
def test_dense_batches_build_no_list_and_recover_from_errors(lib_loaded, rule):
    """Batches with at least twice as many ops as conflict words take the
    path on which mark builds no touched-word list (ids and finish visit
    every word).  A malformed op in such a batch is rejected with the table
    unchanged, and the sparse and dense batches after it still equal the
    oracle: every word the failed batch marked was cleared."""
    rows, cols = 1 << 10, 4  # 4096 cells: 129 conflict words of 32 cells
    dense = gen(11, rows, cols, 4, 8, 0.6, 0.9, 0, 400)  # ~2400 ops >= 2 x 129
    sparse = gen(11, rows, cols, 1, 2, 0.6, 0.9, 1, 40)  # ~60 ops: the list path
    assert len(dense[1]) >= 2 * 129 and len(sparse[1]) < 2 * 129
    with G.Context(device=0, rule=rule) as ctx:
        t = ctx.create_table(rows, cols)
        ctx.fill_seeded(t, 11)
        ref = O.table_init(11, rows, cols)
        b = ctx.batch(400, len(dense[1]))

        def run(tf, keys, opw):
            nonlocal ref
            b.load(tf, keys, opw)
            b.execute()
            commit, vals, st = b.results()
            ref, rc, ro = O.replay(rule, ref, tf, keys, opw)
            assert np.array_equal(commit, rc) and np.array_equal(vals, ro)
            return st

        assert run(*dense).touched_words > 0
        tf, keys, opw = dense
        bad = keys.copy()
        bad[len(bad) // 2] = rows + 3  # a row past the table, mid-batch
        before = ctx.download(t)
        b.load(tf, bad, opw)
        b.execute()
        with pytest.raises(G.LtpError) as ei:
            b.results()
        assert ei.value.status == G.lib.LTP_E_BADARG
        assert np.array_equal(before, ctx.download(t)), "a rejected batch must not change the table"
        run(*sparse)
        run(*dense)
        assert np.array_equal(ctx.download(t), ref)


def test_bad_column_and_table(lib_loaded):
    with G.Context(device=0) as ctx:
        t = ctx.create_table(64, 2)
        ctx.fill_seeded(t, 2)
        b = ctx.batch(4, 4)
        for w in (O.opword(0, 5, 0, 0), O.opword(0, 0, 3, 0), 3):
            b.load(np.array([0, 1], np.uint32), np.array([1], np.uint64), np.array([w], np.uint32))
            b.execute()
            with pytest.raises(G.LtpError):
                b.results()


def test_timeout_status_and_recovery(lib_loaded):
    """The debug stall makes the first stage poll a flag nothing sets; it gives
    up after ~200 ms and the batch reports LTP_E_TIMEOUT.  No GPU fault."""
    rows, cols = 1 << 10, 4
    tf, keys, opw = gen(4, rows, cols, 4, 4, 0.5, 0.9, 0, 500)
    with G.Context(device=0) as ctx:
        t = ctx.create_table(rows, cols)
        ctx.fill_seeded(t, 4)
        b = ctx.batch(500, len(keys))
        b.load(tf, keys, opw)
        ctx.stall_next(200)
        b.execute()
        with pytest.raises(G.LtpError) as ei:
            b.results()
        assert ei.value.status == G.lib.LTP_E_TIMEOUT
        # the context is still usable and the failed batch changed nothing
        b.execute()
        commit, vals, _ = b.results()
        ref_tab, rc, ro = O.replay(0, O.table_init(4, rows, cols), tf, keys, opw)
        assert np.array_equal(vals, ro) and np.array_equal(ctx.download(t), ref_tab)


def test_two_tables(lib_loaded):
    with G.Context(device=0) as ctx:
        a = ctx.create_table(1000, 3)
        bt = ctx.create_table(77, 5)
        ctx.fill_seeded(a, 1)
        ctx.fill_seeded(bt, 2)
        ta, tb = O.table_init(1, 1000, 3), O.table_init(2, 77, 5)
        rng = np.random.default_rng(3)
        keys, opw, tf = [], [], [0]
        for t in range(3000):
            for j in range(4):
                if rng.random() < 0.5:
                    keys.append(int(rng.integers(0, 1000))); opw.append(O.opword(int(rng.random() < 0.4), int(rng.integers(0, 3)), 0, 1))
                else:
                    keys.append(int(rng.integers(0, 77))); opw.append(O.opword(int(rng.random() < 0.4), int(rng.integers(0, 5)), 1, 2))
            tf.append(len(keys))
        b = ctx.batch(3000, len(keys))
        b.load(np.array(tf, np.uint32), np.array(keys, np.uint64), np.array(opw, np.uint32))
        b.execute()
        commit, vals, _ = b.results()
        # serial replay over two tables
        exp = np.zeros(len(keys), np.int32)
        tabs = [ta.copy(), tb.copy()]
        for i, (k, w) in enumerate(zip(keys, opw)):
            tt, col, kind, imm = (w >> 8) & 15, (w >> 2) & 63, w & 3, ((w >> 12) ^ 0x80000) - 0x80000
            v = int(tabs[tt][col, k])
            if kind == 1:
                v = ((v + imm + 2 ** 31) % 2 ** 32) - 2 ** 31
                tabs[tt][col, k] = v
            exp[i] = v
        assert np.array_equal(vals, exp)
        assert np.array_equal(ctx.download(a), tabs[0]) and np.array_equal(ctx.download(bt), tabs[1])


def test_full_size_plain_batches(lib_loaded):
    """Plain batch workload at full size: 2^20 rows x 10 int32, 16 batches of
    2^16 transactions x 10 ops, uniform keys, 50% read / 50% +1 RMW."""
    rows, cols = 1 << 20, 10
    batches = [gen(SEED, rows, cols, 10, 10, 0.5, 0.0, b, 1 << 16) for b in range(16)]
    run_and_check(0, rows, cols, batches, fixed=10, threads=8)


@pytest.mark.parametrize("rule", [0, 1])
def test_full_size_zipf_batches(lib_loaded, rule):
    """High-contention workload at full size: 2^24 rows x 10 int32, batches of
    2^20 transactions x 16 ops, Zipf 0.99 keys, 80% read / 20% RMW."""
    rows, cols = 1 << 24, 10
    batches = [gen(SEED + 2, rows, cols, 16, 16, 0.8, 0.99, b, 1 << 20) for b in range(2 if rule == 0 else 1)]
    stats = run_and_check(rule, rows, cols, batches, seed=SEED + 2, fixed=16, threads=8 if rule == 0 else 0)
    assert stats[0]["contended_ops"] > 0 and stats[0]["contended_cells"] > 0


def _insert_batch(rng, tables, n_txns, p_ins=0.3, max_ops=8):
    """Random multi-table batch mixing reads, RMWs and inserts (payload rows)."""
    tf, keys, opw, payload = [0], [], [], []
    for _ in range(n_txns):
        used = set()
        for _ in range(int(rng.integers(1, max_ops + 1))):
            tb = int(rng.integers(0, len(tables)))
            rows, cols = tables[tb]
            if rng.random() < p_ins:
                keys.append(len(payload))
                opw.append(O.opword(2, 0, tb, 0))
                payload += [int(x) for x in rng.integers(-1000, 1000, cols)]
                continue
            r = int(rng.integers(0, min(rows, 24)) if rng.random() < 0.5 else rng.integers(0, rows))
            c = int(rng.integers(0, cols))
            if (tb, r, c) in used:
                continue
            used.add((tb, r, c))
            keys.append(r)
            opw.append(O.opword(int(rng.random() < 0.4), c, tb, int(rng.integers(-3, 4))))
        tf.append(len(keys))
    return (np.array(tf, np.uint32), np.array(keys, np.uint64), np.array(opw, np.uint32),
            np.array(payload or [0], np.int32))


@pytest.mark.parametrize("rule", [0, 1])
def test_inserts_two_tables_sequence(lib_loaded, rule):
    rng = np.random.default_rng(42 + rule)
    shapes = [(500, 3), (64, 5)]
    with G.Context(device=0, rule=rule) as ctx:
        ids, ref = [], []
        for k, (rows, cols) in enumerate(shapes):
            tid = ctx.create_table(rows, cols, rows_cap=rows + 20000)
            ctx.fill_seeded(tid, 7 + k)
            data = np.zeros((cols, rows + 20000), np.int32)
            data[:, :rows] = O.table_init(7 + k, rows, cols)
            ids.append(tid)
            ref.append((data, rows))
        b = ctx.batch(4000, 4000 * 8)
        cur = list(shapes)
        for step in range(3):
            tf, keys, opw, payload = _insert_batch(rng, cur, 3000)
            b.load(tf, keys, opw)
            b.load_payload(payload)
            b.execute()
            commit, vals, st = b.results()
            ref, rc, ro = O.replay_tables(rule, ref, tf, keys, opw, payload)
            assert np.array_equal(commit, rc)
            assert np.array_equal(vals, ro)
            cur = [(ref[k][1], shapes[k][1]) for k in range(2)]
            for k, tid in enumerate(ids):
                assert ctx.table_rows(tid) == ref[k][1]
                assert np.array_equal(ctx.download(tid), ref[k][0][:, :ref[k][1]])


@pytest.mark.parametrize("layout", ["reversed", "gaps", "half_shuffled"])
def test_inserts_scattered_payload_rows(lib_loaded, layout):
    """Insert rows placed anywhere in the payload (reversed, separated by
    unused words, shuffled in half the batch): tiles whose rows span more
    than the kernel's payload stage read them from global memory, the others
    through the stage; both must give the serial replay's tables."""
    rng = np.random.default_rng(77)
    shapes = [(500, 3), (64, 5)]
    with G.Context(device=0) as ctx:
        ids, ref = [], []
        for k, (rows, cols) in enumerate(shapes):
            tid = ctx.create_table(rows, cols, rows_cap=rows + 20000)
            ctx.fill_seeded(tid, 7 + k)
            data = np.zeros((cols, rows + 20000), np.int32)
            data[:, :rows] = O.table_init(7 + k, rows, cols)
            ids.append(tid)
            ref.append((data, rows))
        tf, keys, opw, payload = _insert_batch(rng, list(shapes), 6000, p_ins=0.4)
        ins = np.nonzero((opw & 3) == 2)[0]
        width = [shapes[(int(opw[i]) >> 8) & 15][1] for i in ins]
        rows_ = [payload[int(keys[i]):int(keys[i]) + w] for i, w in zip(ins, width)]
        order = np.arange(len(ins))
        if layout == "reversed":
            order = order[::-1]
        elif layout == "half_shuffled":
            h = len(order) // 2
            order[:h] = rng.permutation(order[:h])
        new_pay, new_keys = [], keys.copy()
        for j in order:
            if layout == "gaps" and rng.random() < 0.05:
                new_pay.extend(rng.integers(-9, 9, int(rng.integers(1000, 6000))).tolist())
            new_keys[ins[j]] = len(new_pay)
            new_pay.extend(rows_[j].tolist())
        payload = np.array(new_pay, np.int32)
        b = ctx.batch(6000, len(keys))
        b.load(tf, new_keys, opw)
        b.load_payload(payload)
        b.execute()
        commit, vals, st = b.results()
        ref, rc, ro = O.replay_tables(0, ref, tf, new_keys, opw, payload)
        assert np.array_equal(commit, rc) and np.array_equal(vals, ro)
        for k, tid in enumerate(ids):
            assert ctx.table_rows(tid) == ref[k][1]
            assert np.array_equal(ctx.download(tid), ref[k][0][:, :ref[k][1]])


def test_insert_capacity_and_payload_errors(lib_loaded):
    with G.Context(device=0) as ctx:
        t = ctx.create_table(10, 2, rows_cap=12)
        ctx.fill_seeded(t, 1)
        before = ctx.download(t)
        b = ctx.batch(8, 8)
        ins = O.opword(2, 0, 0, 0)
        # three inserts into a table with room for two: rejected, table unchanged
        b.load(np.array([0, 1, 2, 3], np.uint32), np.array([0, 2, 4], np.uint64), np.array([ins] * 3, np.uint32))
        b.load_payload(np.arange(6, dtype=np.int32))
        b.execute()
        with pytest.raises(G.LtpError) as ei:
            b.results()
        assert ei.value.status == G.lib.LTP_E_CAPACITY
        assert ctx.table_rows(t) == 10 and np.array_equal(ctx.download(t), before)
        # payload too short for the row: malformed
        b.load(np.array([0, 1], np.uint32), np.array([5], np.uint64), np.array([ins], np.uint32))
        b.load_payload(np.arange(6, dtype=np.int32))
        b.execute()
        with pytest.raises(G.LtpError) as ei:
            b.results()
        assert ei.value.status == G.lib.LTP_E_BADARG
        # two inserts fit
        b.load(np.array([0, 1, 2], np.uint32), np.array([0, 2], np.uint64), np.array([ins] * 2, np.uint32))
        b.load_payload(np.array([5, 6, 7, 8], np.int32))
        b.execute()
        commit, vals, _ = b.results()
        assert vals.tolist() == [10, 11]
        after = ctx.download(t)
        assert after.shape == (2, 12) and after[:, 10].tolist() == [5, 6] and after[:, 11].tolist() == [7, 8]


@pytest.mark.parametrize("rule", [0, 1])
@pytest.mark.parametrize("mode", [G.lib.MODE_STREAM, G.lib.MODE_GRAPH, G.lib.MODE_PERSISTENT])
def test_multi_batch_modes(lib_loaded, rule, mode):
    """Uneven batches (sizes, ops per transaction and skew vary per batch) run
    through one multi-batch call, twice with new contents of the same sizes
    (the second call replays the cached graph), against the oracle."""
    rows, cols, seed = 1 << 14, 10, 99
    shapes = [(1 << 10, 1, 32, 0.5), (3000, 1, 32, 0.99), (200, 4, 4, 0.8), (1 << 12, 16, 16, 0.7), (1, 1, 1, 0.9)]
    with G.Context(device=0, rule=rule) as ctx:
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
                ref, rc, ro = O.replay(rule, ref, tf, keys, opw)
                assert np.array_equal(commit, rc)
                assert np.array_equal(vals, ro)
            assert np.array_equal(ctx.download(t), ref)


def test_persistent_mode_with_inserts(lib_loaded):
    rng = np.random.default_rng(5)
    with G.Context(device=0) as ctx:
        t = ctx.create_table(300, 4, rows_cap=300 + 5000)
        ctx.fill_seeded(t, 3)
        data = np.zeros((4, 5300), np.int32)
        data[:, :300] = O.table_init(3, 300, 4)
        ref = [(data, 300)]
        bs, batches = [], []
        cur = [(300, 4)]
        for k in range(3):
            tf, keys, opw, payload = _insert_batch(rng, cur, 800, p_ins=0.2)
            # keys of reads/RMWs must name rows that exist before this batch
            b = ctx.batch(800, len(keys))
            b.load(tf, keys, opw)
            b.load_payload(payload)
            bs.append(b)
            batches.append((tf, keys, opw, payload))
        ctx.execute_many(bs, mode=G.lib.MODE_PERSISTENT)
        for (tf, keys, opw, payload), b in zip(batches, bs):
            commit, vals, _ = b.results()
            ref, rc, ro = O.replay_tables(0, ref, tf, keys, opw, payload)
            assert np.array_equal(vals, ro)
        assert ctx.table_rows(t) == ref[0][1]
        assert np.array_equal(ctx.download(t), ref[0][0][:, :ref[0][1]])


@pytest.mark.parametrize("rule", [0, 1])
@pytest.mark.parametrize("persistent", [False, True])
def test_pipeline_matches_oracle(lib_loaded, rule, persistent):
    """Batches submitted through the 3-deep pipeline (overlapped copy-in,
    execution, copy-out; each batch as a kernel sequence or as one
    persistent-kernel launch) give the serial replay of the whole sequence."""
    rows, cols, seed = 1 << 13, 10, 17
    with G.Context(device=0, rule=rule) as ctx:
        t = ctx.create_table(rows, cols)
        ctx.fill_seeded(t, seed)
        ref = O.table_init(seed, rows, cols)
        pipe = G.Pipe(ctx, 3, 4096, 4096 * 32, persistent=persistent)
        subs, pinned = [], []
        for k in range(7):
            n = [4096, 100, 2000, 1, 3000, 4096, 512][k]
            tf, keys, opw = gen(seed, rows, cols, 1, 32, 0.7, 0.9, k, n)
            if k % 2:
                pinned.append(G.PinnedArray((n,), np.uint8))
                commit = pinned[-1].array
            else:
                commit = np.zeros(n, np.uint8)
            vals = np.zeros(len(keys), np.int32)
            subs.append((pipe.submit(tf, keys, opw, commit, vals), tf, keys, opw, commit, vals))
        for tk, tf, keys, opw, commit, vals in subs:
            st = pipe.wait(tk)
            ref, rc, ro = O.replay(rule, ref, tf, keys, opw)
            assert np.array_equal(commit, rc) and np.array_equal(vals, ro)
            assert st.ops == len(keys)
        pipe.close()
        assert np.array_equal(ctx.download(t), ref)


def test_largest_table_row_ids(lib_loaded):
    """A table at the row limit (2^31 rows x 1 int32 column, 8 GiB): ops on
    the last rows and on row 0 share the batch; every index past 2^31 cells
    stays exact (row ids, cell numbers, conflict words)."""
    rows = 1 << 31
    with G.Context(device=0) as ctx:
        t = ctx.create_table(rows, 1)
        hi = np.array([rows - 1, rows - 2, rows - 33, 0, 1], np.uint64)
        init = np.array([7, -5, 2**31 - 1, 11, 0], np.int32)
        for r, v in zip(hi, init):
            ctx.upload_column(t, 0, np.array([v], np.int32), row0=int(r))
        # 3 transactions: RMWs and reads on the boundary rows, some cells shared
        tf = np.array([0, 3, 6, 8], np.uint32)
        keys = np.array([rows - 1, rows - 33, 0, rows - 1, rows - 2, 1, rows - 33, rows - 1], np.uint64)
        opw = np.array([O.opword(1, 0, 0, 3), O.opword(1, 0, 0, 1), O.opword(0, 0, 0, 0),
                        O.opword(0, 0, 0, 0), O.opword(1, 0, 0, -2), O.opword(1, 0, 0, 9),
                        O.opword(0, 0, 0, 0), O.opword(1, 0, 0, 100)], np.uint32)
        b = ctx.batch(3, 8)
        b.load(tf, keys, opw)
        b.execute()
        commit, vals, st = b.results()
        cells = {int(r): int(v) for r, v in zip(hi, init)}
        expect = []
        for k, w in zip(keys, opw):
            imm = int(np.int32(np.uint32(w) >> np.uint32(12) << np.uint32(12)) >> 12) if (w & 3) == 1 else 0
            cells[int(k)] = int(np.int32(np.uint32((cells[int(k)] + imm) & 0xFFFFFFFF)))
            expect.append(cells[int(k)])
        assert list(vals) == expect and st.contended_cells == 2
        out = np.zeros(1, np.int32)
        for r in hi:
            G.lib.load().ltp_table_download(ctx.h, t, 0, int(r), 1, out.ctypes.data)
            assert out[0] == cells[int(r)]


@pytest.mark.parametrize("rule", [0, 1])
def test_pipeline_replays_captured_graphs(lib_loaded, rule):
    """Batches of one shape through the pipeline: from the second batch of
    that shape on a slot, the slot replays a captured CUDA graph; values and
    the table still equal the serial replay, and a shape change falls back
    to launches."""
    rows, cols, seed = 1 << 13, 10, 18
    with G.Context(device=0, rule=rule) as ctx:
        t = ctx.create_table(rows, cols)
        ctx.fill_seeded(t, seed)
        ref = O.table_init(seed, rows, cols)
        pipe = G.Pipe(ctx, 3, 2048, 2048 * 16)
        subs = []
        for k in range(11):
            n = 2048 if k != 7 else 1000  # one shape change in the middle
            tf, keys, opw = gen(seed, rows, cols, 16, 16, 0.7, 0.9, k, n)
            commit = np.zeros(n, np.uint8)
            vals = np.zeros(len(keys), np.int32)
            subs.append((pipe.submit(None, keys, opw, commit, vals, ops_per_txn=16), tf, keys, opw, commit, vals))
        for tk, tf, keys, opw, commit, vals in subs:
            pipe.wait(tk)
            ref, rc, ro = O.replay(rule, ref, tf, keys, opw)
            assert np.array_equal(commit, rc) and np.array_equal(vals, ro)
        pipe.close()
        assert np.array_equal(ctx.download(t), ref)


@pytest.mark.parametrize("rule", [0, 1])
@pytest.mark.parametrize("mode", [G.lib.MODE_STREAM, G.lib.MODE_GRAPH, G.lib.MODE_PERSISTENT])
def test_32_bit_keys(lib_loaded, rule, mode):
    """Batches loaded with 32-bit keys (ltp_batch_load32), fixed- and
    variable-length, in every multi-batch mode, alternating with 64-bit
    loads of the same batch objects (the cached graph and persistent
    descriptors must follow the key width), equal the oracle."""
    rows, cols, seed = 1 << 14, 10, 77
    with G.Context(device=0, rule=rule) as ctx:
        t = ctx.create_table(rows, cols)
        ctx.fill_seeded(t, seed)
        ref = O.table_init(seed, rows, cols)
        bs = [ctx.batch(3000, 3000 * 16), ctx.batch(2000, 2000 * 8)]
        for rep in range(4):
            data = []
            for k, b in enumerate(bs):
                fixed = k == 1
                tf, keys, opw = gen(seed + rep, rows, cols, 8 if fixed else 1, 8 if fixed else 16, 0.7, 0.95, k,
                                    2000 if fixed else 3000)
                kk = keys.astype(np.uint32) if (rep + k) % 2 == 0 else keys
                b.load(None if fixed else tf, kk, opw, ops_per_txn=8 if fixed else 0)
                data.append((tf, keys, opw))
            ctx.execute_many(bs, mode=mode)
            for (tf, keys, opw), b in zip(data, bs):
                commit, vals, st = b.results()
                ref, rc, ro = O.replay(rule, ref, tf, keys, opw)
                assert np.array_equal(commit, rc) and np.array_equal(vals, ro), rep
        assert np.array_equal(ctx.download(t), ref)


def test_pipeline_with_32_bit_keys(lib_loaded):
    rows, cols, seed = 1 << 13, 10, 19
    with G.Context(device=0) as ctx:
        t = ctx.create_table(rows, cols)
        ctx.fill_seeded(t, seed)
        ref = O.table_init(seed, rows, cols)
        pipe = G.Pipe(ctx, 3, 2048, 2048 * 16)
        subs = []
        for k in range(8):
            tf, keys, opw = gen(seed, rows, cols, 16, 16, 0.7, 0.9, k, 2048)
            commit, vals = np.zeros(2048, np.uint8), np.zeros(len(keys), np.int32)
            kk = keys.astype(np.uint32) if k % 3 else keys
            subs.append((pipe.submit(None, kk, opw, commit, vals, ops_per_txn=16), tf, keys, opw, commit, vals))
        for tk, tf, keys, opw, commit, vals in subs:
            pipe.wait(tk)
            ref, rc, ro = O.replay(0, ref, tf, keys, opw)
            assert np.array_equal(vals, ro)
        pipe.close()
        assert np.array_equal(ctx.download(t), ref)


def _pattern_batch(pattern, n_ops, rows, cols, rng):
    """n_ops single- and multi-op transactions over a key pattern."""
    if pattern == "same_cell":
        keys = np.full(n_ops, 7, np.uint64)
        cols_ = np.zeros(n_ops, np.uint32)
    elif pattern == "distinct":
        cells = rng.permutation(rows * cols)[:n_ops]
        keys, cols_ = (cells // cols).astype(np.uint64), (cells % cols).astype(np.uint32)
    elif pattern == "skewed":
        keys = np.minimum(rng.zipf(1.3, n_ops) - 1, rows - 1).astype(np.uint64)
        cols_ = rng.integers(0, 2, n_ops).astype(np.uint32)
    else:  # two hot cells in one conflict word, the rest distinct rows
        keys = np.where(rng.random(n_ops) < 0.5, rng.integers(0, 2, n_ops), rng.integers(2, rows, n_ops))
        keys, cols_ = keys.astype(np.uint64), np.zeros(n_ops, np.uint32)
    kind = (rng.random(n_ops) < 0.5).astype(np.uint32)
    imm = rng.integers(-3, 4, n_ops).astype(np.int64)
    opw = np.array([O.opword(int(k), int(c), 0, int(i) if k else 0) for k, c, i in zip(kind, cols_, imm)], np.uint32)
    cuts = np.unique(np.concatenate([[0, n_ops], rng.integers(0, n_ops + 1, max(1, n_ops // 3))]))
    return cuts.astype(np.uint32), keys, opw


@pytest.mark.parametrize("n_ops", [1, 63, 64, 65, 2047, 2048, 2049, 3071, 3072, 3073, 4097, 12289])
@pytest.mark.parametrize("pattern", ["same_cell", "distinct", "skewed", "hot_pair"])
def test_tile_boundaries_and_adversarial_keys(lib_loaded, n_ops, pattern):
    """Batch sizes around every tile edge of the kernels (warps of 32, the
    2048-op mark/classify/apply/insert/id tiles, the 3072-record sort tile)
    with adversarial key patterns -- every op on one cell, every op on its
    own cell, Zipf 1.3 skew, two hot cells sharing a conflict word -- under
    both rules, loaded with 64- and then 32-bit keys."""
    rows, cols = 1 << 12, 4
    rng = np.random.default_rng(n_ops * 31 + len(pattern))
    tf, keys, opw = _pattern_batch(pattern, n_ops, rows, cols, rng)
    for rule in (0, 1):
        with G.Context(device=0, rule=rule) as ctx:
            t = ctx.create_table(rows, cols)
            ctx.fill_seeded(t, 5)
            ref = O.table_init(5, rows, cols)
            b = ctx.batch(len(tf) - 1, n_ops)
            for kk in (keys, keys.astype(np.uint32)):
                b.load(tf, kk, opw)
                b.execute()
                commit, vals, st = b.results()
                ref, rc, ro = O.replay(rule, ref, tf, keys, opw)
                assert np.array_equal(commit, rc[:len(tf) - 1]) and np.array_equal(vals, ro), (rule, kk.dtype)
            assert np.array_equal(ctx.download(t), ref)
