"""Seeded synthetic workloads with the shapes of the benchmark configurations.

They stand in for YCSB / TPC-C inputs (no suite items are used): the
library's generator draws keys, op kinds and columns from per-transaction
SplitMix64 streams, so every batch is reproducible from (seed, batch index).

plain   2^20 rows x 10 int32, batches of 2^16 transactions x 10 ops, uniform
        keys, 50% reads / 50% +1 read-modify-writes, 16 batches
zipf    2^24 rows x 10 int32, batches of 2^20 transactions x 16 ops, Zipf 0.99
        keys over a seeded permutation, 80% / 20%, 32 batches
uneven  2^24 rows x 10 int32, 64 batches of 2^U[10,20] transactions (log-
        uniform), 1-32 ops per transaction, Zipf theta ~ U[0.5, 0.99] per
        batch, 70% / 30%
tpcc    TPC-C-shaped order entry, 64 warehouses (10 districts, 30,000
        customers, 100,000 stock rows each; 100,000 items), batches of 2^18
        transactions, 50% new-order (5-15 lines) / 50% payment (the library's
        ltp_tpcc generator), 4 batches per step
"""
import math

from . import lib as L

SEED = 0x4C54504D47

SHAPES = {
    "plain": dict(rows=1 << 20, cols=10, batches=16, seed=SEED),
    "zipf": dict(rows=1 << 24, cols=10, batches=32, seed=SEED + 2),
    "uneven": dict(rows=1 << 24, cols=10, batches=64, seed=SEED + 4),
    "tpcc": dict(warehouses=64, batch=1 << 18, batches=4, seed=SEED + 6),
    # the reference's YCSB_E query (cuda/src/gpuquery.cu:3234-3303): 9 scans
    # of rows [r, r+2) and one insert, over the int attributes of its YCSB
    # schema (a, d, g: 3 int32 columns), rows drawn Zipf 0.99
    "ycsbe": dict(rows=1 << 20, cols=3, batch=1 << 16, batches=16, theta=0.99, seed=SEED + 8),
}


def _mix(z):
    z &= 0xFFFFFFFFFFFFFFFF
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & 0xFFFFFFFFFFFFFFFF
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & 0xFFFFFFFFFFFFFFFF
    return z ^ (z >> 31)


def batch_params(name, b, seed=None):
    """(n_txns, ops_min, ops_max, read_frac, theta) of batch b."""
    s = SHAPES[name]["seed"] if seed is None else seed
    if name == "plain":
        return 1 << 16, 10, 10, 0.5, 0.0
    if name == "zipf":
        return 1 << 20, 16, 16, 0.8, 0.99
    u = _mix(s ^ (0xC4 << 40) ^ b)
    v = _mix(u)
    n = int(round(2.0 ** (10 + 10 * ((u >> 11) / float(1 << 53)))))
    theta = 0.5 + 0.49 * ((v >> 11) / float(1 << 53))
    return n, 1, 32, 0.7, theta


def generate(name, b, seed=None, rank=0):
    """(txn_first, keys, opw, n_txns, ops_per_txn) of batch b; ops_per_txn is
    0 when transactions vary in length."""
    sh = SHAPES[name]
    s = (sh["seed"] if seed is None else seed) + rank
    n, omin, omax, rf, th = batch_params(name, b, s)
    tf, keys, opw = L.gen_ycsb(s, sh["rows"], sh["cols"], omin, omax, rf, th, batch=b, n_txns=n)
    return tf, keys, opw, n, (omin if omin == omax else 0)


def algorithmic_bytes(n_ops, n_txns, key_bytes=8):
    """Per op its key (8 B, or 4 with 32-bit keys), opword 4, value read 4,
    value written 4, conflict state 8 (28 B with 64-bit keys) + 4 B per
    transaction (commit word / descriptor)."""
    return (20 + key_bytes) * n_ops + 4 * n_txns


def tpcc_algorithmic_bytes(g, keys, opw, n_txns, key_bytes=8):
    """Bytes a batch of the TPC-C workload must move at least: per op its key
    (8, or 4 with 32-bit keys), opword (4), output (4) and conflict state (8); a read or RMW reads
    its cell (4 or 8 B, the column's width) and an RMW writes it back; an
    insert reads its payload row and writes the new row; 4 B per transaction.
    """
    import numpy as np

    kind = opw & 3
    tb = (opw >> 8) & 15
    col = (opw >> 2) & 63
    width = np.zeros((16, 64), np.int64)
    rowb = np.zeros(16, np.int64)
    for t in range(9):
        n_cols, mask, _ = g.table(t)
        for c in range(n_cols):
            width[t, c] = 8 if (mask >> c) & 1 else 4
        rowb[t] = width[t, :n_cols].sum()
    w = width[tb, col]
    cell = np.where(kind == 0, w, np.where(kind == 1, 2 * w, 2 * rowb[tb]))
    return int((16 + key_bytes) * len(keys) + cell.sum() + 4 * n_txns)


def tpcc_insert_bytes(g, keys, opw, key_bytes=8):
    """Bytes the insert kernel of one batch moves at least: every opword
    (4 B/op), and per insert its key (8, or 4 with 32-bit keys), payload row
    (read), new row (written) and output (4)."""
    import numpy as np

    rowb = np.zeros(16, np.int64)
    for t in range(9):
        n_cols, mask, _ = g.table(t)
        rowb[t] = 4 * n_cols + 4 * bin(mask).count("1")
    ins = (opw & 3) == 2
    return int(4 * len(opw) + ((4 + key_bytes) * ins.sum()) + 2 * rowb[((opw >> 8) & 15)[ins]].sum())


def mixed_pool(ycsb, tpcc, seed, tpcc_table_base=1):
    """Seeded 50/50 blend of two transaction pools in a random order: ycsb =
    (txn_first, keys, opw); tpcc = (txn_first, keys, opw, payload, pay_first)
    whose table ids are shifted by tpcc_table_base.  Returns (txn_first, keys,
    opw, pay_first, payload, is_tpcc): transaction k's payload is
    payload[pay_first[k]:pay_first[k+1]] and insert keys index the whole
    payload."""
    import numpy as np

    ytf, yk, yw = (np.asarray(a) for a in ycsb)
    ttf, tk, tw, tpay, tpf = (np.asarray(a) for a in tpcc)
    tw = tw.astype(np.uint32) + np.uint32(tpcc_table_base << 8)
    ny, nt = len(ytf) - 1, len(ttf) - 1
    src = np.concatenate([np.zeros(ny, np.int8), np.ones(nt, np.int8)])
    np.random.default_rng(seed).shuffle(src)
    is_t = src == 1
    idx = np.where(is_t, np.cumsum(is_t) - 1, np.cumsum(~is_t) - 1)
    ytf64, ttf64, tpf64 = ytf.astype(np.int64), ttf.astype(np.int64), tpf.astype(np.int64)
    first = np.where(is_t, ttf64[np.minimum(idx, nt)], ytf64[np.minimum(idx, ny)])
    lens = np.where(is_t, ttf64[np.minimum(idx + 1, nt)] - ttf64[np.minimum(idx, nt)],
                    ytf64[np.minimum(idx + 1, ny)] - ytf64[np.minimum(idx, ny)])
    tf = np.concatenate([[0], np.cumsum(lens)])
    op_src = np.repeat(first - tf[:-1], lens) + np.arange(tf[-1])
    op_t = np.repeat(is_t, lens)
    keys = np.empty(tf[-1], np.uint64)
    opw = np.empty(tf[-1], np.uint32)
    keys[~op_t] = yk[op_src[~op_t]]
    opw[~op_t] = yw[op_src[~op_t]]
    keys[op_t] = tk[op_src[op_t]]
    opw[op_t] = tw[op_src[op_t]]
    # payload: TPC-C transactions keep their rows, rebased to the blend
    pstart = np.where(is_t, tpf64[np.minimum(idx, nt)], 0)
    plen = np.where(is_t, tpf64[np.minimum(idx + 1, nt)] - tpf64[np.minimum(idx, nt)], 0)
    pay_first = np.concatenate([[0], np.cumsum(plen)])
    pay_src = np.repeat(pstart - pay_first[:-1], plen) + np.arange(pay_first[-1])
    payload = tpay[pay_src] if len(pay_src) else np.zeros(1, np.int32)
    ins = op_t & ((opw & 3) == 2)
    delta = np.repeat(pay_first[:-1] - pstart, lens)
    keys[ins] = (keys[ins].astype(np.int64) + delta[ins]).astype(np.uint64)
    return (tf.astype(np.uint32), keys, opw, pay_first.astype(np.uint64), payload.astype(np.int32),
            src.astype(np.int8))


def expected_txns(name):
    if name != "uneven":
        return SHAPES[name]["batches"] * batch_params(name, 0)[0]
    return sum(batch_params(name, b)[0] for b in range(SHAPES[name]["batches"]))


_ = math


def ycsbe_batch(b, rank=0, n_txns=None):
    """Batch b of the YCSB-E workload, expanded as the compatibility layer
    expands the reference's YCSB_E query: 9 scans of rows [r, r+2) -- each
    row's every int column read, a row past the table's end skipped -- then
    one insert whose int columns hold the query's tenth row id.  Returns
    (txn_first, keys, opw, payload, n_txns, inserts per table)."""
    import numpy as np

    sh = SHAPES["ycsbe"]
    n = sh["batch"] if n_txns is None else n_txns
    rows, cols = sh["rows"], sh["cols"]
    # ten distinct Zipf row ids per transaction from the library's generator
    _, k10, _ = L.gen_ycsb(sh["seed"] + rank, rows, cols, 10, 10, 1.0, sh["theta"], batch=b, n_txns=n)
    k = k10[:10 * n].reshape(n, 10).astype(np.int64)
    scan = k[:, :9, None] + np.arange(2)[None, None, :]                # [n, 9, 2] rows
    rk = np.broadcast_to(scan[..., None], (n, 9, 2, cols))             # [n, 9, 2, cols]
    rc = np.broadcast_to(np.arange(cols), (n, 9, 2, cols))
    keys = np.concatenate([rk.reshape(n, -1), np.arange(n)[:, None] * cols], axis=1)  # insert key: payload offset
    opw = np.concatenate([(rc.reshape(n, -1) << 2).astype(np.uint32), np.full((n, 1), L.OP_INSERT, np.uint32)],
                         axis=1)
    keep = np.concatenate([np.broadcast_to(scan[..., None] < rows, (n, 9, 2, cols)).reshape(n, -1),
                           np.ones((n, 1), bool)], axis=1)
    tf = np.zeros(n + 1, np.uint32)
    tf[1:] = np.cumsum(keep.sum(axis=1))
    payload = np.repeat(k[:, 9], cols).astype(np.int32)
    ins = np.zeros(9, np.int64)
    ins[0] = n
    return tf, keys[keep].astype(np.uint64), opw[keep], payload, n, ins


def ycsbe_algorithmic_bytes(n_ops, n_txns, n_inserts, cols, key_bytes=4):
    """Per op its key, opword (4), value read (4), output (4) and conflict
    state (8); per insert its payload row read and new row written; 4 B per
    transaction."""
    return (20 + key_bytes) * n_ops + 2 * 4 * cols * n_inserts + 4 * n_txns


def ycsbe_insert_bytes(n_ops, n_inserts, cols, key_bytes=4):
    """Bytes the insert kernel moves at least: every opword, and per insert
    its key, payload row, new row and output."""
    return 4 * n_ops + (4 + key_bytes) * n_inserts + 2 * 4 * cols * n_inserts