"""ctypes front end of the CPU oracle (oracle/ltp_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() as
the checker and by bench.py's CPU-baseline leg.  The shipped library never
imports it.  Parity status: the replay restates the reference's per-row
ascending-TID rule; value parity is unpinned by the reference (its operators
do not write); the reference-generator restatements are pinned by
tests/golden/.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libltp_oracle.so")
REF_LIB_PATH = os.path.join(HERE, "_ref", "libltpmg_ref_random.so")

OPW_READ, OPW_ADD, OPW_INSERT = 0, 1, 2


def build(verbose=False):
    """Compile the oracle restatement (gcc; same bits on x86-64 and aarch64)."""
    cmd = ["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-fPIC", "-shared",
           os.path.join(HERE, "ltp_oracle.c"), "-o", LIB_PATH, "-lm", "-lpthread"]
    subprocess.run(cmd, check=True, capture_output=not verbose)
    return LIB_PATH


# where the reference tree is read from when LTPMG_REFERENCE is not set (the
# recipe stages what it needs under oracle/_ref/src, which then travels with
# the working tree to machines without the tree)
REFERENCE_TREE = "/root/reference"
REF_CUDA = os.path.join(HERE, "_ref", "ltpmg_ref_cuda")
REF_GEN = os.path.join(HERE, "_ref", "ltpmg_ref_gen")


def build_ref(verbose=False):
    """Compile the reference's own code into oracle/_ref (build_ref.sh): from
    the reference tree when it is present, else from a staged copy of it;
    a no-op with neither."""
    env = dict(os.environ)
    if not env.get("LTPMG_REFERENCE") and os.path.isdir(REFERENCE_TREE):
        env["LTPMG_REFERENCE"] = REFERENCE_TREE
    subprocess.run(["bash", os.path.join(HERE, "build_ref.sh")], check=True, capture_output=not verbose, env=env)
    return REF_LIB_PATH if os.path.exists(REF_LIB_PATH) else None


def ref_cuda_run(rows, row_ids, ints, epochs=1, workdir=None, timeout=600):
    """Runs the reference's own CUDA path (oracle/_ref/ltpmg_ref_cuda, built
    from its unchanged cuda/src) on one GPU: YCSB_A queries row_ids
    uint32[n, 10] over a table whose int columns are ints int32[rows, 3].
    Returns a dict: per-epoch cost_gpu, the op records (TID, type, table,
    row) in the reference's record order, per-row op counts registered by
    txn_executor (cnt) and scattered by txn_analyze_regular (tmp),
    used-row count, type-list lengths and the int columns after the batch."""
    import tempfile

    row_ids = np.ascontiguousarray(row_ids, np.uint32)
    ints = np.ascontiguousarray(ints, np.int32)
    n = row_ids.shape[0]
    assert row_ids.shape == (n, 10) and ints.shape == (rows, 3)
    d = workdir or tempfile.mkdtemp(prefix="ltpref")
    fin, fout = os.path.join(d, "in.bin"), os.path.join(d, "out.bin")
    with open(fin, "wb") as f:
        f.write(np.array([rows, n, epochs, 0], np.uint32).tobytes())
        f.write(row_ids.tobytes())
        f.write(ints.tobytes())
    r = subprocess.run([REF_CUDA, fin, fout], capture_output=True, text=True, timeout=timeout)
    if r.returncode != 0:
        raise RuntimeError(f"reference CUDA run failed ({r.returncode}): {r.stderr[-2000:]}")
    raw = np.fromfile(fout, np.uint8)
    off = 0

    def take(dtype, count):
        nonlocal off
        a = raw[off:off + count * np.dtype(dtype).itemsize].view(dtype)
        off += count * np.dtype(dtype).itemsize
        return a

    hdr = take(np.uint32, 6)
    n_ops = int(hdr[1])
    out = {"status": int(hdr[0]), "n_ops": n_ops, "used_rows": int(hdr[3]), "select_cur": int(hdr[4]),
           "update_cur": int(hdr[5])}
    out["cost_gpu"] = take(np.float32, epochs).astype(float).tolist()
    out["rec"] = take(np.uint32, n_ops * 4).reshape(n_ops, 4)
    out["cnt"] = take(np.uint32, rows)
    out["tmp"] = take(np.uint32, rows)
    out["ints_after"] = take(np.int32, rows * 3).reshape(rows, 3)
    return out


def ref_gen_time(benchmark, table_size, batch, dist, zipf, reps=1, timeout=900):
    """Seconds per call of the reference's own host generator
    (Query::generate_txn) on every hardware thread; parsed from
    oracle/_ref/ltpmg_ref_gen's JSON line."""
    import json

    r = subprocess.run([REF_GEN, benchmark, str(table_size), str(batch), dist, str(zipf), str(reps)],
                       capture_output=True, text=True, timeout=timeout)
    if r.returncode != 0:
        raise RuntimeError(f"reference generator failed ({r.returncode}): {r.stderr[-2000:]}")
    return json.loads([l for l in r.stdout.splitlines() if l.startswith("{")][-1])


class YcsbParams(ctypes.Structure):
    _fields_ = [("seed", ctypes.c_uint64), ("n_rows", ctypes.c_uint64), ("n_cols", ctypes.c_uint32),
                ("ops_min", ctypes.c_uint32), ("ops_max", ctypes.c_uint32), ("rmw_delta", ctypes.c_int32),
                ("read_frac", ctypes.c_double), ("theta", ctypes.c_double)]


class OTable(ctypes.Structure):
    _fields_ = [("cols", ctypes.POINTER(ctypes.c_void_p)), ("rows_cap", ctypes.c_uint64),
                ("n_rows", ctypes.c_uint64), ("n_cols", ctypes.c_uint32), ("pad", ctypes.c_uint32),
                ("wide", ctypes.c_uint64)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        u64, u32, i32, dbl, vp = ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int32, ctypes.c_double, ctypes.c_void_p
        L.ltpo_mix64.restype = u64
        L.ltpo_mix64.argtypes = [u64]
        L.ltpo_stream_seed.restype = u64
        L.ltpo_stream_seed.argtypes = [u64, u64, u64]
        L.ltpo_feistel_perm.restype = u64
        L.ltpo_feistel_perm.argtypes = [u64, u64, u64]
        L.ltpo_det_log.restype = dbl
        L.ltpo_det_log.argtypes = [dbl]
        L.ltpo_det_exp.restype = dbl
        L.ltpo_det_exp.argtypes = [dbl]
        L.ltpo_zipf_draw.restype = u64
        L.ltpo_zipf_draw.argtypes = [u64, dbl, ctypes.POINTER(u64)]
        L.ltpo_table_value.restype = i32
        L.ltpo_table_value.argtypes = [u64, u64, u32, u32]
        L.ltpo_gen_ycsb_batch.restype = u64
        L.ltpo_gen_ycsb_batch.argtypes = [ctypes.POINTER(YcsbParams), u64, u64, vp, vp, vp, u64]
        L.ltpo_table_init.restype = None
        L.ltpo_table_init.argtypes = [u64, u64, u32, vp]
        L.ltpo_replay.restype = ctypes.c_int
        L.ltpo_replay.argtypes = [ctypes.c_int, u64, u32, vp, u64, vp, vp, vp, vp, vp]
        L.ltpo_replay_r0_mt.restype = ctypes.c_int
        L.ltpo_replay_r0_mt.argtypes = [u64, u32, vp, u64, vp, vp, vp, vp, vp, ctypes.c_int]
        L.ltpo_replay_tables.restype = ctypes.c_int
        L.ltpo_replay_tables.argtypes = [ctypes.c_int, u32, ctypes.POINTER(OTable), u64, vp, vp, vp, vp, u64, vp, vp]
        L.ltpo_replay_tables_r0_mt.restype = ctypes.c_int
        L.ltpo_replay_tables_r0_mt.argtypes = [u32, ctypes.POINTER(OTable), u64, vp, vp, vp, vp, u64, vp, vp,
                                               ctypes.c_int]
        L.ltpo_fnv1a.restype = u64
        L.ltpo_fnv1a.argtypes = [vp, u64]
        L.ltpo_ref_zipf_table.restype = u32
        L.ltpo_ref_zipf_table.argtypes = [u64, dbl, vp]
        L.ltpo_ref_zipf_pick.restype = u32
        L.ltpo_ref_zipf_pick.argtypes = [vp, u32, u32, u32]
        L.ltpo_ref_nurand.restype = u64
        L.ltpo_ref_nurand.argtypes = [u64, u64, u64, u64, u64]
        L.ltpo_ref_ycsb_op_type.restype = u32
        L.ltpo_ref_ycsb_op_type.argtypes = [u32, u32]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def opword(kind, col, table=0, imm=0):
    return (kind | (col << 2) | (table << 8) | ((imm & 0xFFFFF) << 12)) & 0xFFFFFFFF


def ycsb_params(seed, n_rows, n_cols, ops_min, ops_max, read_frac, theta, rmw_delta=1):
    return YcsbParams(seed, n_rows, n_cols, ops_min, ops_max, rmw_delta, read_frac, theta)


def gen_ycsb_batch(p, batch, n_txns):
    """Returns (txn_first uint32[n_txns+1], keys uint64[n_ops], opw uint32[n_ops])."""
    cap = n_txns * p.ops_max
    tf = np.zeros(n_txns + 1, np.uint32)
    keys = np.zeros(max(cap, 1), np.uint64)
    opw = np.zeros(max(cap, 1), np.uint32)
    n = lib().ltpo_gen_ycsb_batch(ctypes.byref(p), batch, n_txns, _p(tf), _p(keys), _p(opw), cap)
    if n == 2 ** 64 - 1:
        raise ValueError("generator rejected the parameters")
    return tf, keys[:n].copy(), opw[:n].copy()


def table_init(seed, n_rows, n_cols):
    tab = np.empty((n_cols, n_rows), np.int32)
    lib().ltpo_table_init(seed, n_rows, n_cols, _p(tab))
    return tab


def replay(rule, tab, txn_first, keys, opw, threads=0):
    """Serial replay on a copy of the column-major table; returns
    (table_after, commit uint8[n_txns], out int32[n_ops])."""
    tab = np.ascontiguousarray(tab, np.int32).copy()
    n_cols, n_rows = tab.shape
    n_txns = len(txn_first) - 1
    commit = np.zeros(max(n_txns, 1), np.uint8)
    out = np.zeros(max(len(keys), 1), np.int32)
    tf = np.ascontiguousarray(txn_first, np.uint32)
    k = np.ascontiguousarray(keys, np.uint64)
    w = np.ascontiguousarray(opw, np.uint32)
    if threads and rule == 0:
        rc = lib().ltpo_replay_r0_mt(n_rows, n_cols, _p(tab), n_txns, _p(tf), _p(k), _p(w), _p(commit), _p(out), threads)
    else:
        rc = lib().ltpo_replay(rule, n_rows, n_cols, _p(tab), n_txns, _p(tf), _p(k), _p(w), _p(commit), _p(out))
    if rc != 0:
        raise ValueError("oracle rejected the batch (malformed op)")
    return tab, commit[:n_txns], out[:len(keys)]


class TablesDB:
    """Tables held as per-column arrays for repeated multi-table replays
    (int32 columns, int64 where the table's wide mask says so).  tables:
    list of (data [n_cols, rows_cap], n_rows) or (data, n_rows, wide_mask)."""

    def __init__(self, tables):
        self.masks, self.cols, self._ptrs = [], [], []
        self.T = (OTable * max(len(tables), 1))()
        for k, tb in enumerate(tables):
            d, n = np.asarray(tb[0]), tb[1]
            mask = tb[2] if len(tb) > 2 else 0
            cols = [np.ascontiguousarray(d[c], np.int64 if (mask >> c) & 1 else np.int32).copy()
                    for c in range(d.shape[0])]
            ptrs = (ctypes.c_void_p * len(cols))(*[c.ctypes.data for c in cols])
            self.masks.append(mask)
            self.cols.append(cols)
            self._ptrs.append(ptrs)
            self.T[k] = OTable(ptrs, d.shape[1], n, d.shape[0], 0, mask)
        self.n = len(tables)

    def replay(self, rule, txn_first, keys, opw, payload=None, threads=0):
        """(commit, out int64) of one batch; threads > 0 runs the ordered
        rule on that many threads."""
        n_txns = len(txn_first) - 1
        commit = np.zeros(max(n_txns, 1), np.uint8)
        out = np.zeros(max(len(keys), 1), np.int64)
        tf = np.ascontiguousarray(txn_first, np.uint32)
        k = np.ascontiguousarray(keys, np.uint64)
        w = np.ascontiguousarray(opw, np.uint32)
        pl = np.ascontiguousarray(payload if payload is not None else np.zeros(1, np.int32), np.int32)
        pn = 0 if payload is None else len(pl)
        if threads > 0:
            assert rule == 0
            rc = lib().ltpo_replay_tables_r0_mt(self.n, self.T, n_txns, _p(tf), _p(k), _p(w), _p(pl), pn,
                                                _p(commit), _p(out), threads)
        else:
            rc = lib().ltpo_replay_tables(rule, self.n, self.T, n_txns, _p(tf), _p(k), _p(w), _p(pl), pn,
                                          _p(commit), _p(out))
        if rc != 0:
            raise ValueError(f"oracle rejected the batch ({rc})")
        return commit[:n_txns], out[:len(keys)]

    def tables(self):
        """[(data [n_cols, rows_cap], n_rows)], int64 for tables with int64 columns."""
        res = []
        for i, cols in enumerate(self.cols):
            dt = np.int64 if self.masks[i] else np.int32
            res.append((np.stack([c.astype(dt) for c in cols]), self.T[i].n_rows))
        return res


def replay_tables(rule, tables, txn_first, keys, opw, payload=None, threads=0):
    """Multi-table replay with inserts.  tables: list of (data [n_cols,
    rows_cap], n_rows) or (data, n_rows, wide_mask); data is int32, or int64
    when wide_mask names int64 columns (int32 columns sign-extended).
    Returns (list of (data, n_rows, wide_mask) after, commit, out int64)."""
    db = TablesDB(tables)
    commit, out = db.replay(rule, txn_first, keys, opw, payload, threads)
    after = [(d, n, m) for (d, n), m in zip(db.tables(), db.masks)]
    return after, commit, out


def fnv1a(a):
    a = np.ascontiguousarray(a)
    return int(lib().ltpo_fnv1a(_p(a), a.nbytes))
