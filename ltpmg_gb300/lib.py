"""ctypes binding of libltpmg_gb300.so (the C ABI in include/ltpmg_gb300.h).

There is no fallback: if the shared library is missing or fails to load,
every entry point raises.  Build it with ``python -c "import
__graft_entry__ as g; g.build()"`` (or ``python ltpmg_gb300/_build.py``).
"""
import ctypes
import os
import re

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
# LTPMG_LIB selects another build of the library (e.g. the bounds-checked one)
LIB_PATH = os.environ.get("LTPMG_LIB") or os.path.join(PKG, "libltpmg_gb300.so")
HEADER = os.path.join(os.path.dirname(PKG), "include", "ltpmg_gb300.h")

LTP_OK = 0
LTP_E_CUDA, LTP_E_CAPACITY, LTP_E_TIMEOUT, LTP_E_BADARG = -1, -2, -3, -4
LTP_E_DEVICE_ASSERT, LTP_E_NOMEM, LTP_E_STATE = -5, -6, -7
RULE_ORDERED, RULE_PRIORITY = 0, 1
OP_READ, OP_ADD, OP_INSERT = 0, 1, 2
FLAG_STAGE_TIMING = 1
MODE_STREAM, MODE_GRAPH, MODE_PERSISTENT = 0, 1, 2
# per-kernel stage times of a batch (ordered rule; under the priority rule
# stages 2-4 are the min-writer, abort and execute kernels)
STAGE_NAMES = ["mark", "ids", "classify", "sort_pass0", "sort_pass1", "sort_pass2", "sort_pass3", "apply",
               "insert", "finish", "unused", "total"]


class LtpError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"ltpmg_gb300 error {status}: {msg}")
        self.status = status


class Config(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int32), ("rule", ctypes.c_int32), ("reserve_ops", ctypes.c_uint64),
                ("flags", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]


class Schema(ctypes.Structure):
    _fields_ = [("n_cols", ctypes.c_uint32), ("reserved", ctypes.c_uint32), ("wide_cols", ctypes.c_uint64)]


class Stats(ctypes.Structure):
    _fields_ = [("txns", ctypes.c_uint64), ("ops", ctypes.c_uint64), ("committed", ctypes.c_uint64),
                ("aborted", ctypes.c_uint64), ("contended_ops", ctypes.c_uint64),
                ("contended_cells", ctypes.c_uint64), ("touched_words", ctypes.c_uint64),
                ("bytes_algorithmic", ctypes.c_uint64), ("ms_stage", ctypes.c_float * 12)]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_ if k != "ms_stage"}
        d["ms_stage"] = dict(zip(STAGE_NAMES, list(self.ms_stage)))
        return d


class YcsbParams(ctypes.Structure):
    _fields_ = [("seed", ctypes.c_uint64), ("n_rows", ctypes.c_uint64), ("n_cols", ctypes.c_uint32),
                ("ops_min", ctypes.c_uint32), ("ops_max", ctypes.c_uint32), ("rmw_delta", ctypes.c_int32),
                ("read_frac", ctypes.c_double), ("theta", ctypes.c_double)]


class ServeConfig(ctypes.Structure):
    _fields_ = [("deadline_us", ctypes.c_uint32), ("depth", ctypes.c_uint32), ("budget_bytes", ctypes.c_uint64),
                ("max_txns", ctypes.c_uint64), ("max_ops", ctypes.c_uint64), ("max_attempts", ctypes.c_uint32),
                ("flags", ctypes.c_uint32)]


SERVE_MAX_OPS = 64
# ltp_serve_config.flags
SERVE_EAGER, SERVE_KEEP_RESULTS, SERVE_PERSISTENT, SERVE_KEYS64, SERVE_JIT = 1, 2, 4, 8, 16


class ServeResult(ctypes.Structure):
    _fields_ = [("tag", ctypes.c_uint64), ("arrival_ns", ctypes.c_uint64), ("done_ns", ctypes.c_uint64),
                ("batch_seq", ctypes.c_uint64), ("pos", ctypes.c_uint32), ("stream", ctypes.c_uint32),
                ("n_ops", ctypes.c_uint32), ("attempts", ctypes.c_uint32), ("committed", ctypes.c_uint32),
                ("pad", ctypes.c_uint32), ("vals", ctypes.c_int64 * SERVE_MAX_OPS)]


class ServeStats(ctypes.Structure):
    _fields_ = [(k, ctypes.c_uint64) for k in ("submitted", "completed", "committed", "aborted_attempts", "batches",
                                               "closed_deadline", "closed_budget", "closed_idle", "ops")] + \
               [(k, ctypes.c_double) for k in ("p50_us", "p99_us", "p999_us", "mean_us", "max_us", "elapsed_s",
                                               "committed_per_s", "dispatch_busy_s", "complete_busy_s",
                                               "loadgen_late_frac")]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Tuning(ctypes.Structure):
    _fields_ = [("block", ctypes.c_uint32), ("ipt", ctypes.c_uint32), ("word_bits", ctypes.c_uint32),
                ("flags", ctypes.c_uint32)]


TUNE_MARK_PRECHECK = 1


_lib = None


def load():
    """Loads the shared library (raises if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise LtpError(LTP_E_STATE, f"{LIB_PATH} is missing: build the CUDA extension first")
    L = ctypes.CDLL(LIB_PATH)
    vp, u64, u32, i32, ci = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int32, ctypes.c_int
    pp = ctypes.POINTER(ctypes.c_void_p)
    sig = {
        "ltp_version": (ctypes.c_char_p, []),
        "ltp_status_string": (ctypes.c_char_p, [ci]),
        "ltp_last_error": (ctypes.c_char_p, [vp]),
        "ltp_init": (ci, [ctypes.POINTER(Config), pp]),
        "ltp_shutdown": (ci, [vp]),
        "ltp_default_stream": (vp, [vp]),
        "ltp_sync": (ci, [vp, vp]),
        "ltp_table_create": (ci, [vp, ctypes.POINTER(Schema), u64, ctypes.POINTER(u32)]),
        "ltp_table_upload": (ci, [vp, u32, u32, u64, u64, vp]),
        "ltp_table_download": (ci, [vp, u32, u32, u64, u64, vp]),
        "ltp_table_fill_seeded": (ci, [vp, u32, u64, vp]),
        "ltp_table_fingerprint": (ci, [vp, u32, ctypes.POINTER(u64)]),
        "ltp_batch_create": (ci, [vp, u64, u64, pp]),
        "ltp_batch_free": (ci, [vp, vp]),
        "ltp_batch_load": (ci, [vp, vp, u64, vp, u32, u64, vp, vp, vp]),
        "ltp_batch_load32": (ci, [vp, vp, u64, vp, u32, u64, vp, vp, vp]),
        "ltp_pipe_submit32": (ci, [vp, u64, vp, u32, u64, vp, vp, vp, u64, vp, vp, ctypes.POINTER(u64)]),
        "ltp_batch_execute": (ci, [vp, vp, vp]),
        "ltp_batch_fetch": (ci, [vp, vp, vp, vp, vp]),
        "ltp_batch_fetch64": (ci, [vp, vp, vp, vp]),
        "ltp_batch_finish": (ci, [vp, vp, ctypes.POINTER(Stats), vp]),
        "ltp_batch_results": (ci, [vp, vp, vp, vp, ctypes.POINTER(Stats)]),
        "ltp_batch_device_ptrs": (ci, [vp, pp, pp, pp, pp, pp]),
        "ltp_host_alloc": (vp, [ctypes.c_size_t]),
        "ltp_host_free": (None, [vp]),
        "ltp_gen_ycsb": (u64, [ctypes.POINTER(YcsbParams), u64, u64, vp, vp, vp, u64, ci]),
        "ltp_tpcc_create": (ci, [ctypes.POINTER(TpccParams), pp]),
        "ltp_tpcc_free": (None, [vp]),
        "ltp_tpcc_table": (ci, [vp, u32, ctypes.POINTER(Schema), ctypes.POINTER(u64)]),
        "ltp_tpcc_column": (ci, [vp, u32, u32, u64, u64, vp]),
        "ltp_tpcc_gen": (ci, [vp, u64, u64, vp, vp, vp, u64, vp, u64, vp, ctypes.POINTER(u64), ctypes.POINTER(u64),
                              ctypes.POINTER(u64), vp, ci]),
        "ltp_table_value": (i32, [u64, u64, u32, u32]),
        "ltp_set_tuning": (ci, [vp, u32, ctypes.POINTER(Tuning)]),
        "ltp_get_tuning": (ci, [vp, u32, ctypes.POINTER(Tuning)]),
        "ltp_debug_stall_next": (ci, [vp, u32]),
        "ltp_table_create_cap": (ci, [vp, ctypes.POINTER(Schema), u64, u64, ctypes.POINTER(u32)]),
        "ltp_table_rows": (ci, [vp, u32, ctypes.POINTER(u64)]),
        "ltp_batch_load_payload": (ci, [vp, vp, vp, u64, vp]),
        "ltp_compat_last_status": (ci, []),
        "ltp_compat_last_error": (ctypes.c_char_p, []),
        "ltp_batches_execute": (ci, [vp, vp, u32, i32, vp]),
        "ltp_pipe_create": (ci, [vp, u32, u64, u64, pp]),
        "ltp_pipe_create2": (ci, [vp, u32, u64, u64, u32, pp]),
        "ltp_pipe_free": (ci, [vp]),
        "ltp_pipe_submit": (ci, [vp, u64, vp, u32, u64, vp, vp, vp, u64, vp, vp, ctypes.POINTER(u64)]),
        "ltp_pipe_wait": (ci, [vp, u64, ctypes.POINTER(Stats)]),
        "ltp_pipe_poll": (ci, [vp, u64]),
        "ltp_set_stage_timing": (ci, [vp, i32]),
        "ltp_serve_open": (ci, [vp, ctypes.POINTER(ServeConfig), pp]),
        "ltp_serve_submit": (ci, [vp, u32, u32, vp, vp, u64, u64]),
        "ltp_serve_submit_rows": (ci, [vp, u32, u32, vp, vp, u32, vp, u64, u64]),
        "ltp_serve_loadgen_rows": (ci, [vp, ctypes.c_double, ctypes.c_double, u32, u64, vp, u64, vp, vp, vp, vp, u32]),
        "ltp_pipe_submit64": (ci, [vp, u64, vp, u32, u64, vp, vp, vp, u64, vp, vp, ctypes.POINTER(u64)]),
        "ltp_table_truncate": (ci, [vp, u32, u64]),
        "ltp_ctx_wide": (ci, [vp]),
        "ltp_serve_poll": (ci, [vp, ctypes.POINTER(ServeResult), u32, ctypes.POINTER(u32)]),
        "ltp_serve_loadgen": (ci, [vp, ctypes.c_double, ctypes.c_double, u32, u64, vp, u64, vp, vp, u32]),
        "ltp_serve_stats_now": (ci, [vp, ctypes.POINTER(ServeStats)]),
        "ltp_serve_close": (ci, [vp, ctypes.POINTER(ServeStats)]),
        "ltp_now_ns": (u64, []),
        "ltp_poisson_arrivals": (ci, [u64, ctypes.c_double, u64, vp, ctypes.c_int]),
        "ltp_ingest_open": (ci, [vp, ctypes.POINTER(ServeConfig), u64, vp, vp, vp, vp, vp, pp]),
        "ltp_ingest_run": (ci, [vp, u64, vp, ctypes.POINTER(ServeStats)]),
        "ltp_ingest_results": (ci, [vp, vp, vp, vp, vp, vp]),
        "ltp_ingest_close": (ci, [vp]),
        "ltp_execute_noalloc": (ci, [i32, i32, vp, u64, u64, u32, u64, vp, u32, u64, vp, vp, vp, vp, vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def header_functions(path=HEADER):
    """Names of every function declared in the public header."""
    txt = open(path).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(ltp_[a-z0-9_]+)\s*\(", txt)) - {"ltp_ctx", "ltp_batch"})


def _p(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


def _stream(s):
    if s is None:
        return None
    if isinstance(s, int):
        return ctypes.c_void_p(s)
    return ctypes.c_void_p(int(getattr(s, "cuda_stream", s)))


class PinnedArray:
    """numpy view over pinned (page-locked) host memory from ltp_host_alloc."""

    def __init__(self, shape, dtype):
        L = load()
        dtype = np.dtype(dtype)
        n = int(np.prod(shape)) if shape else 1
        nbytes = max(n * dtype.itemsize, 1)
        self._ptr = L.ltp_host_alloc(nbytes)
        if not self._ptr:
            raise LtpError(LTP_E_NOMEM, "pinned host allocation failed")
        buf = (ctypes.c_uint8 * nbytes).from_address(self._ptr)
        self.array = np.frombuffer(buf, dtype=dtype, count=n).reshape(shape)

    def __del__(self):
        if getattr(self, "_ptr", None):
            load().ltp_host_free(self._ptr)
            self._ptr = None


def gen_ycsb(seed, n_rows, n_cols, ops_min, ops_max, read_frac, theta, batch, n_txns, rmw_delta=1, threads=0,
             out=None):
    """Seeded batch from the library's host generator.  Returns
    (txn_first uint32[n_txns+1], keys uint64[n_ops], opw uint32[n_ops]);
    `out` may supply preallocated (txn_first, keys, opw) arrays."""
    L = load()
    p = YcsbParams(seed, n_rows, n_cols, ops_min, ops_max, rmw_delta, read_frac, theta)
    cap = n_txns * ops_max
    if out is None:
        tf = np.zeros(n_txns + 1, np.uint32)
        keys = np.zeros(max(cap, 1), np.uint64)
        opw = np.zeros(max(cap, 1), np.uint32)
    else:
        tf, keys, opw = out
        cap = min(len(keys), len(opw))
    n = L.ltp_gen_ycsb(ctypes.byref(p), batch, n_txns, _p(tf), _p(keys), _p(opw), cap, threads)
    if n == 2 ** 64 - 1:
        raise LtpError(LTP_E_BADARG, "generator rejected the parameters")
    return tf[: n_txns + 1], keys[:n], opw[:n]


class TpccParams(ctypes.Structure):
    _fields_ = [("seed", ctypes.c_uint64), ("warehouses", ctypes.c_uint32), ("districts", ctypes.c_uint32),
                ("customers", ctypes.c_uint32), ("items", ctypes.c_uint32), ("ol_min", ctypes.c_uint32),
                ("ol_max", ctypes.c_uint32), ("new_order_frac", ctypes.c_double), ("remote_line", ctypes.c_double),
                ("remote_payment", ctypes.c_double), ("by_last_name", ctypes.c_double)]


TPCC_TABLES = ("warehouse", "district", "customer", "history", "new_order", "order", "order_line", "item", "stock")
TPCC_WAREHOUSE, TPCC_DISTRICT, TPCC_CUSTOMER, TPCC_HISTORY, TPCC_NEW_ORDER, TPCC_ORDER, TPCC_ORDER_LINE, \
    TPCC_ITEM, TPCC_STOCK = range(9)


class Tpcc:
    """The library's TPC-C-shaped order-entry workload (ltp_tpcc_*): schema,
    initial table contents and seeded new-order / payment batches."""

    def __init__(self, warehouses, seed=1, districts=10, customers=3000, items=100000, ol_min=5, ol_max=15,
                 new_order_frac=0.5, remote_line=0.01, remote_payment=0.15, by_last_name=0.6):
        self.L = load()
        self.params = TpccParams(seed, warehouses, districts, customers, items, ol_min, ol_max, new_order_frac,
                                 remote_line, remote_payment, by_last_name)
        h = ctypes.c_void_p()
        rc = self.L.ltp_tpcc_create(ctypes.byref(self.params), ctypes.byref(h))
        if rc:
            raise LtpError(rc, "ltp_tpcc_create rejected the parameters")
        self.h = h

    def close(self):
        if self.h:
            self.L.ltp_tpcc_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def table(self, t):
        """(n_cols, wide_mask, initial rows) of table t."""
        sc, rows = Schema(), ctypes.c_uint64()
        rc = self.L.ltp_tpcc_table(self.h, t, ctypes.byref(sc), ctypes.byref(rows))
        if rc:
            raise LtpError(rc, "ltp_tpcc_table")
        return sc.n_cols, sc.wide_cols, rows.value

    def column(self, t, c, row0=0, n=None):
        n_cols, mask, rows = self.table(t)
        n = rows - row0 if n is None else n
        out = np.empty(n, np.int64 if (mask >> c) & 1 else np.int32)
        rc = self.L.ltp_tpcc_column(self.h, t, c, row0, n, _p(out))
        if rc:
            raise LtpError(rc, "ltp_tpcc_column")
        return out

    def initial(self, t, rows_cap=None):
        """Column-major initial contents [n_cols, rows_cap] (int64 when the
        table has an int64 column), zero beyond the initial rows."""
        n_cols, mask, rows = self.table(t)
        cap = rows if rows_cap is None else rows_cap
        out = np.zeros((n_cols, cap), np.int64 if mask else np.int32)
        for c in range(n_cols):
            out[c, :rows] = self.column(t, c)
        return out

    def gen(self, batch, n_txns, threads=0, with_pay_first=False):
        """(txn_first, keys, opw, payload, n_new_order, inserts[9]) of one
        batch, plus pay_first (where each transaction's payload starts) when
        with_pay_first."""
        n_ops, n_pay, n_no = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
        ins = np.zeros(9, np.uint64)
        tf = np.zeros(n_txns + 1, np.uint32)
        pf = np.zeros(n_txns + 1, np.uint64)
        rc = self.L.ltp_tpcc_gen(self.h, batch, n_txns, _p(tf), None, None, 0, None, 0, None, ctypes.byref(n_ops),
                                 ctypes.byref(n_pay), ctypes.byref(n_no), _p(ins), threads)
        if rc:
            raise LtpError(rc, "ltp_tpcc_gen (sizes)")
        keys = np.zeros(max(n_ops.value, 1), np.uint64)
        opw = np.zeros(max(n_ops.value, 1), np.uint32)
        pay = np.zeros(max(n_pay.value, 1), np.int32)
        rc = self.L.ltp_tpcc_gen(self.h, batch, n_txns, _p(tf), _p(keys), _p(opw), len(keys), _p(pay), len(pay), _p(pf),
                                 ctypes.byref(n_ops), ctypes.byref(n_pay), ctypes.byref(n_no), _p(ins), threads)
        if rc:
            raise LtpError(rc, "ltp_tpcc_gen")
        out = (tf, keys[:n_ops.value], opw[:n_ops.value], pay[:n_pay.value], n_no.value, ins)
        return out + (pf,) if with_pay_first else out

    def create_tables(self, ctx, extra_rows):
        """Creates the nine tables in ctx, each with room for extra_rows[t]
        inserted rows, and uploads the initial contents.  Returns the ids."""
        ids = []
        for t in range(9):
            n_cols, mask, rows = self.table(t)
            wide = [c for c in range(n_cols) if (mask >> c) & 1]
            tid = ctx.create_table(rows, n_cols, rows_cap=max(1, rows + int(extra_rows[t])), wide=wide)
            for c in range(n_cols):
                if rows:
                    ctx.upload_column(tid, c, self.column(t, c))
            ids.append(tid)
        return ids


def opword(kind, col, table=0, imm=0):
    return (kind | (col << 2) | (table << 8) | ((imm & 0xFFFFF) << 12)) & 0xFFFFFFFF


class Context:
    """One GPU, its tables and scratch (the C-ABI ltp_ctx)."""

    def __init__(self, device=0, rule=RULE_ORDERED, reserve_ops=0, stage_timing=False):
        self.L = load()
        cfg = Config(device, rule, reserve_ops, FLAG_STAGE_TIMING if stage_timing else 0, 0)
        h = ctypes.c_void_p()
        rc = self.L.ltp_init(ctypes.byref(cfg), ctypes.byref(h))
        if rc != LTP_OK:
            raise LtpError(rc, self.L.ltp_status_string(rc).decode())
        self.h = h
        self.rule = rule
        self.tables = []

    def check(self, rc):
        if rc != LTP_OK:
            raise LtpError(rc, self.L.ltp_last_error(self.h).decode() or self.L.ltp_status_string(rc).decode())
        return rc

    def close(self):
        if getattr(self, "h", None):
            self.L.ltp_shutdown(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def stream(self):
        return self.L.ltp_default_stream(self.h)

    def sync(self, stream=None):
        self.check(self.L.ltp_sync(self.h, _stream(stream)))

    def create_table(self, rows, cols, rows_cap=None, wide=()):
        """wide: indices of the int64 columns (the others are int32)."""
        tid = ctypes.c_uint32()
        cap = rows if rows_cap is None else rows_cap
        mask = 0
        for c in wide:
            mask |= 1 << int(c)
        self.check(self.L.ltp_table_create_cap(self.h, ctypes.byref(Schema(cols, 0, mask)), rows, cap,
                                               ctypes.byref(tid)))
        self.tables.append((rows, cols, mask))
        return tid.value

    def truncate(self, table, rows):
        self.check(self.L.ltp_table_truncate(self.h, table, rows))

    @property
    def wide(self):
        return bool(self.L.ltp_ctx_wide(self.h))

    def table_rows(self, table):
        v = ctypes.c_uint64()
        self.check(self.L.ltp_table_rows(self.h, table, ctypes.byref(v)))
        return v.value

    def upload(self, table, colmajor, row0=0):
        """colmajor: [n_cols, n] values; each column is stored at its own
        width (int32 columns take the low 32 bits)."""
        mask = self.tables[table][2]
        for c in range(len(colmajor)):
            a = np.ascontiguousarray(np.asarray(colmajor[c]).astype(np.int64 if (mask >> c) & 1 else np.int32))
            self.check(self.L.ltp_table_upload(self.h, table, c, row0, a.shape[0], _p(a)))

    def upload_column(self, table, col, values, row0=0):
        mask = self.tables[table][2]
        a = np.ascontiguousarray(np.asarray(values).astype(np.int64 if (mask >> col) & 1 else np.int32))
        self.check(self.L.ltp_table_upload(self.h, table, col, row0, a.shape[0], _p(a)))

    def download(self, table):
        """int32[n_cols, rows], or int64[n_cols, rows] when the table has an
        int64 column (int32 columns sign-extended)."""
        _, cols, mask = self.tables[table]
        rows = self.table_rows(table)
        out = np.empty((cols, rows), np.int64 if mask else np.int32)
        tmp = np.empty(rows, np.int32)
        for c in range(cols):
            if mask and not (mask >> c) & 1:
                self.check(self.L.ltp_table_download(self.h, table, c, 0, rows, _p(tmp)))
                out[c] = tmp
            else:
                self.check(self.L.ltp_table_download(self.h, table, c, 0, rows, _p(out[c])))
        return out

    def fill_seeded(self, table, seed, stream=None):
        self.check(self.L.ltp_table_fill_seeded(self.h, table, seed, _stream(stream)))

    def fingerprint(self, table):
        v = ctypes.c_uint64()
        self.check(self.L.ltp_table_fingerprint(self.h, table, ctypes.byref(v)))
        return v.value

    def batch(self, max_txns, max_ops):
        return Batch(self, max_txns, max_ops)

    def set_tuning(self, bucket, block, ipt, word_bits=32, flags=0):
        self.check(self.L.ltp_set_tuning(self.h, bucket, ctypes.byref(Tuning(block, ipt, word_bits, flags))))

    def get_tuning(self, bucket):
        """(block, ipt, word_bits, flags) of a size bucket."""
        t = Tuning()
        self.check(self.L.ltp_get_tuning(self.h, bucket, ctypes.byref(t)))
        return (t.block, t.ipt, t.word_bits, t.flags)

    def execute_many(self, batches, mode=0, stream=None):
        """Executes batches in order: mode 0 stream, 1 CUDA graph, 2 persistent kernel."""
        arr = (ctypes.c_void_p * max(len(batches), 1))(*[b.h.value for b in batches])
        self.check(self.L.ltp_batches_execute(self.h, arr, len(batches), mode, _stream(stream)))

    def set_stage_timing(self, on):
        self.check(self.L.ltp_set_stage_timing(self.h, 1 if on else 0))

    def stall_next(self, ms):
        self.check(self.L.ltp_debug_stall_next(self.h, ms))


class Batch:
    """Device-resident batch (the C-ABI ltp_batch)."""

    def __init__(self, ctx, max_txns, max_ops):
        self.ctx = ctx
        h = ctypes.c_void_p()
        ctx.check(ctx.L.ltp_batch_create(ctx.h, max_txns, max_ops, ctypes.byref(h)))
        self.h = h
        self.n_txns = 0
        self.n_ops = 0

    def free(self):
        if getattr(self, "h", None) and self.ctx.h:
            self.ctx.L.ltp_batch_free(self.ctx.h, self.h)
        self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    def load(self, txn_first, keys, opw, ops_per_txn=0, stream=None):
        """txn_first may be None when every transaction has ops_per_txn ops;
        uint32 keys load as 32-bit keys (ltp_batch_load32), others as 64-bit."""
        k32 = isinstance(keys, np.ndarray) and keys.dtype == np.uint32
        keys = np.ascontiguousarray(keys, np.uint32 if k32 else np.uint64)
        opw = np.ascontiguousarray(opw, np.uint32)
        if txn_first is not None:
            txn_first = np.ascontiguousarray(txn_first, np.uint32)
            n_txns = len(txn_first) - 1
        else:
            n_txns = len(keys) // ops_per_txn if ops_per_txn else 0
        self._keep = (txn_first, keys, opw)  # asynchronous copy: keep the sources alive
        self._keep_payload = None  # a load drops the previous payload
        fn = self.ctx.L.ltp_batch_load32 if k32 else self.ctx.L.ltp_batch_load
        self.ctx.check(fn(self.ctx.h, self.h, n_txns, _p(txn_first), ops_per_txn, len(keys), _p(keys), _p(opw),
                          _stream(stream)))
        self.n_txns, self.n_ops = n_txns, len(keys)

    def load_payload(self, payload, stream=None):
        payload = np.ascontiguousarray(payload, np.int32)
        self._keep_payload = payload
        self.ctx.check(self.ctx.L.ltp_batch_load_payload(self.ctx.h, self.h, _p(payload), len(payload), _stream(stream)))

    def execute(self, stream=None):
        self.ctx.check(self.ctx.L.ltp_batch_execute(self.ctx.h, self.h, _stream(stream)))

    def fetch(self, commit=None, vals=None, stream=None):
        self.ctx.check(self.ctx.L.ltp_batch_fetch(self.ctx.h, self.h, _p(commit), _p(vals), _stream(stream)))

    def fetch64(self, vals, stream=None):
        self.ctx.check(self.ctx.L.ltp_batch_fetch64(self.ctx.h, self.h, _p(vals), _stream(stream)))

    def finish(self, stream=None):
        st = Stats()
        self.ctx.check(self.ctx.L.ltp_batch_finish(self.ctx.h, self.h, ctypes.byref(st), _stream(stream)))
        return st

    def results(self):
        commit = np.zeros(max(self.n_txns, 1), np.uint8)
        vals = np.zeros(max(self.n_ops, 1), np.int32)
        st = Stats()
        self.ctx.check(self.ctx.L.ltp_batch_results(self.ctx.h, self.h, _p(commit), _p(vals), ctypes.byref(st)))
        return commit[: self.n_txns], vals[: self.n_ops], st

    def results64(self):
        """(commit, int64 values, stats); the context must have an int64 column."""
        commit = np.zeros(max(self.n_txns, 1), np.uint8)
        vals = np.zeros(max(self.n_ops, 1), np.int64)
        self.fetch(commit=commit)
        self.fetch64(vals)
        st = self.finish()
        return commit[: self.n_txns], vals[: self.n_ops], st


class Pipe:
    """Pipelined submission (the C-ABI ltp_pipe): copy-in, execution and
    copy-out of consecutive batches overlap on three streams."""

    def __init__(self, ctx, depth, max_txns, max_ops, persistent=False):
        self.ctx = ctx
        h = ctypes.c_void_p()
        ctx.check(ctx.L.ltp_pipe_create2(ctx.h, depth, max_txns, max_ops, 1 if persistent else 0, ctypes.byref(h)))
        self.h = h
        self._keep = {}

    def submit(self, txn_first, keys, opw, commit_out=None, vals_out=None, ops_per_txn=0, payload=None):
        """Arrays must stay alive (and unchanged) until wait(ticket); uint32 keys
        go through ltp_pipe_submit32."""
        if txn_first is not None:
            n_txns = len(txn_first) - 1
        else:
            n_txns = len(keys) // ops_per_txn if ops_per_txn else 0
        t = ctypes.c_uint64()
        fn = self.ctx.L.ltp_pipe_submit32 if keys.dtype == np.uint32 else self.ctx.L.ltp_pipe_submit
        self.ctx.check(fn(
            self.h, n_txns, _p(txn_first), ops_per_txn, len(keys), _p(keys), _p(opw), _p(payload),
            0 if payload is None else len(payload), _p(commit_out), _p(vals_out), ctypes.byref(t)))
        self._keep[t.value] = (txn_first, keys, opw, commit_out, vals_out, payload)
        return t.value

    def wait(self, ticket):
        st = Stats()
        rc = self.ctx.L.ltp_pipe_wait(self.h, ticket, ctypes.byref(st))
        self._keep.pop(ticket, None)
        self.ctx.check(rc)
        return st

    def poll(self, ticket):
        return self.ctx.L.ltp_pipe_poll(self.h, ticket) == 0

    def close(self):
        if getattr(self, "h", None):
            self.ctx.L.ltp_pipe_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """The continuous-batching request loop (the C-ABI ltp_server)."""

    def __init__(self, ctx, deadline_us=250, depth=3, budget_bytes=4 << 30, max_txns=1 << 20, max_ops=1 << 24,
                 max_attempts=64, eager=True, keep_results=True, persistent=False):
        self.ctx = ctx
        flags = (SERVE_EAGER if eager else 0) | (SERVE_KEEP_RESULTS if keep_results else 0) | \
            (SERVE_PERSISTENT if persistent else 0)
        cfg = ServeConfig(deadline_us, depth, budget_bytes, max_txns, max_ops, max_attempts, flags)
        h = ctypes.c_void_p()
        ctx.check(ctx.L.ltp_serve_open(ctx.h, ctypes.byref(cfg), ctypes.byref(h)))
        self.h = h
        self._pool = None

    def submit(self, stream, keys, opw, tag=0, arrival_ns=0, payload=None):
        """payload: the transaction's insert rows; its insert ops' keys are
        offsets into it."""
        keys = np.ascontiguousarray(keys, np.uint64)
        opw = np.ascontiguousarray(opw, np.uint32)
        if payload is None:
            self.ctx.check(self.ctx.L.ltp_serve_submit(self.h, stream, len(keys), _p(keys), _p(opw), tag, arrival_ns))
        else:
            pl = np.ascontiguousarray(payload, np.int32)
            self.ctx.check(self.ctx.L.ltp_serve_submit_rows(self.h, stream, len(keys), _p(keys), _p(opw), len(pl),
                                                            _p(pl), tag, arrival_ns))

    def loadgen(self, rate, seconds, n_streams, txn_first, keys, opw, seed=1, threads=8, pay_first=None,
                payload=None):
        """Open-loop Poisson load from a pool; with pay_first/payload the pool
        holds inserts (insert keys are offsets into the whole payload)."""
        self._pool = (np.ascontiguousarray(txn_first, np.uint32), np.ascontiguousarray(keys, np.uint64),
                      np.ascontiguousarray(opw, np.uint32),
                      None if pay_first is None else np.ascontiguousarray(pay_first, np.uint64),
                      None if payload is None else np.ascontiguousarray(payload, np.int32))
        tf, k, w, pf, pl = self._pool
        self.ctx.check(self.ctx.L.ltp_serve_loadgen_rows(self.h, rate, seconds, n_streams, seed, _p(tf), len(tf) - 1,
                                                         _p(k), _p(w), _p(pf), _p(pl), threads))

    def poll(self, max_results=4096):
        buf = (ServeResult * max_results)()
        n = ctypes.c_uint32()
        self.ctx.check(self.ctx.L.ltp_serve_poll(self.h, buf, max_results, ctypes.byref(n)))
        return buf[:n.value]

    def stats(self):
        st = ServeStats()
        self.ctx.check(self.ctx.L.ltp_serve_stats_now(self.h, ctypes.byref(st)))
        return st.as_dict()

    def close(self):
        st = ServeStats()
        if getattr(self, "h", None):
            rc = self.ctx.L.ltp_serve_close(self.h, ctypes.byref(st))
            self.h = None
            self.ctx.check(rc)
        return st.as_dict()


class Ingest:
    """Serving from a device-resident request log (the C-ABI ltp_ingest):
    the pool goes to the device once; run() serves requests 0..n-1 (request i
    = pool transaction i mod pool size) at their arrival times.  keys64 keeps
    64-bit keys on the device even when every key fits 32 bits; jit queues
    the next batch only once the batch ahead is past its sort."""

    def __init__(self, ctx, txn_first, keys, opw, pay_first=None, payload=None, deadline_us=250, depth=3,
                 budget_bytes=4 << 30, max_txns=1 << 20, max_ops=1 << 24, max_attempts=64, eager=True,
                 keep_results=False, keys64=False, jit=False):
        self.ctx = ctx
        flags = (SERVE_EAGER if eager else 0) | (SERVE_KEEP_RESULTS if keep_results else 0) | \
            (SERVE_KEYS64 if keys64 else 0) | (SERVE_JIT if jit else 0)
        cfg = ServeConfig(deadline_us, depth, budget_bytes, max_txns, max_ops, max_attempts, flags)
        self._pool = (np.ascontiguousarray(txn_first, np.uint32), np.ascontiguousarray(keys, np.uint64),
                      np.ascontiguousarray(opw, np.uint32),
                      None if pay_first is None else np.ascontiguousarray(pay_first, np.uint64),
                      None if payload is None else np.ascontiguousarray(payload, np.int32))
        tf, k, w, pf, pl = self._pool
        self.n_pool = len(tf) - 1
        h = ctypes.c_void_p()
        ctx.check(ctx.L.ltp_ingest_open(ctx.h, ctypes.byref(cfg), self.n_pool, _p(tf), _p(k), _p(w), _p(pf), _p(pl),
                                        ctypes.byref(h)))
        self.h = h
        self.n = 0

    def run(self, arrival_ns):
        """arrival_ns[i]: request i's arrival in ns after the run's start."""
        arr = np.ascontiguousarray(arrival_ns, np.uint64)
        st = ServeStats()
        self.ctx.check(self.ctx.L.ltp_ingest_run(self.h, len(arr), _p(arr), ctypes.byref(st)))
        self.n = len(arr)
        return st.as_dict()

    def results(self, values=False):
        """(committed, batch_seq, pos, attempts[, values in log op order])."""
        n = self.n
        c = np.zeros(n, np.uint8)
        seq = np.zeros(n, np.uint64)
        pos = np.zeros(n, np.uint32)
        att = np.zeros(n, np.uint32)
        vals = None
        if values:
            tf = self._pool[0]
            vals = np.zeros(int(tf[n]) if n else 0, np.int64)
        self.ctx.check(self.ctx.L.ltp_ingest_results(self.h, _p(c), _p(seq), _p(pos), _p(att), _p(vals)))
        return (c, seq, pos, att, vals) if values else (c, seq, pos, att)

    def close(self):
        if getattr(self, "h", None):
            rc = self.ctx.L.ltp_ingest_close(self.h)
            self.h = None
            self.ctx.check(rc)


def poisson_arrivals(n, rate, seed, threads=0):
    """uint64[n] arrival times (ns after the start) of an open-loop Poisson
    process at `rate` requests/s (the merged arrivals of independent Poisson
    client streams), for Ingest.run."""
    L = load()
    out = np.empty(max(int(n), 1), np.uint64)
    rc = L.ltp_poisson_arrivals(int(n), float(rate), int(seed), _p(out), int(threads))
    if rc:
        raise LtpError(rc, "ltp_poisson_arrivals")
    return out[:int(n)]


PROBE_LOAD, PROBE_ATOMIC, PROBE_REDUCE = 0, 1, 2
PROBE_LIB_PATH = os.path.join(PKG, "libltpmg_probe.so")
_probe = None


def probe_random_access(device, nbytes, mode):
    """Random 4-byte accesses per second over an array of nbytes (mode:
    PROBE_LOAD, PROBE_ATOMIC with result, PROBE_REDUCE).  A benchmark tool in
    its own library (libltpmg_probe.so), not part of the product's C ABI."""
    global _probe
    if _probe is None:
        if not os.path.exists(PROBE_LIB_PATH):
            raise LtpError(LTP_E_STATE, f"{PROBE_LIB_PATH} is not built")
        _probe = ctypes.CDLL(PROBE_LIB_PATH)
        _probe.ltp_probe_random_access.restype = ctypes.c_int
        _probe.ltp_probe_random_access.argtypes = [ctypes.c_int32, ctypes.c_uint64, ctypes.c_int32,
                                                   ctypes.POINTER(ctypes.c_double)]
    out = ctypes.c_double()
    rc = _probe.ltp_probe_random_access(device, nbytes, mode, ctypes.byref(out))
    if rc:
        raise LtpError(rc, "ltp_probe_random_access")
    return out.value
