"""The reference's eight GPU entry points (cuda/src/gpuscheduler.cu:3-47),
served by libltpmg_gb300.so through include/ltpmg_compat.h.

CPU: the library exports the eight functions under the reference's own C++
symbol names and a driver written against the compat header links.
GPU: the driver runs the reference's Scheduler::start sequence for YCSB_A..E
(the same batch re-sent every epoch) and the final int table equals the
oracle's serial replay of the expanded batch, bit for bit.
"""
import os
import re
import subprocess

import numpy as np
import pytest

import ltpmg_gb300 as G
import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
DRIVER_SRC = os.path.join(HERE, "compat", "compat_driver.cpp")
DRIVER = os.path.join(HERE, "compat", "compat_driver")

# the reference's declarations (include/database.h:66-70, include/query.h:63-70,
# include/scheduler.h:33-37) mangle to these names
REFERENCE_SYMBOLS = [
    "_Z24transfer_database_to_GPUSt10shared_ptrI5ParamEP17Global_Table_InfoP12Global_TableP18Global_Table_Index",
    "_Z24transfer_database_to_CPUSt10shared_ptrI5ParamEP17Global_Table_InfoP12Global_TableP18Global_Table_Index",
    "_Z20initial_query_on_GPUSt10shared_ptrI5ParamES_ISt6vectorISt3anySaIS3_EEEP15Global_Txn_Info",
    "_Z21transfer_query_to_GPUSt10shared_ptrI5ParamES_ISt6vectorISt3anySaIS3_EEEP15Global_Txn_Info",
    "_Z21transfer_query_to_CPUSt10shared_ptrI5ParamES_ISt6vectorISt3anySaIS3_EEEP15Global_Txn_Info",
    "_Z23initial_launcher_on_GPUSt10shared_ptrI5ParamE",
    "_Z14execute_on_GPUSt10shared_ptrI5ParamE",
    "_Z20free_launcher_on_GPUSt10shared_ptrI5ParamE",
]


def build_driver():
    libdir = os.path.dirname(G.lib.LIB_PATH)
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), DRIVER_SRC, "-L", libdir,
                    "-lltpmg_gb300", f"-Wl,-rpath,{libdir}", "-o", DRIVER], check=True, capture_output=True)
    return DRIVER


def test_reference_symbols_exported(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", G.lib.LIB_PATH], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    missing = [s for s in REFERENCE_SYMBOLS if s not in exported]
    assert not missing, missing


def test_driver_links(lib):
    assert os.path.exists(build_driver())


def expand(variant, queries, rows):
    """The compat layer's expansion of YCSB queries (3 int columns)."""
    tf, keys, opw, payload = [0], [], [], []
    for q in queries:
        for i in range(10):
            kind = O.lib().ltpo_ref_ycsb_op_type(variant, i)
            r = int(q[1 + i])
            if kind == 1:
                keys.append(len(payload))
                opw.append(O.opword(2, 0, 0, 0))
                payload += [r, r, r]
                continue
            span = 2 if kind == 4 else 1
            for rr in range(r, min(r + span, rows)):
                for c in range(3):
                    keys.append(rr)
                    opw.append(O.opword(1, c, 0, 1) if kind == 2 else O.opword(0, c, 0, 0))
        tf.append(len(keys))
    return (np.array(tf, np.uint32), np.array(keys, np.uint64), np.array(opw, np.uint32),
            np.array(payload or [0], np.int32))


@pytest.mark.gpu
@pytest.mark.parametrize("variant", [0, 1, 2, 3, 4])
def test_scheduler_sequence_matches_oracle(lib, tmp_path, variant):
    rows, txns, epochs, seed = 4096, 3000, 3, 11 + variant
    build_driver()
    out = tmp_path / "out.bin"
    r = subprocess.run([DRIVER, str(out), str(variant), str(rows), str(txns), str(epochs), str(seed)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    raw = np.fromfile(out, np.int32)
    st, nrows, ntx, nep = raw[:4]
    assert st == 0 and nrows == rows
    queries = raw[4:4 + ntx * 11].view(np.uint32).reshape(ntx, 11)
    final = raw[4 + ntx * 11:].reshape(rows, 3)
    init = np.array([[lib.ltp_table_value(seed, rr, c, 3) for rr in range(rows)] for c in range(3)], np.int32)
    cap = rows + (txns * epochs if variant == 4 else 0)
    data = np.zeros((3, cap), np.int32)
    data[:, :rows] = init
    tables = [(data, rows)]
    tf, keys, opw, payload = expand(variant, queries, rows)
    for _ in range(epochs):
        tables, commit, vals = O.replay_tables(0, tables, tf, keys, opw, payload if variant == 4 else None)
    exp = tables[0][0][:, :rows].T
    assert np.array_equal(final, exp)
    if variant == 4:
        assert tables[0][1] == rows + txns * epochs


REF_HOST = os.path.join(ROOT, "oracle", "_ref", "ltpmg_host")


def test_reference_host_program_links_against_the_library():
    """The reference's whole host program (its src/*.cpp, main included,
    compiled with the gflags/glog stand-ins) links against
    libltpmg_gb300.so in place of its CUDA library: every GPU entry point it
    calls resolves here.  Built by oracle/build_ref.sh where the reference
    tree is present."""
    if not os.path.exists(REF_HOST):
        pytest.skip("reference host program not built (reference tree absent)")
    und = subprocess.run(["nm", "-D", "--undefined-only", REF_HOST], capture_output=True, text=True).stdout
    for sym in REFERENCE_SYMBOLS:
        assert sym in und, sym
    deps = subprocess.run(["ldd", REF_HOST], capture_output=True, text=True).stdout
    assert "libltpmg_gb300.so" in deps and "not found" not in deps


@pytest.mark.gpu
def test_reference_host_program_runs_its_epochs_on_the_library():
    """The reference's whole host program -- its own main, Database::generate,
    Query::generate_txn and Scheduler::start, compiled from its sources with
    the flag and log stand-ins -- runs four YCSB_A epochs of 2^14 Zipf 0.99
    transactions over 10^6 rows against libltpmg_gb300.so: every epoch is
    executed here and commits its whole batch (the library's exit report),
    and the reference's own timing lines report each measured epoch."""
    if not os.path.exists(REF_HOST):
        pytest.skip("reference host program not built (reference sources absent)")
    env = dict(os.environ, LTPMG_COMPAT_REPORT="1", LTPMG_SHIM_LOG="1")
    cwd = os.path.join(os.path.dirname(REF_HOST), "src", "src")  # it reads its schemas from ../data
    r = subprocess.run([REF_HOST, "--benchmark=YCSB_A", "--table_size=1", "--batch_size=16384", "--epoch_tp=4",
                        "--deviceIDs=0", "--data_distribution=zipf", "--zipf_config=0.99"],
                       cwd=cwd, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    rep = [line for line in r.stderr.splitlines() if line.startswith("ltp_compat:")]
    assert rep, r.stderr[-2000:]
    m = re.match(r"ltp_compat: batches=(\d+) committed=(\d+) status=(-?\d+)", rep[-1])
    assert m and m.group(3) == "0", rep[-1]
    assert int(m.group(1)) == 4 and int(m.group(2)) == 4 * 16384, rep[-1]
    # Scheduler::start logs the epochs strictly between 10% and 90% of the run
    times = [float(x) for x in re.findall(r"Execution time: ([0-9.eE+-]+) s\.", r.stderr)]
    assert len(times) == 3 and all(t > 0 for t in times), times


TPCC_INT_COLS = [1, 3, 5, 3, 5, 7, 8, 5, 2]  # int attributes of data/TPCC.json's nine tables


def expand_tpcc(flat, cidx, rows):
    """The compat layer's expansion of TPC-C queries (the row operations of
    parse<Neworder_Query> / parse<Payment_Query>, cuda/src/gpuquery.cu:2474-2734,
    on every int column; rows modulo the table's rows; inserts append the ids
    the query names)."""
    tf, keys, opw, payload = [0], [], [], []

    def row_op(kind, t, row, vals=()):
        cols = TPCC_INT_COLS[t]
        if kind == 1:
            keys.append(len(payload))
            opw.append(O.opword(2, 0, t, 0))
            payload.extend([int(v) for v in vals] + [0] * (cols - len(vals)))
            return
        r = row % rows[t]
        for c in range(cols):
            keys.append(r)
            opw.append(O.opword(1, c, t, 1) if kind == 2 else O.opword(0, c, t, 0))

    i = 0
    while i < len(flat):
        kind = int(flat[i])
        if kind == 0:
            q = [int(x) for x in flat[i + 1:i + 54]]
            i += 54
            tid, w, d, c, o_id, n_o_id, ol_cnt, _ = q[:8]
            info = [q[8 + 3 * k:11 + 3 * k] for k in range(15)]
            wd = w * 10 + d
            lines = min(ol_cnt, 15)
            local = all(info[k][1] == w for k in range(lines))
            row_op(0, 0, w)
            row_op(0, 1, wd)
            row_op(0, 2, wd * 3000 + c)
            row_op(1, 3, 0, (n_o_id, d, w))
            row_op(1, 5, 0, (o_id, d, w, c, 0, lines, 1 if local else 0))
            for k in range(lines):
                i_id, sw, qty = info[k]
                row_op(1, 6, 0, (o_id, d, w, k + 1, i_id, sw, 0, qty))
                row_op(2, 7, sw * 1000000 + i_id)
                row_op(2, 7, sw * 1000000 + i_id)
        else:
            q = [int(x) for x in flat[i + 1:i + 11]]
            i += 11
            tid, w, d, c, c_last, is_name, c_d, c_w, _, _ = q
            wd = w * 10 + d
            if is_name == 1:
                c = 0
                for k in range(3000):
                    at = wd * 3000 + k
                    if at < len(cidx) and int(cidx[at]) == c_last:
                        c = k
                        break
            cust = (c_w * 10 + c_d) * 3000 + c
            row_op(0, 0, w)
            row_op(0, 1, wd)
            row_op(0, 2, cust)
            row_op(2, 2, cust)
            row_op(2, 0, w)
            row_op(2, 1, wd)
            row_op(1, 4, 0, (c, c_d, c_w, d, w))
        tf.append(len(keys))
    return (np.array(tf, np.uint32), np.array(keys, np.uint64), np.array(opw, np.uint32),
            np.array(payload or [0], np.int32))


@pytest.mark.gpu
def test_tpcc_scheduler_sequence_matches_oracle(lib, tmp_path):
    """TPCC_PART through the reference's eight entry points: new-order and
    payment queries (the reference's own structs) re-sent every epoch; the
    final int tables equal the oracle's serial replay of the expanded batch."""
    W, txns, epochs, seed = 2, 2000, 2, 31
    build_driver()
    out = tmp_path / "tpcc.bin"
    r = subprocess.run([DRIVER, str(out), "5", str(W), str(txns), str(epochs), str(seed)], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr
    raw = np.fromfile(out, np.int32)
    st, w_, ntx, nep = raw[:4]
    assert st == 0 and w_ == W and ntx == txns
    nflat = int(raw[4])
    flat = raw[5:5 + nflat].view(np.uint32)
    d = W * 10
    rows = [W, d, d * 3000, d * 3000, d * 3000, d * 3000, d * 45000, W * 100000, 100000]
    cidx = raw[5 + nflat:5 + nflat + rows[2]].view(np.uint32)
    off = 5 + nflat + rows[2]
    finals = []
    for t in range(9):
        n = rows[t] * TPCC_INT_COLS[t]
        finals.append(raw[off:off + n].reshape(rows[t], TPCC_INT_COLS[t]))
        off += n
    tf, keys, opw, payload = expand_tpcc(flat, cidx, rows)
    assert len(tf) - 1 == txns
    tables = []
    for t in range(9):
        cols = TPCC_INT_COLS[t]
        cap = rows[t] + (txns * epochs * (15 if t == 6 else 1) if 3 <= t <= 6 else 0)
        data = np.zeros((cols, cap), np.int32)
        data[:, :rows[t]] = O.table_init(seed + t, rows[t], cols)  # ltp_table_value, column-major
        tables.append((data, rows[t]))
    for _ in range(epochs):
        tables, commit, vals = O.replay_tables(0, tables, tf, keys, opw, payload)
        assert commit.all()
    for t in range(9):
        assert np.array_equal(finals[t], tables[t][0][:, :rows[t]].T), t

